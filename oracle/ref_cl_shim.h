// TEST INFRASTRUCTURE ONLY. Lets the reference's OpenCL C kernel files (src/Domino/*.cl,
// src/TinyMT/*.clh) compile as C++ on the host so that oracle/_ref can run them as a
// single-threaded NDRange loop.  Defines the handful of OpenCL built-ins they use.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cstring>

typedef unsigned int uint;
#define __kernel
#define __global
#define __constant static const
#define KERNEL_PROGRAM 1

namespace refcl {
inline thread_local size_t gid[3] = {0, 0, 0};
inline thread_local size_t gsize[3] = {1, 1, 1};
}  // namespace refcl

inline size_t get_global_id(int d) { return refcl::gid[d]; }
inline size_t get_global_size(int d) { return refcl::gsize[d]; }
inline size_t get_global_offset(int) { return 0; }
inline float as_float(uint x) {
  float f;
  std::memcpy(&f, &x, sizeof f);
  return f;
}
template <class T>
inline T select(T x, T y, bool c) {
  return c ? y : x;
}
