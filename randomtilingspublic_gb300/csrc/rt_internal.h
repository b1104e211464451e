// Internal helpers shared by the translation units of librt_tilings.so.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/rt_tilings.h"

namespace rt {

// Per-thread message of the last failure, returned by rt_last_error().
void set_error(const std::string& msg);
void clear_error();
inline rt_status fail(rt_status code, const std::string& msg) {
  set_error(msg);
  return code;
}

// Stream-ordered device allocations from the library's per-device pool (device_pool.cpp):
// use the block only on stream s (or after synchronising with it) and free it on a stream.
rt_status dev_alloc(void** p, size_t bytes, cudaStream_t s);
void dev_free(void* p, cudaStream_t s);
template <class T>
inline rt_status dev_alloc(T** p, size_t bytes, cudaStream_t s) {
  void* v = nullptr;
  rt_status st = dev_alloc(&v, bytes, s);
  *p = static_cast<T*>(v);
  return st;
}

// Vertex classes of DomainToVertices: 0 outside, 1 interior, 2 boundary.
void domino_vertex_classes(const int32_t* domain, int m_side, int32_t* out);
// Interior vertices (flip candidates) of the domain a tiling covers.
int64_t domino_count_interior_from_tiling(const int32_t* tiling, int n_side);

}  // namespace rt
