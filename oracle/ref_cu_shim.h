// TEST INFRASTRUCTURE ONLY.  Lets the rotate kernels of the reference's CUDA build
// (src/Domino/dominokernel*.cu, src/Lozenge/lozengekernel.cu,
// src/RectTriangle/recttrianglekernel.cu, src/TriangleDimer/triangledimerkernel.cu) compile
// as host C++, so that oracle/_ref can run
// them as a sequential loop over an emulated launch grid.  The kernel file is read through
// a filter that drops its #include lines and its launch statements (the <<< >>> lines of
// the host wrappers); this header stands in for what they provided: the CUDA qualifiers,
// dim3, the built-in index variables, a no-op getLastCudaError, and curand_uniform on a
// stand-in MTGP32 state that returns the draw the emulation assigns to the calling thread.
// The filter also wraps the file's code in a namespace of its own, one per kernel file.
#pragma once
#include <cstddef>
#include <cstdint>

#define __global__
#define __device__
#define __constant__

struct dim3 {
  unsigned x, y, z;
  dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
struct uint3 {
  unsigned x, y, z;
};
struct curandStateMtgp32 {
  int unused;
};

namespace refcu {
inline thread_local uint3 block_idx, thread_idx;
inline thread_local dim3 block_dim, grid_dim;
// The draws of one emulated launch, rows x cols, row-major by the thread's global x and y
// index; threads outside that grid receive `outside`.
inline thread_local const float* draws = nullptr;
inline thread_local int rows = 0, cols = 0;
inline thread_local float outside = 0.5f;
}  // namespace refcu

#define blockIdx refcu::block_idx
#define threadIdx refcu::thread_idx
#define blockDim refcu::block_dim
#define gridDim refcu::grid_dim

inline float curand_uniform(curandStateMtgp32*) {
  const unsigned x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if ((int)x < refcu::rows && (int)y < refcu::cols) return refcu::draws[(size_t)x * refcu::cols + y];
  return refcu::outside;
}
inline void getLastCudaError(const char*) {}
