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

// cuRAND MTGP32 generators in the reference's CUDA geometry (domino_mtgp.cu): 8 x 8 thread
// blocks over a rows x cols grid of sites (row from the x index, column from the y index),
// block (bx, by) drawing from generator bx * gy + by.
struct MtgpGrid {
  int gx = 0, gy = 0;
  int count() const { return gx * gy; }
};
constexpr int kMtgpBlock = 8;  // BLOCK_DIM of the reference (dominokernel.cuh:4, lozengekernel.cuh:4)
inline MtgpGrid mtgp_grid(int rows, int cols) {
  return MtgpGrid{(rows + kMtgpBlock - 1) / kMtgpBlock, (cols + kMtgpBlock - 1) / kMtgpBlock};
}
size_t mtgp_state_bytes(int count);
// Seeds generator k with seed + k through curandMakeMTGP32KernelState (blocking copies, so
// the stream is drained first).
rt_status mtgp_seed(void* states, int count, int64_t seed, cudaStream_t stream);
// The draws of `launches` launches on a fresh grid seeded seed + k: out[h][x][y] for
// x < rows, y < cols (host memory).
rt_status mtgp_draws_grid(int rows, int cols, int64_t seed, int64_t launches, float* out);

// Per-generator TinyMT parameters of the reference's LoadTinyMT (file_reader.cpp:22-38):
// o.tinymt_params holds o.tinymt_params_count triples (mat1, mat2, tmat), triple k for
// generator k.  Allocates (cudaMalloc) and fills a device table of `count` uint4
// {mat1, mat2, tmat, 0}; generators beyond the triples keep the TinyMT32 jump set, as the
// reference's default parameters do.  *out stays NULL when o carries no table.
rt_status tmt_param_table(const rt_walk_opts& o, int64_t count, uint4** out, cudaStream_t s);

// The autotuner's table (tune.cpp): the engine, bands and threads per band measured fastest
// for a model, tiling side, chain count and random mode; false when the table has none.
bool tune_lookup(int model, int n_side, int chains, int rng, int* engine, int* bands, int* threads);

// Vertex classes of DomainToVertices: 0 outside, 1 interior, 2 boundary.
void domino_vertex_classes(const int32_t* domain, int m_side, int32_t* out);
// Interior vertices (flip candidates) of the domain a tiling covers.
int64_t domino_count_interior_from_tiling(const int32_t* tiling, int n_side);

}  // namespace rt
