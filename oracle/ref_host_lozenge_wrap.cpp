// TEST INFRASTRUCTURE ONLY. extern "C" wrapper over the reference's own LozengeTiler static
// host functions (src/Lozenge/LozengeTiler.cpp:173-556), compiled from the reference tree by
// oracle/Makefile.
#include <cstdlib>
#include <cstring>
#include <cuda_runtime.h>
#include <curand_mtgp32.h>
#include "src/common/common.h"
#include "src/Lozenge/LozengeTiler.h"

// Never called: only the static host utilities are used through this library.
void RotateTiles(dim3, dim3, curandStateMtgp32*, char*, const int) { std::abort(); }
void UpdateTiles(dim3, dim3, char*, char*, char*, const int, const int) { std::abort(); }

static void copy_out(const std::vector<int>& v, int* out) { std::memcpy(out, v.data(), v.size() * sizeof(int)); }
extern "C" int refh_lz_almost_hex_domain(int n, int m, int* out, long cap) {
  domain d = LozengeTiler::AlmostHexDomain(n, m);
  if ((long)d.size() > cap) return -1;
  copy_out(d, out);
  return (int)std::lround(std::sqrt((double)d.size() / 2));
}
extern "C" void refh_lz_max_tiling(const int* d, int M, int* out) {
  copy_out(LozengeTiler::MaxTiling(domain(d, d + (size_t)2 * M * M)), out);
}
extern "C" void refh_lz_min_tiling(const int* d, int M, int* out) {
  copy_out(LozengeTiler::MinTiling(domain(d, d + (size_t)2 * M * M)), out);
}
extern "C" void refh_lz_domain_to_vertices(const int* d, int M, int* out) {
  copy_out(LozengeTiler::DomainToVertices(domain(d, d + (size_t)2 * M * M)), out);
}
extern "C" void refh_lz_tiling_to_heightfunc(const int* t, const int* d, int N, int* out) {
  copy_out(LozengeTiler::TilingToHeightfunc(tiling(t, t + (size_t)N * N), domain(d, d + (size_t)2 * (N - 1) * (N - 1))), out);
}
extern "C" void refh_lz_heightfunc_to_tiling(const int* h, const int* d, int N, int* out) {
  copy_out(LozengeTiler::HeightfuncToTiling(heightfunc(h, h + (size_t)N * N), domain(d, d + (size_t)2 * (N - 1) * (N - 1))), out);
}
