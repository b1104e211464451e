// TEST INFRASTRUCTURE ONLY. extern "C" wrapper over the reference's own DominoTiler static
// host functions (src/Domino/DominoTiler.cpp:249-631), compiled from the reference tree by
// oracle/Makefile, so that tests can pin the oracle's restatement against them.
#include <cstring>
#include "src/common/common.h"
#include "src/Domino/DominoTiler.h"
#include <cstdlib>
#include <cuda_runtime.h>
#include <curand_mtgp32.h>

// Never called: only the static host utilities are used through this library.
void RotateTiles(dim3, dim3, curandStateMtgp32*, char*, const int, const int) { std::abort(); }
void UpdateTiles(dim3, dim3, char*, char*, const int, const int) { std::abort(); }

extern "C" int refh_dm_aztec_rectangle(int n, const int* remove, int k, int* out, long cap) {
  std::vector<int> rm(remove, remove + k);
  domain d = DominoTiler::AztecRectangle(n, rm);
  if ((long)d.size() > cap) return -1;
  std::memcpy(out, d.data(), d.size() * sizeof(int));
  return (int)std::lround(std::sqrt((double)d.size()));
}
extern "C" int refh_dm_rectangle(int m, int n, int* out, long cap) {
  domain d = DominoTiler::Rectangle(m, n);
  if ((long)d.size() > cap) return -1;
  std::memcpy(out, d.data(), d.size() * sizeof(int));
  return (int)std::lround(std::sqrt((double)d.size()));
}
static void copy_out(const std::vector<int>& v, int* out) { std::memcpy(out, v.data(), v.size() * sizeof(int)); }
extern "C" void refh_dm_max_tiling(const int* d, int M, int* out) {
  copy_out(DominoTiler::MaxTiling(domain(d, d + (size_t)M * M)), out);
}
extern "C" void refh_dm_min_tiling(const int* d, int M, int* out) {
  copy_out(DominoTiler::MinTiling(domain(d, d + (size_t)M * M)), out);
}
extern "C" void refh_dm_domain_to_vertices(const int* d, int M, int* out) {
  copy_out(DominoTiler::DomainToVertices(domain(d, d + (size_t)M * M)), out);
}
extern "C" void refh_dm_tiling_to_heightfunc(const int* t, const int* d, int N, int* out) {
  copy_out(DominoTiler::TilingToHeightfunc(tiling(t, t + (size_t)N * N), domain(d, d + (size_t)(N - 1) * (N - 1))), out);
}
extern "C" void refh_dm_heightfunc_to_tiling(const int* h, const int* d, int N, int* out) {
  copy_out(DominoTiler::HeightfuncToTiling(heightfunc(h, h + (size_t)N * N), domain(d, d + (size_t)(N - 1) * (N - 1))), out);
}
extern "C" void refh_dm_tiling_to_domain(const int* t, int N, int* out) {
  copy_out(DominoTiler::TilingToDomain(tiling(t, t + (size_t)N * N)), out);
}
