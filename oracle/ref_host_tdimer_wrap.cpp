// TEST INFRASTRUCTURE ONLY. extern "C" wrapper over the reference's TriangleDimerTiler static
// host functions (src/TriangleDimer/TriangleDimerTiler.cpp:697-982), compiled from the reference
// tree by oracle/Makefile.  The CUDA launch wrappers the class declares are never called here;
// oracle/Makefile generates abort() stubs for them from triangledimerkernel.cuh.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <cuda_runtime.h>
#include <curand_mtgp32.h>
#include "src/common/common.h"
#include "src/TriangleDimer/TriangleDimerTiler.h"
#include "src/TriangleDimer/triangledimerkernel.cuh"

#include "td_stubs.inc"

extern "C" int refh_td_icecream(int n, int m, int* out, long cap) {
  tiling t = TriangleDimerTiler::IceCreamCone(n, m);
  if ((long)t.size() > cap) return -1;
  std::memcpy(out, t.data(), t.size() * sizeof(int));
  return (int)std::lround(std::sqrt((double)t.size()));
}

extern "C" void refh_td_tri_flips(const int* t, int N, int* out) {
  tiling tt(t, t + (size_t)N * N);
  std::vector<int> v = TriangleDimerTiler::TilingToTriangleFlips(tt);
  std::memcpy(out, v.data(), v.size() * sizeof(int));
}

extern "C" void refh_td_bfly_flips(const int* t, int N, int* out) {
  tiling tt(t, t + (size_t)N * N);
  std::vector<int> v = TriangleDimerTiler::TilingToButterflyFlips(tt);
  std::memcpy(out, v.data(), v.size() * sizeof(int));
}

extern "C" void refh_td_vertices(const int* t, int N, int* out) {
  tiling tt(t, t + (size_t)N * N);
  std::vector<int> v = TriangleDimerTiler::TilingToVertices(tt);
  std::memcpy(out, v.data(), v.size() * sizeof(int));
}

extern "C" void refh_td_domain(const int* t, int N, int* out) {
  tiling tt(t, t + (size_t)N * N);
  domain d = TriangleDimerTiler::TilingToDomain(tt);
  std::memcpy(out, d.data(), d.size() * sizeof(int));
}

extern "C" void refh_td_dimer_indicator(const int* t, int N, int c, int* out) {
  tiling tt(t, t + (size_t)N * N);
  std::vector<int> v = TriangleDimerTiler::DimerIndicator(tt, c);
  std::memcpy(out, v.data(), v.size() * sizeof(int));
}

extern "C" int refh_td_test_butterfly(int type, int* out, long cap) {
  tiling t = TriangleDimerTiler::TestButterfly(type);
  if ((long)t.size() > cap) return -1;
  std::memcpy(out, t.data(), t.size() * sizeof(int));
  return (int)std::lround(std::sqrt((double)t.size()));
}
