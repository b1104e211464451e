// TEST INFRASTRUCTURE ONLY. Host driver for the reference's src/Lozenge/lozengekernel.cl (and,
// built a second time, qlozengekernel.cl),
// compiled from the reference tree by oracle/Makefile.  The kernels come verbatim from the
// reference file; this driver states the OpenCL host loop of LozengeTiler::Walk
// (src/Lozenge/LozengeTiler.cpp:27-159, the #ifndef __NVCC__ branches) as NDRange loops.
#include <cstdint>
#include <random>
#include <vector>

#include "ref_cl_shim.h"

// REF_CELL: the element type the kernel file uses (char in lozengekernel.cl, int in
// qlozengekernel.cl); REF_LZ_WALK: the exported name.
#ifndef REF_CELL
#define REF_CELL char
#endif
#ifndef REF_LZ_WALK
#define REF_LZ_WALK ref_lz_walk
#endif

namespace refloz {
#include REF_CL
}

extern "C" int REF_LZ_WALK(int* t, int N, long steps, long seed, const uint32_t* params, long nparams) {
  const int M = N / 3;
  std::vector<REF_CELL> R((size_t)N * M, 0), B((size_t)N * M, 0), G((size_t)N * M, 0);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      int c = ((j - i) % 3 + 3) % 3;
      (c == 0 ? R : c == 1 ? B : G)[(size_t)i * M + j / 3] = (REF_CELL)t[(size_t)i * N + j];
    }
  std::vector<refloz::tinymt32wp_t> st((size_t)N * M);
  for (size_t k = 0; k < st.size(); ++k) {
    if (params && (long)k < nparams) {
      st[k].mat1 = params[3 * k]; st[k].mat2 = params[3 * k + 1]; st[k].tmat = params[3 * k + 2];
    } else {
      st[k].mat1 = TINYMT32J_MAT1; st[k].mat2 = TINYMT32J_MAT2; st[k].tmat = TINYMT32J_TMAT;
    }
  }
  refcl::gsize[0] = (size_t)N * M; refcl::gsize[1] = 1; refcl::gsize[2] = 1; refcl::gid[1] = 0; refcl::gid[2] = 0;
  for (size_t k = 0; k < st.size(); ++k) {
    refcl::gid[0] = k;
    refloz::InitTinyMT(st.data(), (uint)seed);
  }
  std::default_random_engine generator;
  std::uniform_int_distribution<int> distribution(0, 2);
  generator.seed(seed);
  REF_CELL* X[3] = {R.data(), B.data(), G.data()};
  for (long s = 0; s < steps; ++s) {
    int r = distribution(generator);
    refcl::gsize[0] = N; refcl::gsize[1] = M; refcl::gsize[2] = 1; refcl::gid[2] = 0;
    for (size_t x = 0; x < (size_t)N; ++x)
      for (size_t y = 0; y < (size_t)M; ++y) {
        refcl::gid[0] = x; refcl::gid[1] = y;
        refloz::RotateTiles(st.data(), X[r], N);
      }
    for (size_t x = 0; x < (size_t)N; ++x)
      for (size_t y = 0; y < (size_t)M; ++y) {
        refcl::gid[0] = x; refcl::gid[1] = y;
        refloz::UpdateTiles(X[r], X[(r + 1) % 3], X[(r + 2) % 3], N, r);
      }
  }
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      int c = ((j - i) % 3 + 3) % 3;
      t[(size_t)i * N + j] = (c == 0 ? R : c == 1 ? B : G)[(size_t)i * M + j / 3];
    }
  return 0;
}
