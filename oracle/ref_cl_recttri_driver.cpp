// TEST INFRASTRUCTURE ONLY. Host driver for the reference's
// src/RectTriangle/recttrianglekernel.cl (kernels verbatim from the reference file), stating
// the OpenCL host loop of RectTriangleTiler::Walk (RectTriangleTiler.cpp:33-171) as NDRange
// loops.
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include "ref_cl_shim.h"

namespace refrt {
#include REF_CL
}

extern "C" int ref_rt_walk(int* t, int N, long steps, long seed, const uint32_t* params, long nparams) {
  const int M = N / 3;
  std::vector<int> X[3];
  for (auto& x : X) x.assign((size_t)N * M, 0);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) X[((i - j) % 3 + 3) % 3][(size_t)i * M + j / 3] = t[(size_t)i * N + j];
  std::vector<refrt::tinymt32wp_t> st((size_t)N * M);
  // The parameter buffer of LoadTinyMT (file_reader.cpp: one (mat1, mat2, tmat) per
  // generator, the rest of the buffer the jump set here).
  for (size_t k = 0; k < st.size(); ++k) {
    auto& s = st[k];
    if (params && (long)k < nparams) {
      s.mat1 = params[3 * k]; s.mat2 = params[3 * k + 1]; s.tmat = params[3 * k + 2];
    } else {
      s.mat1 = TINYMT32J_MAT1; s.mat2 = TINYMT32J_MAT2; s.tmat = TINYMT32J_TMAT;
    }
  }
  refcl::gsize[0] = (size_t)N * M; refcl::gsize[1] = 1; refcl::gsize[2] = 1; refcl::gid[1] = 0; refcl::gid[2] = 0;
  for (size_t k = 0; k < st.size(); ++k) {
    refcl::gid[0] = k;
    refrt::InitTinyMT(st.data(), (uint)seed);
  }
  std::default_random_engine generator;
  std::uniform_int_distribution<int> distribution(0, 2);
  generator.seed(seed);
  for (long s = 0; s < steps; ++s) {
    const int r = distribution(generator);
    refcl::gsize[0] = N; refcl::gsize[1] = M; refcl::gsize[2] = 1; refcl::gid[2] = 0;
    for (size_t x = 0; x < (size_t)N; ++x)
      for (size_t y = 0; y < (size_t)M; ++y) {
        refcl::gid[0] = x; refcl::gid[1] = y;
        refrt::flipTiles(st.data(), X[r].data(), N);
      }
    for (size_t x = 0; x < (size_t)N; ++x)
      for (size_t y = 0; y < (size_t)M; ++y) {
        refcl::gid[0] = x; refcl::gid[1] = y;
        refrt::updateTiles1(X[r].data(), X[(r + 1) % 3].data(), N, r);
      }
    for (size_t x = 0; x < (size_t)N; ++x)
      for (size_t y = 0; y < (size_t)M; ++y) {
        refcl::gid[0] = x; refcl::gid[1] = y;
        refrt::updateTiles2(X[r].data(), X[(r + 2) % 3].data(), N, r);
      }
  }
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) t[(size_t)i * N + j] = X[((i - j) % 3 + 3) % 3][(size_t)i * M + j / 3];
  return 0;
}
