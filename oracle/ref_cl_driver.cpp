// TEST INFRASTRUCTURE ONLY. Host driver for one of the reference's domino .cl kernel files,
// compiled from the reference tree by oracle/Makefile (REF_CL names the file, NS the prefix
// of the exported symbols).  The kernels come verbatim from the reference file; this driver
// states its OpenCL host loop (src/Domino/DominoTiler.cpp:18-122 and :125-231, the
// #ifndef __NVCC__ branches) as sequential NDRange loops.
#include <cstdint>
#include <random>
#include <vector>

#include "ref_cl_shim.h"

namespace NS {
#include REF_CL
}
#undef a
#undef b

#define CAT2(x, y) x##y
#define CAT(x, y) CAT2(x, y)
#define EXPORT(name) CAT(NS, name)

namespace {

struct RefState {
  int N;
  std::vector<char> B, W;
  std::vector<NS::tinymt32wp_t> st;
};

void split(const int* t, int N, RefState& s) {
  s.N = N;
  s.B.assign((size_t)(N / 2) * N, 0);
  s.W.assign((size_t)(N / 2) * N, 0);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      if ((i + j) % 2 == 0) s.B[(size_t)i * (N / 2) + (j / 2)] = (char)t[(size_t)i * N + j];
      else s.W[(size_t)i * (N / 2) + (j / 2)] = (char)t[(size_t)i * N + j];
    }
}

void merge(const RefState& s, int* t) {
  const int N = s.N;
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j)
      t[(size_t)i * N + j] = ((i + j) % 2 == 0) ? s.B[(size_t)i * (N / 2) + (j / 2)] : s.W[(size_t)i * (N / 2) + (j / 2)];
}

void load_params(RefState& s, const uint32_t* params, long nparams) {
  const size_t total = (size_t)s.N * s.N / 2;
  s.st.assign(total, NS::tinymt32wp_t{});
  for (size_t k = 0; k < total; ++k) {
    if (params && (long)k < nparams) {
      s.st[k].mat1 = params[3 * k]; s.st[k].mat2 = params[3 * k + 1]; s.st[k].tmat = params[3 * k + 2];
    } else {
      s.st[k].mat1 = TINYMT32J_MAT1; s.st[k].mat2 = TINYMT32J_MAT2; s.st[k].tmat = TINYMT32J_TMAT;
    }
  }
}

void init_tinymt(RefState& s, uint seed) {
  const size_t total = (size_t)s.N * s.N / 2;
  refcl::gsize[0] = total; refcl::gsize[1] = 1; refcl::gsize[2] = 1;
  refcl::gid[1] = 0; refcl::gid[2] = 0;
  for (size_t k = 0; k < total; ++k) {
    refcl::gid[0] = k;
    NS::InitTinyMT(s.st.data(), seed);
  }
}

void step(RefState& s, int r) {
  const int N = s.N;
  refcl::gsize[0] = N - 2; refcl::gsize[1] = N / 2 - 2; refcl::gsize[2] = 1; refcl::gid[2] = 0;
  char* act = r == 1 ? s.B.data() : s.W.data();
  char* pas = r == 1 ? s.W.data() : s.B.data();
  for (size_t x = 0; x < (size_t)(N - 2); ++x)
    for (size_t y = 0; y < (size_t)(N / 2 - 2); ++y) {
      refcl::gid[0] = x; refcl::gid[1] = y;
      NS::RotateTiles(s.st.data(), act, N, r);
    }
  for (size_t x = 0; x < (size_t)(N - 2); ++x)
    for (size_t y = 0; y < (size_t)(N / 2 - 2); ++y) {
      refcl::gid[0] = x; refcl::gid[1] = y;
      NS::UpdateTiles(pas, act, N, r);
    }
}

}  // namespace

extern "C" int EXPORT(_walk)(int* t, int N, long steps, long seed, const uint32_t* params, long nparams) {
  RefState s;
  split(t, N, s);
  load_params(s, params, nparams);
  std::mt19937 mt_rand(seed);
  init_tinymt(s, (uint)mt_rand());
  for (long i = 0; i < steps; ++i) step(s, (int)(mt_rand() % 2));
  merge(s, t);
  return 0;
}

extern "C" int EXPORT(_walk_epochs)(int* t, int N, const long* steps, const long* seeds, int nepochs,
                                     const uint32_t* params, long nparams) {
  RefState s;
  split(t, N, s);
  load_params(s, params, nparams);
  for (int k = 0; k < nepochs; ++k) {
    std::mt19937 mt_rand(seeds[k]);
    init_tinymt(s, (uint)seeds[k]);
    for (long i = 0; i < steps[k]; ++i) step(s, (int)(mt_rand() % 2));
  }
  merge(s, t);
  return 0;
}
