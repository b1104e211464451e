// TEST INFRASTRUCTURE ONLY. Host driver for the reference's
// src/TriangleDimer/triangledimerkernel.cl (kernels verbatim from the reference file), stating
// the OpenCL host loop of TriangleDimerTiler::Walk (TriangleDimerTiler.cpp:101-695, the
// #ifndef __NVCC__ branches) as NDRange loops over M x M work items.  The start states of the
// triangle and butterfly arrays come from the reference's own TilingToTriangleFlips /
// TilingToButterflyFlips (ref_host_tdimer_wrap.cpp).
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include "ref_cl_shim.h"

namespace reftd {
#include REF_CL
}

extern "C" void refh_td_tri_flips(const int* t, int N, int* out);
extern "C" void refh_td_bfly_flips(const int* t, int N, int* out);

namespace {

int g_M = 0;

template <class F>
void ndrange(F f) {
  refcl::gsize[0] = g_M; refcl::gsize[1] = g_M; refcl::gsize[2] = 1; refcl::gid[2] = 0;
  for (size_t x = 0; x < (size_t)g_M; ++x)
    for (size_t y = 0; y < (size_t)g_M; ++y) {
      refcl::gid[0] = x; refcl::gid[1] = y;
      f();
    }
}

}  // namespace

extern "C" int ref_td_walk(int* t, int N, long steps, long seed, const uint32_t* params, long nparams) {
  const int M = N / 2;
  g_M = M;
  std::vector<int> tTri((size_t)(N / 2) * N), tB((size_t)N * N);
  refh_td_tri_flips(t, N, tTri.data());
  refh_td_bfly_flips(t, N, tB.data());
  std::vector<int> eR((size_t)M * M), eL((size_t)M * M), eH((size_t)M * M), tU((size_t)M * M), tD((size_t)M * M),
      bR((size_t)M * M), bL((size_t)M * M), bH((size_t)M * M);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      const size_t k = (size_t)(i / 2) * M + j / 2;
      if (i % 2 == 0) {
        if (j % 2 == 1) eH[k] = t[(size_t)i * N + j], bH[k] = tB[(size_t)i * N + j];
      } else if (j % 2 == 0) {
        eL[k] = t[(size_t)i * N + j], bL[k] = tB[(size_t)i * N + j];
      } else {
        eR[k] = t[(size_t)i * N + j], bR[k] = tB[(size_t)i * N + j];
      }
    }
  for (int i = 0; i < N / 2; ++i)
    for (int j = 0; j < N; ++j) (j % 2 == 0 ? tD : tU)[(size_t)i * M + j / 2] = tTri[(size_t)i * N + j];
  std::vector<reftd::tinymt32wp_t> st((size_t)M * M);
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
  refcl::gsize[0] = (size_t)M * M; refcl::gsize[1] = 1; refcl::gsize[2] = 1; refcl::gid[1] = 0; refcl::gid[2] = 0;
  for (size_t k = 0; k < st.size(); ++k) {
    refcl::gid[0] = k;
    reftd::InitTinyMT(st.data(), (uint)seed);
  }
  using namespace reftd;
  int *H = eH.data(), *L = eL.data(), *R = eR.data(), *U = tU.data(), *D = tD.data(), *BH = bH.data(),
      *BL = bL.data(), *BR = bR.data();
  reftd::tinymt32wp_t* S = st.data();
  std::default_random_engine generator;
  std::uniform_int_distribution<int> d1(0, 2);
  std::uniform_int_distribution<int> d2(0, 1);
  generator.seed(seed);
  auto butterflies_from_lozenges = [&]() {
    ndrange([&] { UpdateButterflysHFromLozenge(BH, H, L, R, M); });
    ndrange([&] { UpdateButterflysLFromLozenge(BL, H, L, R, M); });
    ndrange([&] { UpdateButterflysRFromLozenge(BR, H, L, R, M); });
  };
  for (long s = 0; s < steps; ++s) {
    const int type = d1(generator), r1 = d1(generator), r2 = d2(generator);
    if (type == 0) {
      int* X = r1 == 0 ? H : r1 == 1 ? L : R;
      ndrange([&] { RotateLozenges(S, X, M, r1, r2); });
      ndrange([&] { UpdateLozengesFlipped(X, M, r1, r2); });
      if (r1 == 0) ndrange([&] { UpdateLozenges0(H, L, R, M); });
      else if (r1 == 1) ndrange([&] { UpdateLozenges1(L, R, H, M); });
      else ndrange([&] { UpdateLozenges2(R, H, L, M); });
      ndrange([&] { UpdateTriangleUFromLozenges(H, L, U, M); });
      ndrange([&] { UpdateTriangles(U, D, M, 0); });
      butterflies_from_lozenges();
    } else if (type == 1) {
      if (r2 == 1) {
        ndrange([&] { RotateTriangles(S, D, M, r1); });
        ndrange([&] { UpdateTrianglesFlipped1(D, M, r1); });
        ndrange([&] { UpdateTriangles(D, U, M, r2); });
      } else {
        ndrange([&] { RotateTriangles(S, U, M, r1); });
        ndrange([&] { UpdateTrianglesFlipped0(U, M, r1); });
        ndrange([&] { UpdateTriangles(U, D, M, r2); });
      }
      ndrange([&] { UpdateLozengeHFromTriangles(U, D, H, M); });
      ndrange([&] { UpdateLozengeLFromTriangles(U, D, L, M); });
      ndrange([&] { UpdateLozengeRFromTriangles(U, D, R, M); });
      butterflies_from_lozenges();
    } else {
      const int p1 = d1(generator), p2 = d2(generator);
      if (r1 == 0) {
        ndrange([&] { RotateButterflys(S, BH, M, r1, p1, p2); });
        ndrange([&] { UpdateButterflysFlippedH1(BH, M, p1, p2); });
        ndrange([&] { UpdateButterflysFlippedH21(BH, M, p1); });
        ndrange([&] { UpdateButterflysFlippedH22(BH, M, p1); });
        ndrange([&] { UpdateButterflysFlippedH23(BH, M, p1); });
        ndrange([&] { UpdateLozengeFromButterflysH(BH, H, L, R, M); });
        ndrange([&] { UpdateButterflysLFromLozenge(BL, H, L, R, M); });
        ndrange([&] { UpdateButterflysRFromLozenge(BR, H, L, R, M); });
      } else if (r1 == 1) {
        ndrange([&] { RotateButterflys(S, BL, M, r1, p1, p2); });
        ndrange([&] { UpdateButterflysFlippedL1(BL, M, p1, p2); });
        ndrange([&] { UpdateButterflysFlippedL21(BL, M, p1); });
        ndrange([&] { UpdateButterflysFlippedL22(BL, M, p1); });
        ndrange([&] { UpdateButterflysFlippedL23(BL, M, p1); });
        ndrange([&] { UpdateLozengeFromButterflysL(BL, H, L, R, M); });
        ndrange([&] { UpdateButterflysHFromLozenge(BH, H, L, R, M); });
        ndrange([&] { UpdateButterflysRFromLozenge(BR, H, L, R, M); });
      } else {
        ndrange([&] { RotateButterflys(S, BR, M, r1, p1, p2); });
        ndrange([&] { UpdateButterflysFlippedR1(BR, M, p1, p2); });
        ndrange([&] { UpdateButterflysFlippedR21(BR, M, p1); });
        ndrange([&] { UpdateButterflysFlippedR22(BR, M, p1); });
        ndrange([&] { UpdateButterflysFlippedR23(BR, M, p1); });
        ndrange([&] { UpdateLozengeFromButterflysR(BR, H, L, R, M); });
        ndrange([&] { UpdateButterflysLFromLozenge(BL, H, L, R, M); });
        ndrange([&] { UpdateButterflysHFromLozenge(BH, H, L, R, M); });
      }
      ndrange([&] { UpdateTriangleUFromLozenges(H, L, U, M); });
      ndrange([&] { UpdateTriangles(U, D, M, 0); });
    }
  }
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      const size_t k = (size_t)(i / 2) * M + j / 2;
      if (i % 2 == 0) {
        if (j % 2 == 1) t[(size_t)i * N + j] = eH[k];
      } else {
        t[(size_t)i * N + j] = j % 2 == 0 ? eL[k] : eR[k];
      }
    }
  return 0;
}
