// Bibone tilings: dimer coverings of regions of the triangular lattice (reference:
// src/TriangleDimer/, class TriangleDimerTiler).
//
// The reference stores, per lattice edge, the states of the edges around it in eight arrays
// (three lozenge, two triangle, three butterfly orientations) and re-derives all of them
// after each move with up to 11 kernels.  Here the state is the dimer configuration itself,
// one byte per vertex (bit 1: H(a,b) = (a,b)-(a,b+1), bit 2: L(a,b) = (a,b)-(a-1,b), bit 4:
// R(a,b) = (a,b)-(a-1,b+1)), and every move of the reference is the toggle of an alternating
// cycle of edges: lozenges (4-cycles, triangledimerkernel.cl:4-22), side-2 triangles
// (6-cycles, :191-211) and butterflies (8-cycles, :331-353).  A step is one kernel: each
// site of the chosen class whose cycle has one half covered flips with probability 1/2.
// Same-class cycles are edge-disjoint (the reference's colourings), and two cycles that can
// flip together share no vertex, so byte read-modify-writes never race.
#include <cuda_runtime.h>
#include <curand_kernel.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "pdl.cuh"
#include "rng.cuh"
#include "rt_internal.h"

namespace rt {
namespace {

enum : uint8_t { kH = 1, kL = 2, kR = 4 };

struct TdEdge {
  int8_t da, db;
  uint8_t bit;
};
struct TdCycle {
  int n;
  TdEdge a[4], b[4];  // the two alternating halves; a = state 5 / 45 / 85, b = 10 / 54 / 170
};

// Cycles by class: lozenge H, L, R (eH/eL/eR of the reference), triangle up / down (tU/tD),
// butterfly H, L, R (bH/bL/bR), at site (a, b).
__constant__ TdCycle c_cycles[8] = {
    {2, {{-1, 0, kR}, {0, 0, kR}}, {{-1, 1, kL}, {0, 0, kL}}},
    {2, {{-1, 0, kH}, {0, -1, kH}}, {{0, 0, kR}, {0, -1, kR}}},
    {2, {{-1, 0, kH}, {0, 0, kH}}, {{0, 1, kL}, {0, 0, kL}}},
    {3, {{-1, 0, kH}, {0, 1, kR}, {1, 0, kL}}, {{0, 0, kL}, {-1, 1, kH}, {1, 0, kR}}},
    {3, {{0, -1, kH}, {0, 1, kL}, {-1, 0, kR}}, {{0, -1, kR}, {0, 0, kH}, {-1, 1, kL}}},
    {4, {{-1, 0, kL}, {-2, 1, kH}, {0, 1, kL}, {0, -1, kH}}, {{-2, 0, kH}, {-1, 1, kR}, {0, 0, kH}, {0, -1, kR}}},
    {4, {{-1, 0, kR}, {0, 1, kL}, {1, -1, kR}, {0, -1, kL}}, {{-1, 1, kL}, {0, 0, kH}, {1, -1, kL}, {-1, -1, kH}}},
    {4, {{-1, 0, kR}, {-1, 1, kH}, {1, 0, kR}, {0, -1, kH}}, {{-1, 1, kL}, {0, 1, kR}, {1, 0, kL}, {0, -1, kR}}},
};

// One step's class: move type (0 lozenge, 1 triangle, 2 butterfly), orientation / colour r1,
// colour r2, butterfly slice p1 and parity p2 (TriangleDimerTiler.cpp:269-276, 459-460).
struct TdStep {
  int type, r1, r2, p1, p2;
};

__host__ __device__ inline int td_cycle_of(const TdStep& s) {
  return s.type == 0 ? s.r1 : s.type == 1 ? (s.r2 == 1 ? 4 : 3) : 5 + s.r1;
}

__host__ __device__ inline bool td_in_class(const TdStep& s, int a, int b) {
  if (s.type == 0) return (((1 - (s.r1 & 1)) * a + ((1 + s.r1) / 2) * b) % 2) == s.r2;
  if (s.type == 1) return (((b - a) % 3 + 3) % 3) == s.r1;
  const int b1 = 1 - (s.r1 & 1), b2 = (1 + s.r1) / 2, b3 = s.r1 & 1;
  return ((b1 * a + b2 * b) % 3) == s.p1 && ((b1 * b + b3 * a) & 1) == s.p2;
}

__device__ __forceinline__ void td_try_flip(uint8_t* D, int M, int c, int a, int b) {
  const TdCycle& C = c_cycles[c];
  bool ha = true, hb = true;
  for (int k = 0; k < C.n; ++k) {
    const int xa = a + C.a[k].da, ya = b + C.a[k].db, xb = a + C.b[k].da, yb = b + C.b[k].db;
    // cycles reaching past the array never move (the padding keeps every domain cycle inside)
    if (xa < 0 || ya < 0 || xa >= M || ya >= M || xb < 0 || yb < 0 || xb >= M || yb >= M) return;
    ha = ha && (D[(size_t)xa * M + ya] & C.a[k].bit);
    hb = hb && (D[(size_t)xb * M + yb] & C.b[k].bit);
  }
  if (!ha && !hb) return;
  for (int k = 0; k < C.n; ++k) {
    D[(size_t)(a + C.a[k].da) * M + b + C.a[k].db] ^= C.a[k].bit;
    D[(size_t)(a + C.b[k].da) * M + b + C.b[k].db] ^= C.b[k].bit;
  }
}

// InitTinyMT (triangledimerkernel.cl:749-756): generator k, of the work item (k / M, k mod M),
// seeded seed + k with its own parameters when a table is loaded.
__global__ void k_td_seed(uint4* st, const uint4* params, int64_t count, uint32_t seed) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const uint4 p = params ? params[k] : make_uint4(kTmtMat1, kTmtMat2, kTmtTmat, 0);
  st[k] = tmt_seed(seed + (uint32_t)k, p.x, p.y, p.z);
}

// TinyMT mode: every generator draws (as every work item of the reference's rotate kernel
// does); sites of the class flip when rd < 0.5, i.e. the 23-bit draw is below 2^22.
__global__ void k_td_step_tmt(uint8_t* D, uint4* tmt, const uint4* params, int M, TdStep s) {
  pdl_begin();
  const int b = blockIdx.x * blockDim.x + threadIdx.x, a = blockIdx.y;
  if (b >= M) return;
  const size_t k = (size_t)a * M + b;
  uint4 g = tmt[k];
  const uint4 p = params ? params[k] : make_uint4(kTmtMat1, kTmtMat2, kTmtTmat, 0);
  const uint32_t u = tmt_next_u23(g, p.x, p.y, p.z);
  tmt[k] = g;
  if (u < (1u << 22) && td_in_class(s, a, b)) td_try_flip(D, M, td_cycle_of(s), a, b);
}

// MTGP mode: the reference's CUDA launch (8 x 8 blocks over the M x M sites, row a from
// the x index, one cuRAND MTGP32 generator per block, TriangleDimerTiler.cpp:279-291); every
// thread draws before its tests (triangledimerkernel.cu, the three Rotate*Kernel).
__global__ void __launch_bounds__(kMtgpBlock* kMtgpBlock) k_td_step_mtgp(uint8_t* D, int M, TdStep s,
                                                                          curandStateMtgp32* states) {
  pdl_begin();
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y * blockDim.y + threadIdx.y;
  const float rd = curand_uniform(states + blockIdx.x * gridDim.y + blockIdx.y);
  if (a >= M || b >= M) return;
  if (rd < 0.5f && td_in_class(s, a, b)) td_try_flip(D, M, td_cycle_of(s), a, b);
}

// Fast mode: a thread owns columns 4q .. 4q+3 of row a and one Philox block of draws.
__global__ void k_td_step_fast(uint8_t* D, int M, TdStep s, uint64_t seed, uint32_t stream, int64_t h) {
  pdl_begin();
  const int q = blockIdx.x * blockDim.x + threadIdx.x, a = blockIdx.y * blockDim.y + threadIdx.y;
  if (4 * q >= M || a >= M) return;
  bool any = false;
#pragma unroll
  for (int k = 0; k < 4; ++k) any |= (4 * q + k < M) && td_in_class(s, a, 4 * q + k);
  if (!any) return;
  const uint4 d = fast_quad(seed, stream, h, (uint32_t)a, (uint32_t)q);
  const uint32_t u[4] = {d.x, d.y, d.z, d.w};
  const int c = td_cycle_of(s);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int b = 4 * q + k;
    if (b < M && u[k] < 0x80000000u && td_in_class(s, a, b)) td_try_flip(D, M, c, a, b);
  }
}

// Philox4x32-10 on the host (the fast-mode step schedule).
void philox_host(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0, n1 = (uint32_t)p1, n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1,
                   n3 = (uint32_t)p0;
    c[0] = n0, c[1] = n1, c[2] = n2, c[3] = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

// Fast-mode schedule: step h's class from Philox(ctr = {~0, ~0, lo32(h), hi16(h) | s << 16}).
TdStep td_fast_step(uint64_t seed, uint32_t stream, int64_t h) {
  uint32_t c[4] = {0xffffffffu, 0xffffffffu, (uint32_t)(uint64_t)h,
                   ((uint32_t)((uint64_t)h >> 32) & 0xffffu) | (stream << 16)};
  philox_host(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  return TdStep{(int)(c[0] % 3u), (int)(c[1] % 3u), (int)(c[2] & 1u), (int)((c[3] >> 1) % 3u), (int)(c[3] & 1u)};
}

void td_from_tiling(const int32_t* t, int N, uint8_t* D) {
  const int M = N / 2;
  for (int a = 0; a < M; ++a)
    for (int b = 0; b < M; ++b) {
      const int eR = t[(size_t)(2 * a + 1) * N + 2 * b + 1], eH = t[(size_t)(2 * a) * N + 2 * b + 1];
      D[(size_t)a * M + b] = (uint8_t)(((eR & 4) ? kH : 0) | ((eR & 8) ? kL : 0) | ((eH & 4) ? kR : 0));
    }
}

// Lozenge states from the dimers (the reference's tiling format); the (even, even) entries,
// which hold no state, are left as they are.
void td_to_tiling(const uint8_t* D, int N, int32_t* t) {
  const int M = N / 2;
  auto bit = [&](int a, int b, int k) -> int {
    return (a >= 0 && b >= 0 && a < M && b < M && (D[(size_t)a * M + b] & k)) ? 1 : 0;
  };
  for (int a = 0; a < M; ++a)
    for (int b = 0; b < M; ++b) {
      t[(size_t)(2 * a) * N + 2 * b + 1] = bit(a - 1, b, kR) + 2 * bit(a - 1, b + 1, kL) + 4 * bit(a, b, kR) + 8 * bit(a, b, kL);
      t[(size_t)(2 * a + 1) * N + 2 * b] = bit(a - 1, b, kH) + 2 * bit(a, b, kR) + 4 * bit(a, b - 1, kH) + 8 * bit(a, b - 1, kR);
      t[(size_t)(2 * a + 1) * N + 2 * b + 1] = bit(a - 1, b, kH) + 2 * bit(a, b + 1, kL) + 4 * bit(a, b, kH) + 8 * bit(a, b, kL);
    }
}

// Number of dimers at each vertex: 0 off the domain, 1 on it for a dimer covering.
std::vector<int> td_cover(const uint8_t* D, int M) {
  std::vector<int> c((size_t)M * M, 0);
  auto add = [&](int a, int b) {
    if (a >= 0 && b >= 0 && a < M && b < M) ++c[(size_t)a * M + b];
  };
  for (int a = 0; a < M; ++a)
    for (int b = 0; b < M; ++b) {
      const uint8_t v = D[(size_t)a * M + b];
      if (v & kH) add(a, b), add(a, b + 1);
      if (v & kL) add(a, b), add(a - 1, b);
      if (v & kR) add(a, b), add(a - 1, b + 1);
    }
  return c;
}

}  // namespace
}  // namespace rt

using namespace rt;

extern "C" {

RT_API rt_status rt_td_icecream_cone(int32_t n, int32_t m, int32_t* out, int64_t cap, int32_t* side) {
  clear_error();
  if (n < 1 || m < 0 || !side) return fail(RT_ERR_INVALID_ARGUMENT, "bibone icecream_cone: n >= 1, m >= 0");
  const int E = n + 4, T = 2 * E, k = ((n + 1) * (n + 2) / 2) % 2;
  *side = T;
  if (!out || cap < (int64_t)T * T) return fail(RT_ERR_BUFFER_TOO_SMALL, "bibone icecream_cone: output too small");
  // As the reference, the layout is built even when m > n - 1 or the vertex count is odd (it
  // prints a warning and covers the domain less its top-right vertex).
  // The reference's dimer layout (TriangleDimerTiler.cpp:714-740): horizontal dimers in every
  // other column, the slanted right side closed by L / R dimers, the cut corner staggered
  std::vector<uint8_t> D((size_t)E * E, 0);
  auto set = [&](int a, int b, uint8_t bit) {
    if (a >= 0 && a < E) D[(size_t)a * E + b] |= bit;
  };
  for (int i = 2; i < E - 2; ++i)
    for (int j = 2; j < E - i; ++j) {
      if (i < m + 2) {
        if ((i + j) % 2 == m % 2 && (m != 0 && j > m + 3 - i)) set(i - 1, j, kH);
        if ((n - m) % 2 == 0 && (i % 2) == 0 && j == E - i - 1) set(i, j, kR);
      } else {
        const bool closes_l = i % 4 == (3 + n % 2 + 2 * k) % 4 && j == E - i - 1;
        if (j % 2 == 0 && !closes_l) set(i - 1, j, kH);
        if (closes_l) set(i, j, kL);
        if (i % 4 == (2 + n % 2 + 2 * k) % 4 && j == E - i - 1) set(i, j, kR);
      }
    }
  std::vector<int32_t> t((size_t)T * T, 0);
  td_to_tiling(D.data(), T, t.data());
  for (int i = 0; i < T; ++i)
    for (int j = 0; j < T; ++j)
      out[(size_t)i * T + j] = (i >= 3 && j >= 3 && i < T - 1 && j < T - 1) ? t[(size_t)i * T + j] : 0;
  return RT_OK;
}

// TriangleDimerTiler::TestButterfly(type) (TriangleDimerTiler.cpp:795-845): one butterfly of
// orientation type (0 H, 1 L, 2 R) of four dimers in a side-16 tiling; other types give the
// all-zero tiling (the reference prints a message).
RT_API rt_status rt_td_test_butterfly(int32_t type, int32_t* out, int64_t cap, int32_t* side) {
  clear_error();
  const int E = 8, T = 2 * E;
  if (!side) return fail(RT_ERR_INVALID_ARGUMENT, "test_butterfly: side is NULL");
  *side = T;
  if (!out || cap < (int64_t)T * T) return fail(RT_ERR_BUFFER_TOO_SMALL, "test_butterfly: output too small");
  std::fill(out, out + (size_t)T * T, 0);
  if (type < 0 || type > 2) return RT_OK;
  std::vector<uint8_t> D((size_t)E * E, 0);
  auto set = [&](int a, int b, uint8_t bit) { D[(size_t)a * E + b] |= bit; };
  // the reference's h edges sit one vertex row below the edge they stand for
  if (type == 0) set(1, 3, kH), set(3, 3, kH), set(2, 4, kR), set(3, 2, kR);
  else if (type == 1) set(2, 3, kR), set(4, 2, kR), set(3, 2, kL), set(3, 4, kL);
  else set(2, 4, kL), set(4, 3, kL), set(3, 2, kR), set(3, 4, kR);
  std::vector<int32_t> t((size_t)T * T, 0);
  td_to_tiling(D.data(), T, t.data());
  for (int i = 3; i < T - 1; ++i)
    for (int j = 3; j < T - 1; ++j) out[(size_t)i * T + j] = t[(size_t)i * T + j];
  return RT_OK;
}

// TriangleDimerTiler::TilingToTriangleFlips (:846-873): (N/2) x N; row i, even column j the
// state of the down triangle, odd column the up triangle, as three base-4 digits (the edge of
// each neighbouring triangle that holds a dimer: 1, 2, 3, or 0), read from the lozenge states.
RT_API rt_status rt_td_triangle_flips(const int32_t* t, int32_t n_side, int32_t* out) {
  clear_error();
  if (!t || !out || n_side < 4 || n_side % 2) return fail(RT_ERR_INVALID_ARGUMENT, "triangle_flips: even side >= 4");
  const int N = n_side;
  auto at = [&](int i, int j) { return t[(size_t)i * N + j]; };
  std::fill(out, out + (size_t)(N / 2) * N, 0);
  for (int i = 1; i < N / 2 - 1; ++i)
    for (int j = 1; j < N - 1; ++j) {
      const int eL = at(2 * i + 1, j), eR = at(2 * i + 1, j + 1), eU = at(2 * i, j + 1);  // j even: down triangle
      int v;
      if (j % 2 == 0) {
        v = (((eL >> 2) & 1) + 2 * ((eL >> 3) & 1) + 3 * ((eR >> 3) & 1)) +
            4 * (((eR >> 2) & 1) + 2 * ((eL >> 1) & 1) + 3 * ((eR >> 1) & 1)) +
            16 * (2 * (eU & 1) + (eL & 1) + 3 * ((eU >> 1) & 1));
      } else {
        const int r = at(2 * i + 1, j), l = at(2 * i + 1, j + 1), h = at(2 * i + 2, j);  // odd: up triangle
        v = ((r & 1) + 2 * ((r >> 3) & 1) + 3 * ((l >> 3) & 1)) + 4 * ((l & 1) + 2 * ((r >> 1) & 1) + 3 * ((l >> 1) & 1)) +
            16 * (2 * ((h >> 3) & 1) + 3 * ((h >> 2) & 1) + ((r >> 2) & 1));
      }
      out[(size_t)i * N + j] = v;
    }
  return RT_OK;
}

// TriangleDimerTiler::TilingToButterflyFlips (:875-921): N x N, at each H / L / R position
// the four neighbouring triangles' digits (weights 1, 4, 16, 64) and the centre edge (256).
RT_API rt_status rt_td_butterfly_flips(const int32_t* t, int32_t n_side, int32_t* out) {
  clear_error();
  if (!t || !out || n_side < 4 || n_side % 2) return fail(RT_ERR_INVALID_ARGUMENT, "butterfly_flips: even side >= 4");
  const int N = n_side;
  auto at = [&](int i, int j) { return t[(size_t)i * N + j]; };
  auto bit = [](int v, int k) { return (v >> k) & 1; };
  std::fill(out, out + (size_t)N * N, 0);
  for (int i = 2; i < N - 2; ++i)
    for (int j = 2; j < N - 2; ++j) {
      const int c0 = at(i, j);
      int f1, f4, f16, f64, c;
      if (i % 2 == 0) {
        if (j % 2 == 0) continue;
        const int up = at(i - 1, j), upr = at(i - 1, j + 1), dn = at(i + 1, j), dnl = at(i + 1, j - 1);
        f1 = bit(up, 3) + 2 * bit(up, 0) + 3 * bit(c0, 0);
        f4 = bit(upr, 0) + 2 * bit(upr, 1) + 3 * bit(c0, 1);
        f16 = bit(dn, 1) + 2 * bit(dn, 2) + 3 * bit(c0, 2);
        f64 = bit(dnl, 2) + 2 * bit(dnl, 3) + 3 * bit(c0, 3);
        c = bit(upr, 2);
      } else if (j % 2 == 0) {
        const int ur = at(i - 1, j + 1), rr = at(i, j + 1), dl = at(i + 1, j - 1), ll = at(i, j - 1);
        f1 = bit(ur, 0) + 2 * bit(ur, 1) + 3 * bit(c0, 0);
        f4 = bit(rr, 1) + 2 * bit(rr, 2) + 3 * bit(c0, 1);
        f16 = bit(dl, 2) + 2 * bit(dl, 3) + 3 * bit(c0, 2);
        f64 = bit(ll, 3) + 2 * bit(ll, 0) + 3 * bit(c0, 3);
        c = bit(rr, 3);
      } else {
        const int uu = at(i - 1, j), rr = at(i, j + 1), dd = at(i + 1, j), ll = at(i, j - 1);
        f1 = bit(uu, 0) + 2 * bit(uu, 1) + 3 * bit(c0, 0);
        f4 = bit(rr, 0) + 2 * bit(rr, 1) + 3 * bit(c0, 1);
        f16 = bit(dd, 2) + 2 * bit(dd, 3) + 3 * bit(c0, 2);
        f64 = bit(ll, 2) + 2 * bit(ll, 3) + 3 * bit(c0, 3);
        c = bit(rr, 3);
      }
      out[(size_t)i * N + j] = f1 + 4 * f4 + 16 * f16 + 64 * f64 + 256 * c;
    }
  return RT_OK;
}

RT_API rt_status rt_td_rhombus_brick(int32_t rows, int32_t cols, int32_t* out, int64_t cap, int32_t* side) {
  clear_error();
  if (rows < 1 || cols < 2 || cols % 2 || !side)
    return fail(RT_ERR_INVALID_ARGUMENT, "bibone rhombus: rows >= 1 and an even number of columns >= 2");
  const int M = std::max(rows, cols) + 6, T = 2 * M;
  *side = T;
  if (!out || cap < (int64_t)T * T) return fail(RT_ERR_BUFFER_TOO_SMALL, "bibone rhombus: output too small");
  std::vector<uint8_t> D((size_t)M * M, 0);
  for (int a = 0; a < rows; ++a)
    for (int b = 0; b < cols; b += 2) D[(size_t)(a + 3) * M + b + 3] = kH;
  std::fill(out, out + (size_t)T * T, 0);
  td_to_tiling(D.data(), T, out);
  return RT_OK;
}

RT_API rt_status rt_td_dimers(const int32_t* t, int32_t n_side, uint8_t* out) {
  clear_error();
  if (!t || !out || n_side < 2 || n_side % 2) return fail(RT_ERR_INVALID_ARGUMENT, "bibone dimers: even side >= 2");
  td_from_tiling(t, n_side, out);
  return RT_OK;
}

RT_API rt_status rt_td_from_dimers(const uint8_t* dimers, int32_t n_side, int32_t* out) {
  clear_error();
  if (!dimers || !out || n_side < 2 || n_side % 2) return fail(RT_ERR_INVALID_ARGUMENT, "bibone from_dimers: even side >= 2");
  td_to_tiling(dimers, n_side, out);
  return RT_OK;
}

// TriangleDimerTiler::TilingToVertices (TriangleDimerTiler.cpp:923-949): an (N/2+1)^2 grid,
// entry (i, j) (2 <= i, j < N/2 - 1) is 1 when vertex (i-1, j) is covered by a dimer.
RT_API rt_status rt_td_vertices(const int32_t* tiling, int32_t n_side, int32_t* out) {
  clear_error();
  if (!tiling || !out || n_side < 4 || n_side % 2) return fail(RT_ERR_INVALID_ARGUMENT, "bibone vertices: even side >= 4");
  const int M = n_side / 2, V = M + 1;
  std::vector<uint8_t> D((size_t)M * M);
  td_from_tiling(tiling, n_side, D.data());
  const std::vector<int> c = td_cover(D.data(), M);
  std::fill(out, out + (size_t)V * V, 0);
  for (int i = 2; i < V - 2; ++i)
    for (int j = 2; j < V - 2; ++j) out[(size_t)i * V + j] = c[(size_t)(i - 1) * M + j] > 0;
  return RT_OK;
}

// TriangleDimerTiler::TilingToDomain (:951-982): (V-1) x 2(V-1) triangles over the vertex grid
// above, even columns the triangle (i, j/2), (i, j/2+1), (i+1, j/2), odd columns
// (i, j/2+1), (i+1, j/2), (i+1, j/2+1); 1 when all three vertices are covered.
RT_API rt_status rt_td_domain(const int32_t* tiling, int32_t n_side, int32_t* out) {
  clear_error();
  if (!tiling || !out || n_side < 4 || n_side % 2) return fail(RT_ERR_INVALID_ARGUMENT, "bibone domain: even side >= 4");
  const int V = n_side / 2 + 1;
  std::vector<int32_t> v((size_t)V * V);
  rt_td_vertices(tiling, n_side, v.data());
  auto at = [&](int i, int j) { return v[(size_t)i * V + j]; };
  for (int i = 0; i < V - 1; ++i)
    for (int j = 0; j < 2 * (V - 1); ++j) {
      const bool in = j % 2 == 0 ? (at(i, j / 2) && at(i, j / 2 + 1) && at(i + 1, j / 2))
                                 : (at(i, j / 2 + 1) && at(i + 1, j / 2) && at(i + 1, j / 2 + 1));
      out[(size_t)i * 2 * (V - 1) + j] = in ? 1 : 0;
    }
  return RT_OK;
}

// TriangleDimerTiler::DimerIndicator(t, c) (:35-99): M x M, for c = 0 the horizontal dimers
// (entry (a, b) is the edge (a-1, b)-(a-1, b+1)), c = 1 the up-left ones (a, b)-(a-1, b),
// c = 2 the up-right ones (a, b)-(a-1, b+1).
RT_API rt_status rt_td_dimer_indicator(const int32_t* tiling, int32_t n_side, int32_t c, int32_t* out) {
  clear_error();
  if (!tiling || !out || n_side < 4 || n_side % 2 || c < 0 || c > 2)
    return fail(RT_ERR_INVALID_ARGUMENT, "bibone dimer_indicator: even side >= 4, c in {0, 1, 2}");
  const int M = n_side / 2;
  std::vector<uint8_t> D((size_t)M * M);
  td_from_tiling(tiling, n_side, D.data());
  for (int a = 0; a < M; ++a)
    for (int b = 0; b < M; ++b) {
      const int v = c == 0 ? (a > 0 ? (D[(size_t)(a - 1) * M + b] & kH) : 0)
                           : (D[(size_t)a * M + b] & (c == 1 ? kL : kR));
      out[(size_t)a * M + b] = v ? 1 : 0;
    }
  return RT_OK;
}

RT_API rt_status rt_td_mtgp_draws(int32_t n_side, int64_t seed, int64_t launches, float* out) {
  clear_error();
  if (n_side < 8 || n_side % 2 || n_side > 2 * 32767 || launches < 0 || (launches > 0 && !out))
    return fail(RT_ERR_INVALID_ARGUMENT, "bibone mtgp_draws: even n_side in [8, 65534], launches >= 0");
  return mtgp_draws_grid(n_side / 2, n_side / 2, seed, launches, out);
}

RT_API rt_status rt_td_walk(int32_t* tiling, int32_t n_side, int64_t steps, int64_t seed, const rt_walk_opts* opts,
                            rt_cftp_stats* stats) {
  clear_error();
  rt_walk_opts o;
  rt_walk_opts_default(&o);
  if (opts) o = *opts;
  if (!tiling || steps < 0) return fail(RT_ERR_INVALID_ARGUMENT, "bibone walk: NULL tiling or negative steps");
  if (n_side < 8 || n_side % 2 || n_side > 2 * 32767)
    return fail(RT_ERR_INVALID_ARGUMENT, "bibone tiling side must be even, in [8, 65534]");
  if (o.rng_mode != RT_RNG_TINYMT && o.rng_mode != RT_RNG_FAST && o.rng_mode != RT_RNG_MTGP)
    return fail(RT_ERR_INVALID_ARGUMENT, "unknown rng mode");
  if (o.rng_mode == RT_RNG_FAST && o.fast_stream >= 65536u) return fail(RT_ERR_INVALID_ARGUMENT, "fast_stream must be < 65536");
  if (o.tinymt_params && o.rng_mode != RT_RNG_TINYMT)
    return fail(RT_ERR_INVALID_ARGUMENT, "bibone walk: a TinyMT parameter table needs the TinyMT mode");
  const int N = n_side, M = N / 2;
  std::vector<uint8_t> D((size_t)M * M);
  td_from_tiling(tiling, N, D.data());
  {
    // the state must be a dimer covering of its vertex set, and must round-trip
    std::vector<int32_t> back((size_t)N * N, 0);
    for (size_t p = 0; p < back.size(); ++p) back[p] = tiling[p];
    td_to_tiling(D.data(), N, back.data());
    for (size_t p = 0; p < back.size(); ++p)
      if (back[p] != tiling[p]) return fail(RT_ERR_INVALID_ARGUMENT, "bibone walk: tiling states are not those of a dimer configuration");
    for (int v : td_cover(D.data(), M))
      if (v > 1) return fail(RT_ERR_INVALID_ARGUMENT, "bibone walk: two dimers share a vertex");
  }
  int devs = 0;
  if (cudaGetDeviceCount(&devs) != cudaSuccess || devs == 0) {
    cudaGetLastError();
    return fail(RT_ERR_CUDA, "no CUDA device: the sweep has no CPU fallback");
  }
  // flip attempts: sites of each class whose cycle anchor is a covered vertex
  std::vector<int> cover = td_cover(D.data(), M);
  cudaStream_t st = (cudaStream_t)o.cuda_stream;
  uint8_t* dD = nullptr;
  uint4 *tmt = nullptr, *tmt_params = nullptr;
  void* mtgp = nullptr;
  const MtgpGrid mg = mtgp_grid(M, M);
  auto cleanup = [&]() {
    if (dD) cudaFree(dD);
    if (tmt) cudaFree(tmt);
    if (tmt_params) cudaFree(tmt_params);
    if (mtgp) cudaFree(mtgp);
  };
  if (cudaMalloc(&dD, D.size()) != cudaSuccess ||
      (o.rng_mode == RT_RNG_TINYMT && cudaMalloc(&tmt, (size_t)M * M * sizeof(uint4)) != cudaSuccess) ||
      (o.rng_mode == RT_RNG_MTGP && cudaMalloc(&mtgp, mtgp_state_bytes(mg.count())) != cudaSuccess)) {
    cudaGetLastError();
    cleanup();
    return fail(RT_ERR_OUT_OF_MEMORY, "bibone walk: device allocation failed");
  }
  cudaMemcpyAsync(dD, D.data(), D.size(), cudaMemcpyHostToDevice, st);
  if (o.rng_mode == RT_RNG_TINYMT) {
    if (rt_status ps = tmt_param_table(o, (int64_t)M * M, &tmt_params, st)) {
      cleanup();
      return ps;
    }
  }
  std::vector<TdStep> sched((size_t)steps);
  if (o.rng_mode != RT_RNG_FAST) {
    // TriangleDimerTiler.cpp:269-276, 459-460: type, r1, r2 (and p1, p2 for butterflies)
    std::default_random_engine gen;
    std::uniform_int_distribution<int> d1(0, 2), d2(0, 1);
    gen.seed(seed);
    for (auto& s : sched) {
      s.type = d1(gen);
      s.r1 = d1(gen);
      s.r2 = d2(gen);
      s.p1 = s.p2 = 0;
      if (s.type == 2) s.p1 = d1(gen), s.p2 = d2(gen);
    }
  } else {
    for (int64_t h = 0; h < steps; ++h) sched[(size_t)h] = td_fast_step((uint64_t)seed, o.fast_stream, h);
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  if (o.rng_mode == RT_RNG_TINYMT) {
    const int64_t count = (int64_t)M * M;
    k_td_seed<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(tmt, tmt_params, count, (uint32_t)seed);
  } else if (o.rng_mode == RT_RNG_MTGP) {
    // TriangleDimerTiler.cpp:287-289: block generator k seeded seed + k
    if (rt_status ms = mtgp_seed(mtgp, mg.count(), seed, st)) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      cleanup();
      return ms;
    }
  }
  cudaEventRecord(e0, st);
  const dim3 g_all((M + 127) / 128, M), g_quad(((M + 3) / 4 + 31) / 32, (M + 7) / 8);
  for (int64_t h = 0; h < steps; ++h) {
    if (o.rng_mode == RT_RNG_TINYMT)
      pdl_launch(k_td_step_tmt, g_all, dim3(128), st, dD, tmt, (const uint4*)tmt_params, M, sched[(size_t)h]);
    else if (o.rng_mode == RT_RNG_MTGP)
      pdl_launch(k_td_step_mtgp, dim3(mg.gx, mg.gy), dim3(kMtgpBlock, kMtgpBlock), st, dD, M, sched[(size_t)h],
                 static_cast<curandStateMtgp32*>(mtgp));
    else
      pdl_launch(k_td_step_fast, g_quad, dim3(32, 8), st, dD, M, sched[(size_t)h], (uint64_t)seed, o.fast_stream, h);
  }
  cudaEventRecord(e1, st);
  cudaError_t le = cudaGetLastError();
  cudaMemcpyAsync(D.data(), dD, D.size(), cudaMemcpyDeviceToHost, st);
  const cudaError_t se = cudaStreamSynchronize(st);
  float ms = 0.f;
  if (se == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cleanup();
  if (le != cudaSuccess || se != cudaSuccess)
    return fail(RT_ERR_CUDA, std::string("bibone walk: ") + cudaGetErrorString(le != cudaSuccess ? le : se));
  td_to_tiling(D.data(), N, tiling);
  if (stats) {
    std::memset(stats, 0, sizeof *stats);
    // per class, the sites whose anchor vertex is covered
    int64_t attempts = 0;
    std::vector<int64_t> per_class(3 * 3 * 2 * 3 * 2, -1);
    for (const TdStep& s : sched) {
      const size_t key = (((size_t)s.type * 3 + s.r1) * 2 + s.r2) * 6 + (s.type == 2 ? s.p1 * 2 + s.p2 : 0);
      if (per_class[key] < 0) {
        int64_t c = 0;
        for (int a = 0; a < M; ++a)
          for (int b = 0; b < M; ++b) c += cover[(size_t)a * M + b] && td_in_class(s, a, b);
        per_class[key] = c;
      }
      attempts += per_class[key];
    }
    stats->attempts = 1;
    stats->total_steps = steps;
    stats->final_steps = steps;
    stats->flip_attempts = attempts;
    stats->seconds = ms * 1e-3;
  }
  return RT_OK;
}

}  // extern "C"
