// Rectangle-triangle tilings of a hexagon (reference: src/RectTriangle/).
//
// A vertex of the triangular lattice holds the covering codes of its six surrounding
// triangles, one hexadecimal digit each (d5..d0 as drawn at RectTriangleTiler.h:14-22).  The
// sweep has three colours, (i - j) mod 3.  One step draws a colour, offers every vertex of
// that colour a move - with probability 0.9 - and rebuilds the six digits of each vertex of
// the two other colours from its neighbours.  The offered move, and whether the weight ratio
// accepts it, follow flipTiles (recttrianglekernel.cl:25-118):
//   * the five hexagons made of triangles or of one rectangle move to the state picked by
//     the quarter of the rescaled draw;
//   * the twelve rectangle-pair hexagons toggle with their partner.
// The nine weights are runtime arguments; the reference hard-codes them at
// recttrianglekernel.cl:3-11.  MTGP mode: the reference's CUDA build's random stream (8 x 8
// blocks over the N x N/3 slots of the drawn colour, one cuRAND MTGP32 generator per block
// seeded seed + block; RectTriangleTiler.cpp:75-85, recttrianglekernel.cu:31-43).
#include <cuda_runtime.h>
#include <curand_kernel.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "pdl.cuh"
#include "rng.cuh"
#include "rt_internal.h"

namespace rt {
namespace {

struct RtWeights {
  float w[16];  // by digit: 0, wt1..3, wr1..3, wr1..3, wm1..3, wm1..3 (recttrianglekernel.cl:13)
};

__host__ __device__ inline float ratio_of(const RtWeights& W, int a, int b) {
  const float* w = W.w;
  return (w[(b >> 20) & 15] * w[(b >> 16) & 15] * w[(b >> 12) & 15] * w[(b >> 8) & 15] * w[(b >> 4) & 15] * w[b & 15]) /
         (w[(a >> 20) & 15] * w[(a >> 16) & 15] * w[(a >> 12) & 15] * w[(a >> 8) & 15] * w[(a >> 4) & 15] * w[a & 15]);
}

// The decision of flipTiles for state hex and uniform rd in [0, 1): float arithmetic in the
// reference's order (rd / 0.9f, quarter boundaries, (rd - sc) * 4).
__host__ __device__ inline int rt_flip(int hex, float rd, const RtWeights& W) {
  if (!(rd < 0.9f)) return hex;
  rd /= 0.9f;
  int next = hex;
  float sc = rd < 0.25f ? 0.0f : (rd < 0.5f ? 0.25f : (rd < 0.75f ? 0.5f : 0.75f));
  if (hex == 0x122133 || hex == 0x331221 || hex == 0x8ebbe8 || hex == 0xfc99cf || hex == 0xa7dd7a) {
    const int target = rd < 0.25f ? 0xa7dd7a : (rd < 0.5f ? 0xfc99cf : (rd < 0.75f ? 0x8ebbe8 : 0x331221));
    next = target == hex ? 0x122133 : target;
  } else {
    switch (hex) {
      case 0x47d47a: next = 0xd22a33; break;
      case 0xd22a33: next = 0x47d47a; break;
      case 0xa74d74: next = 0x33a22d; break;
      case 0x33a22d: next = 0xa74d74; break;
      case 0x8eb558: next = 0x331eb1; break;
      case 0x331eb1: next = 0x8eb558; break;
      case 0x855be8: next = 0x1be133; break;
      case 0x1be133: next = 0x855be8; break;
      case 0x6699cf: next = 0xcf1221; break;
      case 0xcf1221: next = 0x6699cf; break;
      case 0xfc9966: next = 0x1221fc; break;
      case 0x1221fc: next = 0xfc9966; break;
      default: return hex;  // no move offered: ratio 1 (or 0/0) leaves the state as it is
    }
    sc = 1.0f;
  }
  const float ratio = ratio_of(W, hex, next);
  rd = (sc == 1.0f) ? rd : (rd - sc) * 4;
  return ratio >= rd ? next : hex;
}

struct RtView {
  int32_t* base;
  int N, M, P;
  size_t colour_stride;
  uint4* tmt;
  const uint4* tmt_params;  // per-generator {mat1, mat2, tmat} (LoadTinyMT), or NULL
  __device__ int32_t* colour(int c) const { return base + (size_t)c * colour_stride; }
};

// InitTinyMT (recttrianglekernel.cl:148-155): generator k, of the work item (k / M, k mod M),
// seeded seed + k with its own parameters when a table is loaded.
__global__ void k_rt_seed(uint4* st, const uint4* params, int64_t count, uint32_t seed) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const uint4 p = params ? params[k] : make_uint4(kTmtMat1, kTmtMat2, kTmtTmat, 0);
  st[k] = tmt_seed(seed + (uint32_t)k, p.x, p.y, p.z);
}

__global__ void k_rt_flip_tmt(RtView v, int r, RtWeights W) {
  pdl_begin();
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
  if (j >= v.M) return;
  const int64_t k = (int64_t)i * v.M + j;
  uint4 s = v.tmt[k];
  const uint4 pr = v.tmt_params ? v.tmt_params[k] : make_uint4(kTmtMat1, kTmtMat2, kTmtTmat, 0);
  const uint32_t u = tmt_next_u23(s, pr.x, pr.y, pr.z);
  v.tmt[k] = s;
  int32_t* p = v.colour(r) + (size_t)i * v.P + j;
  const int e = *p, n = rt_flip(e, (float)u * (1.0f / 8388608.0f), W);
  if (n != e) *p = n;
}

// MTGP mode: every thread of the block draws before the bounds test (recttrianglekernel.cu:35-43);
// flipTilesKernel decides as flipTiles does.
__global__ void __launch_bounds__(kMtgpBlock* kMtgpBlock) k_rt_flip_mtgp(RtView v, int r, RtWeights W,
                                                                          curandStateMtgp32* states) {
  pdl_begin();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const float rd = curand_uniform(states + blockIdx.x * gridDim.y + blockIdx.y);
  if (i >= v.N || j >= v.M) return;
  int32_t* p = v.colour(r) + (size_t)i * v.P + j;
  const int e = *p, n = rt_flip(e, rd, W);
  if (n != e) *p = n;
}

__global__ void k_rt_flip_fast(RtView v, int r, RtWeights W, uint64_t seed, uint32_t stream, int64_t h) {
  pdl_begin();
  const int q = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
  if (4 * q >= v.M) return;
  const uint4 d = fast_quad(seed, stream, h, (uint32_t)i, (uint32_t)q);
  const uint32_t u4[4] = {d.x, d.y, d.z, d.w};
  int32_t* row = v.colour(r) + (size_t)i * v.P;
#pragma unroll
  for (int k4 = 0; k4 < 4; ++k4) {
    const int j = 4 * q + k4;
    if (j >= v.M) break;
    const int e = row[j], n = rt_flip(e, (float)(u4[k4] >> 8) * (1.0f / 16777216.0f), W);
    if (n != e) row[j] = n;
  }
}

// updateTiles1 / updateTiles2 (recttrianglekernel.cl:120-146): the digits of colour
// (r+1) mod 3 and (r+2) mod 3 rebuilt from the rotated colour's neighbours.
__global__ void k_rt_update(RtView v, int r) {
  pdl_begin();
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1, i = blockIdx.y + 1;
  if (j > v.M - 2 || i > v.N - 2) return;
  const int32_t* A = v.colour(r);
  const int im = i % 3;
  {
    const int p1 = im == r, p2 = im == (r + 1) % 3;
    const int up = A[(size_t)(i - 1) * v.P + j], same = A[(size_t)i * v.P + j + p1], dn = A[(size_t)(i + 1) * v.P + j - p2];
    v.colour((r + 1) % 3)[(size_t)i * v.P + j] = ((up & 0xf0) << 16) | ((up & 0xf) << 16) | ((same & 0xf00000) >> 8) |
                                                  ((dn & 0x0f0000) >> 8) | ((dn & 0x00f000) >> 8) | ((same & 0xf00) >> 8);
  }
  {
    const int p1 = im == (r + 2) % 3, p2 = im == (r + 1) % 3;
    const int same = A[(size_t)i * v.P + j - p1], up = A[(size_t)(i - 1) * v.P + j + p2], dn = A[(size_t)(i + 1) * v.P + j];
    v.colour((r + 2) % 3)[(size_t)i * v.P + j] = ((same & 0xf000) << 8) | ((up & 0xf00) << 8) | ((up & 0xf0) << 8) |
                                                  ((same & 0xf) << 8) | ((dn & 0xf00000) >> 16) | ((dn & 0x0f0000) >> 16);
  }
}

// Region codes of the extremal tilings of the hexagon of side n (RectTriangleTiler.cpp:
// 480-600), then the shear of row i by n + 3 - i columns into a padded array whose side is a
// multiple of 3.
std::vector<int32_t> hex_extremal(int n, bool top) {
  const int M = 2 * n + 1;
  std::vector<int32_t> t((size_t)M * M, 0);
  auto at = [&](int i, int j) -> int32_t& { return t[(size_t)i * M + j]; };
  for (int i = 1; i < M - 1; ++i)
    for (int j = top ? 0 : 1; j < (top ? M : M - 1); ++j) {
      if (j - i > n || i - j > n) continue;
      int32_t v = 0;
      if (top) {
        if (i < n && j < n) v = 0x333333;
        else if (i < j && j > n) v = 0x111111;
        else if (i > n && i > j) v = 0x222222;
        else if (i == n && j < n) v = 0x333222;
        else if (i < n && j == n) v = 0x331311;
        else if (i == j && i > n) v = 0x211221;
        else if (i == n && j == n) v = 0x331221;
      } else {
        if (i > n && j > n) v = 0x333333;
        else if (i > j && j < n) v = 0x111111;
        else if (i < n && i < j) v = 0x222222;
        else if (i == n && j > n) v = 0x222333;
        else if (i > n && j == n) v = 0x113133;
        else if (i == j && i < n) v = 0x122112;
        else if (i == n && j == n) v = 0x122133;
      }
      at(i, j) = v;
    }
  // the rim of the hexagon: half-covered vertices
  const int32_t edge[2][6] = {{0x001011, 0x000222, 0x330300, 0x333000, 0x200220, 0x011001},
                              {0x003033, 0x000333, 0x110100, 0x222000, 0x100110, 0x022002}};
  const int32_t* e = edge[top ? 1 : 0];
  for (int i = 1; i < n; ++i) at(i, 0) = e[0], at(0, i) = e[1];
  for (int i = n + 1; i < M - 1; ++i) at(i, M - 1) = e[2], at(M - 1, i) = e[3];
  for (int i = 1; i < n; ++i) at(i, i + n) = e[4], at(i + n, i) = e[5];
  if (top) {
    at(0, 0) = 0x000033; at(n, 0) = 0x003002; at(0, n) = 0x000310;
    at(M - 1, M - 1) = 0x210000; at(n, M - 1) = 0x100100; at(M - 1, n) = 0x022000;
  } else {
    at(0, 0) = 0x000012; at(M - 1, n) = 0x013000; at(n, M - 1) = 0x200300;
    at(0, n) = 0x000220; at(n, 0) = 0x001001; at(M - 1, M - 1) = 0x330000;
  }
  const int M2 = M + 6 + (3 - M % 3) % 3;
  std::vector<int32_t> out((size_t)M2 * M2, 0);
  for (int i = 0; i < M; ++i)
    for (int j = 0; j < M; ++j) {
      const int j2 = j + n + 3 - i;
      if (j2 < M2) out[(size_t)(i + 3) * M2 + j2] = t[(size_t)i * M + j];
    }
  return out;
}

// slopeHex (RectTriangleTiler.cpp:173-478): a start tiling of the hexagon of side n with the
// hexagon split into six sloped sectors, each filled with a two-row (or two-column) periodic
// pattern of rectangles, stitched along the three main lines and the diagonal.  Every vertex
// (i, j) of the (2n+1)^2 array takes the code of the first region (in this order) that holds
// it; `alt` picks between a region's two codes.
std::vector<int32_t> hex_slope(int n) {
  const int M = 2 * n + 1;
  const bool ev = n % 2 == 0;
  std::vector<int32_t> t((size_t)M * M, 0);
  auto code = [&](int i, int j) -> int32_t {
    auto pick = [](bool odd, int32_t a, int32_t b) { return odd ? a : b; };
    const bool io = i % 2 == 1, jo = j % 2 == 1, pa = (i + j) % 2 != n % 2;
    if (i == n && j == n) return ev ? 0x213312 : 0x122133;
    if (i == n) {
      if (j < n - 1) return pick(jo, 0x1be1fc, 0xe81c91);
      if (j == n - 1) return ev ? 0x122133 : 0xe81c91;
      if (j > n + 1) return pick(jo, 0xcf1eb1, 0x19c18e);
      return ev ? 0x331221 : 0x29c38e;  // j == n + 1
    }
    if (j == n) {
      if (i < n - 1) return pick(io, 0xd22afc, 0x7af229);
      if (i == n - 1) return ev ? 0x122133 : 0x7af229;
      if (i > n + 1) return pick(io, 0xcfa22d, 0x922fa7);
      return ev ? 0x331221 : 0x913fa7;  // i == n + 1
    }
    if (i == j) {
      if (i < n - 1) return pick(io, 0x33aebd, 0xbd7833);
      if (i > n + 1) return pick(io, 0xdbea33, 0x3387db);
      if (i == n + 1) return ev ? 0x122133 : 0x3387db;
      return ev ? 0x331221 : 0xbd7812;  // i == n - 1
    }
    if (i < n && j < i) {
      if (i == n - 1 && j < i - 1) return pick(jo, 0x855be8, 0x58881b);
      if (i < n - 1 && j == i - 1) return pick(jo, 0x8eb558, 0x58388e);
      if (i == n - 1 && j == i - 1) return ev ? 0x583812 : 0x8ebbe8;
      return pick(jo, 0x855558, 0x588885);
    }
    if (i > n && j > i) {
      if (i == n + 1 && j > i + 1) return pick(jo, 0x8eb558, 0xb18885);
      if (i > n + 1 && j == i + 1) return pick(jo, 0x855be8, 0xe88385);
      if (i == n + 1 && j == i + 1) return ev ? 0x218385 : 0x8ebbe8;
      return pick(jo, 0x855558, 0x588885);
    }
    if (j < n && i < j) {
      if (j == n - 1 && i < j - 1) return pick(io, 0x47d47a, 0x7477d2);
      if (j < n - 1 && i == j - 1) return pick(io, 0xa74d74, 0x7473a7);
      if (j == n - 1 && i == j - 1) return ev ? 0x747312 : 0xa7dd7a;
      return pick(io, 0x474474, 0x747747);
    }
    if (j > n && i > j) {
      if (j == n + 1 && i > j + 1) return pick(io, 0xa74d74, 0x2d7747);
      if (j > n + 1 && i == j + 1) return pick(io, 0x47d47a, 0x7a3747);
      if (j == n + 1 && i == j + 1) return ev ? 0x213747 : 0xa7dd7a;
      return pick(io, 0x474474, 0x747747);
    }
    if (i < n && j > n && i > j - n) {
      if (i == n - 1 && j > n + 1) return pick(pa, 0x6699cf, 0x996f19);
      if (i < n - 1 && j == n + 1) return pick(pa, 0xfc9966, 0x296c99);
      if (i == n - 1 && j == n + 1) return ev ? 0x296319 : 0xfc99cf;
      return pick(pa, 0x669966, 0x996699);
    }
    if (i > n && j < n && i < j + n) {
      if (i == n + 1 && j < n - 1) return pick(pa, 0xfc9966, 0x91f699);
      if (i > n + 1 && j == n - 1) return pick(pa, 0x6699cf, 0x99c692);
      if (i == n + 1 && j == n - 1) return ev ? 0x913692 : 0xfc99cf;
      return pick(pa, 0x669966, 0x996699);
    }
    return 0;
  };
  for (int i = 1; i < M - 1; ++i)
    for (int j = 1; j < M - 1; ++j) t[(size_t)i * M + j] = code(i, j);
  auto at = [&](int i, int j) -> int32_t& { return t[(size_t)i * M + j]; };
  // the rim: runs of half-covered vertices along the six sides, then their ends
  for (int i = 2; i < n - 1; ++i) at(i, 0) = 0x008085, at(0, i) = 0x000747;
  at(1, 0) = 0x00308e, at(0, 1) = 0x0003a7, at(n - 1, 0) = 0x00801b, at(0, n - 1) = 0x0007d2;
  for (int i = n + 2; i < M - 2; ++i) at(i, M - 1) = 0x580800, at(M - 1, i) = 0x747000;
  at(n + 1, M - 1) = 0xb10800, at(M - 1, n + 1) = 0x2d7000, at(M - 2, M - 1) = 0xe80300, at(M - 1, M - 2) = 0x7a3000;
  for (int i = 2; i < n - 1; ++i) at(i, i + n) = 0x900690, at(i + n, i) = 0x096009;
  at(1, n + 1) = 0x200c90, at(n + 1, 1) = 0x01f009, at(n - 1, M - 2) = 0x900f10, at(M - 2, n - 1) = 0x09c002;
  // the six corners (n == 1: the single hexagon of triangles)
  at(0, 0) = n == 1 ? 0x000012 : 0x000033;
  at(M - 1, n) = n == 1 ? 0x013000 : 0x022000;
  at(n, M - 1) = n == 1 ? 0x200300 : 0x100100;
  at(0, n) = 0x000220, at(n, 0) = 0x001001, at(M - 1, M - 1) = 0x330000;
  const int M2 = M + 6 + (3 - M % 3) % 3;
  std::vector<int32_t> out((size_t)M2 * M2, 0);
  for (int i = 0; i < M; ++i)
    for (int j = 0; j < M; ++j) {
      const int j2 = j + n + 3 - i;
      if (j2 < M2) out[(size_t)(i + 3) * M2 + j2] = t[(size_t)i * M + j];
    }
  return out;
}

RtWeights make_weights(const double* w9) {
  // w9 = {wt1, wt2, wt3, wm1, wm2, wm3, wr1, wr2, wr3}; NULL: all 1 (the reference's values)
  float v[9];
  for (int k = 0; k < 9; ++k) v[k] = w9 ? (float)w9[k] : 1.0f;
  RtWeights W;
  const float tab[16] = {0.0f, v[0], v[1], v[2], v[6], v[7], v[8], v[6], v[7], v[8], v[3], v[4], v[5], v[3], v[4], v[5]};
  std::memcpy(W.w, tab, sizeof tab);
  return W;
}

}  // namespace
}  // namespace rt

using namespace rt;

extern "C" {

RT_API rt_status rt_recttri_hex_tiling(int32_t n, int32_t top, int32_t* out, int64_t cap, int32_t* side) {
  clear_error();
  if (n < 2 || !side || top < 0 || top > 2) return fail(RT_ERR_INVALID_ARGUMENT, "recttri hex_tiling: side n >= 2, top 0, 1 or 2");
  std::vector<int32_t> t = top == 2 ? hex_slope(n) : hex_extremal(n, top != 0);
  const int s = (int)std::lround(std::sqrt((double)t.size()));
  *side = s;
  if (!out || cap < (int64_t)t.size()) return fail(RT_ERR_BUFFER_TOO_SMALL, "recttri hex_tiling: output too small");
  std::memcpy(out, t.data(), t.size() * sizeof(int32_t));
  return RT_OK;
}

// Each lozenge triangle of the domain becomes one triangle of the rectangle-triangle tiling,
// its digit (1, 2, 3) the orientation of the lozenge covering it, written into the three
// vertices around it (RectTriangleTiler.cpp:602-644).  Up triangles (even domain column)
// touch vertices (i, j/2), (i, j/2 + 1), (i + 1, j/2); down triangles (odd column) touch
// (i, j/2 + 1), (i + 1, j/2), (i + 1, j/2 + 1).
RT_API rt_status rt_recttri_from_lozenge(const int32_t* lozenge, int32_t n_side, const int32_t* domain, int32_t m_rows,
                                         int32_t* out) {
  clear_error();
  if (!lozenge || !domain || !out || n_side < 1 || m_rows < 1)
    return fail(RT_ERR_INVALID_ARGUMENT, "recttri from_lozenge: NULL buffer or empty size");
  const int N = n_side, M = m_rows;
  std::fill(out, out + (size_t)N * N, 0);
  for (int i = 0; i < M; ++i)
    for (int j = 0; j < 2 * M; ++j) {
      if (domain[(size_t)i * 2 * M + j] != 1) continue;
      const int64_t a = (int64_t)i * N + j / 2 + (j & 1);  // the vertex whose edge mask is read
      const int64_t v[3] = {a, j & 1 ? a + N - 1 : a + 1, a + N};
      const int sh[3] = {j & 1 ? 4 : 0, j & 1 ? 12 : 8, j & 1 ? 20 : 16};
      if (i + 1 >= N || j / 2 + 1 >= N) return fail(RT_ERR_INVALID_ARGUMENT, "recttri from_lozenge: domain needs padding");
      const int e = lozenge[a];
      const int d = (j & 1) ? ((e & 16) ? 2 : (e & 32) ? 3 : 1) : ((e & 8) ? 1 : (e & 32) ? 3 : 2);
      for (int k = 0; k < 3; ++k) out[v[k]] += d << sh[k];
    }
  return RT_OK;
}

RT_API rt_status rt_recttri_mtgp_draws(int32_t n_side, int64_t seed, int64_t launches, float* out) {
  clear_error();
  if (n_side < 9 || n_side % 3 || n_side > 32766 || launches < 0 || (launches > 0 && !out))
    return fail(RT_ERR_INVALID_ARGUMENT, "recttri mtgp_draws: n_side a multiple of 3 in [9, 32766], launches >= 0");
  return mtgp_draws_grid(n_side, n_side / 3, seed, launches, out);
}

RT_API rt_status rt_recttri_walk(int32_t* tiling, int32_t n_side, int64_t steps, int64_t seed, const double* weights9,
                                 const rt_walk_opts* opts) {
  clear_error();
  rt_walk_opts o;
  rt_walk_opts_default(&o);
  if (opts) o = *opts;
  if (!tiling || steps < 0) return fail(RT_ERR_INVALID_ARGUMENT, "recttri walk: NULL tiling or negative steps");
  if (n_side < 9 || n_side % 3 || n_side > 32766)
    return fail(RT_ERR_INVALID_ARGUMENT, "recttri tiling side must be a multiple of 3 in [9, 32766]");
  if (o.rng_mode != RT_RNG_TINYMT && o.rng_mode != RT_RNG_FAST && o.rng_mode != RT_RNG_MTGP)
    return fail(RT_ERR_INVALID_ARGUMENT, "unknown rng mode");
  if (o.rng_mode == RT_RNG_FAST && o.fast_stream >= 65536u) return fail(RT_ERR_INVALID_ARGUMENT, "fast_stream must be < 65536");
  if (o.tinymt_params && o.rng_mode != RT_RNG_TINYMT)
    return fail(RT_ERR_INVALID_ARGUMENT, "recttri walk: a TinyMT parameter table needs the TinyMT mode");
  for (size_t p = 0; p < (size_t)n_side * n_side; ++p)
    if ((uint32_t)tiling[p] > 0xffffffu) return fail(RT_ERR_INVALID_ARGUMENT, "recttri tiling values must be six hex digits");
  int devs = 0;
  if (cudaGetDeviceCount(&devs) != cudaSuccess || devs == 0) {
    cudaGetLastError();
    return fail(RT_ERR_CUDA, "no CUDA device: the sweep has no CPU fallback");
  }
  const int N = n_side, M = N / 3, P = (M + 3) / 4 * 4;
  const RtWeights W = make_weights(weights9);
  cudaStream_t stream = (cudaStream_t)o.cuda_stream;
  int32_t *base = nullptr, *scratch = nullptr;
  uint4 *tmt = nullptr, *tmt_params = nullptr;
  void* mtgp = nullptr;
  const MtgpGrid mg = mtgp_grid(N, M);
  auto cleanup = [&]() {
    if (base) cudaFree(base);
    if (scratch) cudaFree(scratch);
    if (tmt) cudaFree(tmt);
    if (tmt_params) cudaFree(tmt_params);
    if (mtgp) cudaFree(mtgp);
  };
  const size_t cs = (size_t)N * P;
  rt_status status = RT_OK;
  do {
    if (cudaMalloc(&base, 3 * cs * sizeof(int32_t)) != cudaSuccess || cudaMalloc(&scratch, (size_t)N * N * sizeof(int32_t)) != cudaSuccess ||
        (o.rng_mode == RT_RNG_TINYMT && cudaMalloc(&tmt, (size_t)N * M * sizeof(uint4)) != cudaSuccess) ||
        (o.rng_mode == RT_RNG_MTGP && cudaMalloc(&mtgp, mtgp_state_bytes(mg.count())) != cudaSuccess)) {
      cudaGetLastError();
      status = fail(RT_ERR_OUT_OF_MEMORY, "recttri walk: device allocation failed");
      break;
    }
    // colour split on the host (the reference does the same, RectTriangleTiler.cpp:35-51)
    std::vector<int32_t> h(3 * cs, 0);
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) h[(size_t)(((i - j) % 3 + 3) % 3) * cs + (size_t)i * P + j / 3] = tiling[(size_t)i * N + j];
    cudaMemcpyAsync(base, h.data(), h.size() * sizeof(int32_t), cudaMemcpyHostToDevice, stream);
    if (o.rng_mode == RT_RNG_TINYMT && (status = tmt_param_table(o, (int64_t)N * M, &tmt_params, stream)) != RT_OK) break;
    RtView v{base, N, M, P, cs, tmt, tmt_params};
    const dim3 gr((M + 127) / 128, N), gq(((M + 3) / 4 + 127) / 128, N), gu((M + 127) / 128, N - 2);
    if (o.rng_mode == RT_RNG_TINYMT) {
      const int64_t count = (int64_t)N * M;
      k_rt_seed<<<(unsigned)((count + 255) / 256), 256, 0, stream>>>(tmt, tmt_params, count, (uint32_t)seed);
      // RectTriangleTiler.cpp:74-76: colours from default_random_engine(seed)
      std::default_random_engine gen;
      std::uniform_int_distribution<int> dist(0, 2);
      gen.seed(seed);
      for (int64_t s = 0; s < steps; ++s) {
        const int r = dist(gen);
        pdl_launch(k_rt_flip_tmt, gr, dim3(128), stream, v, r, W);
        pdl_launch(k_rt_update, gu, dim3(128), stream, v, r);
      }
    } else if (o.rng_mode == RT_RNG_MTGP) {
      // RectTriangleTiler.cpp:75-85 (CUDA branch): block generator k seeded seed + k; the
      // colours as above.
      if ((status = mtgp_seed(mtgp, mg.count(), seed, stream)) != RT_OK) break;
      std::default_random_engine gen;
      std::uniform_int_distribution<int> dist(0, 2);
      gen.seed(seed);
      for (int64_t s = 0; s < steps; ++s) {
        const int r = dist(gen);
        pdl_launch(k_rt_flip_mtgp, dim3(mg.gx, mg.gy), dim3(kMtgpBlock, kMtgpBlock), stream, v, r, W,
                   static_cast<curandStateMtgp32*>(mtgp));
        pdl_launch(k_rt_update, gu, dim3(128), stream, v, r);
      }
    } else {
      for (int64_t s = 0; s < steps; ++s) {
        const int r = (int)(s % 3);
        pdl_launch(k_rt_flip_fast, gq, dim3(128), stream, v, r, W, (uint64_t)seed, o.fast_stream, s);
        pdl_launch(k_rt_update, gu, dim3(128), stream, v, r);
      }
    }
    cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) {
      status = fail(RT_ERR_CUDA, std::string("recttri walk: ") + cudaGetErrorString(le));
      break;
    }
    cudaMemcpyAsync(h.data(), base, h.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    cudaError_t se = cudaStreamSynchronize(stream);
    if (se != cudaSuccess) {
      status = fail(RT_ERR_CUDA, std::string("recttri walk: ") + cudaGetErrorString(se));
      break;
    }
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) tiling[(size_t)i * N + j] = h[(size_t)(((i - j) % 3 + 3) % 3) * cs + (size_t)i * P + j / 3];
  } while (false);
  cleanup();
  return status;
}

}  // extern "C"
