// Six-vertex model: heat-bath sweep and coupling from the past on the height function.
//
// The reference has no six-vertex model; the definition is the library's own:
//   * n x n vertices, height points (y, x), 0 <= y, x <= n; h(below) - h(above) = +1 across a
//     horizontal edge whose arrow points right, h(right) - h(left) = +1 across a vertical
//     edge whose arrow points up;
//   * vertex types from the corner heights NW, NE, SW, SE: a (NE == SW, NW != SE), b (NW ==
//     SE, NE != SW), c (both equal), weights a, b, c;
//   * four point classes (x mod 2, y mod 2); sub-sweep s updates class s mod 4 by heat bath at
//     every interior point whose four edge neighbours share one height h': h' + 1 with
//     probability P(k1, k2), h' - 1 otherwise (k1, k2: diagonal points equal to h' + 1 on the
//     a/c and on the b/c diagonals), drawn as u < T[3 k1 + k2], u from 32 Philox bit planes.
//
// Layout in HBM.  Heights are kept mod 4; within a class the parity of x + y is fixed, so one
// bit per point is enough (sigma = ((h - parity) / 2) mod 2).  One chain = 4 class arrays,
// each R = n/2 + 1 rows of P 32-bit words; word 0 and the words past the data are zero guards,
// bit b of data word w is point k = 32 w + b of the class row (x = 2k + px, y = 2r + py).
// A thread owns one word: 32 points updated with bitwise logic, the random comparison done
// bit-sliced from the most significant plane down and stopped once every lane is decided.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "pdl.cuh"
#include "rng.cuh"
#include "rt_internal.h"

namespace rt {
namespace {

struct SvGeom {
  int n, R, P;           // side, rows per class, words per row (with guards)
  size_t class_words;    // R * P
  size_t chain_words;    // 4 * R * P
};

SvGeom sv_geom(int n) {
  SvGeom g;
  g.n = n;
  g.R = n / 2 + 1;
  g.P = (n / 2 + 1 + 31) / 32 + 2;
  g.class_words = (size_t)g.R * g.P;
  g.chain_words = 4 * g.class_words;
  return g;
}

struct SvLaunch {
  uint32_t* base;   // chain 0; chain c at base + c * chain_words
  size_t chain_words, class_words;
  int P, n;
  int px, py, r_lo, words, rows;  // the class being updated and its interior extent
  int k_lo, k_hi;
  uint32_t leaf[32][9];  // leaf[j][m]: all ones where bit j of threshold T[m] is set (sv_leaves)
  uint64_t seed;
  uint32_t stream;
  int64_t s;
};

// Per-plane leaf words of the nine heat-bath thresholds: leaf[j][m] is all ones where bit j
// of T[m] is set, so that a point's threshold bit in plane j is the OR over the nine
// vertex-weight classes m of (class mask & leaf[j][m]) - one three-input logic operation
// each, with the leaf a constant operand once the plane loop is unrolled.
inline void sv_leaves(const uint32_t* T, uint32_t (&leaf)[32][9]) {
  for (int j = 0; j < 32; ++j)
    for (int m = 0; m < 9; ++m) leaf[j][m] = ((T[m] >> j) & 1u) ? 0xffffffffu : 0u;
}

__device__ __forceinline__ uint32_t west_of(const uint32_t* row, int idx, int px) {
  return px ? row[idx] : __funnelshift_l(row[idx - 1], row[idx], 1);
}
__device__ __forceinline__ uint32_t east_of(const uint32_t* row, int idx, int px) {
  return px ? __funnelshift_r(row[idx], row[idx + 1], 1) : row[idx];
}

// The rows one word update reads and writes: the word's own row F (class px, py), the same
// row of class (1-px, py) (west/east neighbours), rows above/below of class (px, 1-py)
// (north/south) and of class (1-px, 1-py) (diagonals).
struct SvRows {
  uint32_t* F;
  const uint32_t *H, *Vn, *Vs, *Dn, *Ds;
};

// Updates data word w (index idx = w + 1) of class row r in NCH chains that share the draws.
__device__ __forceinline__ uint4 sv_block(uint32_t w, uint32_t r, int q, uint32_t c2, uint32_t c3, uint64_t seed) {
  return philox4x32_10(make_uint4(w | ((uint32_t)q << 24), r, c2, c3), (uint32_t)seed, (uint32_t)(seed >> 32));
}

// Blocks q < NPRE of the draws arrive precomputed in pre[] (they do not depend on the state).
template <int NCH, int NPRE = 0>
__device__ __forceinline__ void sv_update_word(const SvRows (&rows)[NCH], int idx, int px, int py, uint32_t imask,
                                               uint32_t w, uint32_t r, const uint32_t (&leaf)[32][9], uint64_t seed,
                                               uint32_t c2, uint32_t c3, const uint4* pre = nullptr) {
  uint32_t f[NCH], flip[NCH], sup[NCH], mk[NCH][9], lt[NCH], und[NCH];
  uint32_t any = 0;
#pragma unroll
  for (int c = 0; c < NCH; ++c) {
    const SvRows& R = rows[c];
    f[c] = R.F[idx];
    const uint32_t wv = west_of(R.H, idx, px), ev = east_of(R.H, idx, px);
    const uint32_t nv = R.Vn[idx], sv = R.Vs[idx];
    flip[c] = ~(wv ^ ev) & ~(wv ^ nv) & ~(wv ^ sv) & imask;
    sup[c] = (px ^ py) ? wv : ~wv;  // sigma of h' + 1 (neighbour parity 1 - (px ^ py))
    const uint32_t e1a = ~(west_of(R.Dn, idx, px) ^ sup[c]), e1b = ~(east_of(R.Ds, idx, px) ^ sup[c]);
    const uint32_t e2a = ~(east_of(R.Dn, idx, px) ^ sup[c]), e2b = ~(west_of(R.Ds, idx, px) ^ sup[c]);
    const uint32_t a0 = ~(e1a | e1b), a1 = e1a ^ e1b, a2 = e1a & e1b;
    const uint32_t b0 = ~(e2a | e2b), b1 = e2a ^ e2b, b2 = e2a & e2b;
    mk[c][0] = a0 & b0, mk[c][1] = a0 & b1, mk[c][2] = a0 & b2;
    mk[c][3] = a1 & b0, mk[c][4] = a1 & b1, mk[c][5] = a1 & b2;
    mk[c][6] = a2 & b0, mk[c][7] = a2 & b1, mk[c][8] = a2 & b2;
    lt[c] = 0;
    und[c] = flip[c];
    any |= flip[c];
  }
  if (!any) return;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    uint32_t open = 0;
#pragma unroll
    for (int c = 0; c < NCH; ++c) open |= und[c];
    if (!open) break;
    const uint4 Rq = q < NPRE ? pre[q] : sv_block(w, r, q, c2, c3, seed);
    const uint32_t planes[4] = {Rq.x, Rq.y, Rq.z, Rq.w};
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int j = 31 - (4 * q + t);
#pragma unroll
      for (int c = 0; c < NCH; ++c) {
        uint32_t Tj = 0;  // bit j of each point's threshold
#pragma unroll
        for (int m = 0; m < 9; ++m) Tj |= mk[c][m] & leaf[j][m];
        lt[c] |= und[c] & ~planes[t] & Tj;
        und[c] &= ~(planes[t] ^ Tj);
      }
    }
  }
#pragma unroll
  for (int c = 0; c < NCH; ++c)
    if (flip[c]) rows[c].F[idx] = (f[c] & ~flip[c]) | (flip[c] & ~(lt[c] ^ sup[c]));
}

__device__ __forceinline__ uint32_t interior_mask(int w, int k_lo, int k_hi) {
  const int k0 = 32 * w;
  const int lo = max(k_lo - k0, 0), hi = min(k_hi - k0, 31);
  if (hi < lo) return 0u;
  return (hi - lo == 31 ? 0xffffffffu : ((1u << (hi - lo + 1)) - 1u)) << lo;
}

// One sub-sweep of one class over global memory; blockIdx.y is the chain.
__global__ void __launch_bounds__(128) k_sv_sub(SvLaunch L) {
  pdl_begin();
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= L.words * L.rows) return;
  const int w = g % L.words, r = L.r_lo + g / L.words;
  const int px = L.px, py = L.py, cls = px | (py << 1);
  const uint32_t imask = interior_mask(w, L.k_lo, L.k_hi);
  if (!imask) return;
  uint32_t* chain = L.base + (size_t)blockIdx.y * L.chain_words;
  const uint32_t* V = chain + (size_t)(cls ^ 2) * L.class_words;
  const uint32_t* D = chain + (size_t)(cls ^ 3) * L.class_words;
  const int rn = py ? r : r - 1, rs = py ? r + 1 : r;
  const SvRows rows[1] = {{chain + (size_t)cls * L.class_words + (size_t)r * L.P,
                           chain + (size_t)(cls ^ 1) * L.class_words + (size_t)r * L.P, V + (size_t)rn * L.P,
                           V + (size_t)rs * L.P, D + (size_t)rn * L.P, D + (size_t)rs * L.P}};
  const uint32_t c2 = (uint32_t)(uint64_t)L.s, c3 = ((uint32_t)((uint64_t)L.s >> 32) & 0xffffu) | (L.stream << 16);
  sv_update_word<1>(rows, w + 1, px, py, imask, (uint32_t)w, (uint32_t)r, L.leaf, L.seed, c2, c3);
}

// Resident engine: one thread-block cluster holds NCH chains in shared memory, CTA `rank`
// owning class rows [rank * rpc, rank * rpc + rpc) of all four classes; the one halo row
// above and below is read from the neighbouring CTA's shared memory (distributed shared
// memory).  A cluster barrier separates sub-sweeps; no other waits.
struct SvClusterArgs {
  uint32_t* base;
  size_t chain_words, class_words;
  int P, n, R, rpc;
  uint32_t leaf[32][9];  // as SvLaunch::leaf
  uint64_t seed;
  uint32_t stream;
  int64_t s0, count;
};

template <int NCH>
constexpr int sv_cluster_max_threads() {
  return 512;
}

__device__ __forceinline__ void cluster_arrive_release() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait_acquire() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }

// The class rows, words and interior columns of sub-sweep s restricted to rows [r0, r1).
struct SvSub {
  int px, py, cls, r_lo, r_hi, k_lo, k_hi, words;
  uint32_t c2, c3;
};

__device__ __forceinline__ SvSub sv_sub_of(int64_t s, int n, int r0, int r1, uint32_t stream) {
  SvSub u;
  u.px = (int)(s & 1);
  u.py = (int)((s >> 1) & 1);
  u.cls = u.px | (u.py << 1);
  u.r_lo = max(u.py ? 0 : 1, r0);
  u.r_hi = min((n - 1 - u.py) / 2, r1 - 1);
  u.k_lo = u.px ? 0 : 1;
  u.k_hi = (n - 1 - u.px) / 2;
  u.words = u.k_hi / 32 + 1;
  u.c2 = (uint32_t)(uint64_t)s;
  u.c3 = ((uint32_t)((uint64_t)s >> 32) & 0xffffu) | (stream << 16);
  return u;
}

template <int NCH>
__global__ void __launch_bounds__(sv_cluster_max_threads<NCH>()) k_sv_cluster(SvClusterArgs A) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ uint32_t sm[];  // [NCH][4][rpc][P]
  const int rank = (int)cluster.block_rank(), C = (int)cluster.num_blocks();
  const int r0 = rank * A.rpc, r1 = min(r0 + A.rpc, A.R), P = A.P;
  const int own = max(r1 - r0, 0);
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int i = tid; i < NCH * 4 * own * P; i += nt) {
    const int p = i % P, lr = (i / P) % own, cc = i / (P * own);  // cc = chain * 4 + class
    sm[((size_t)cc * A.rpc + lr) * P + p] =
        A.base[(size_t)(cc >> 2) * A.chain_words + (size_t)(cc & 3) * A.class_words + (size_t)(r0 + lr) * P + p];
  }
  // shared memory of the CTAs above and below (rows r0 - 1 and r1 live there)
  uint32_t* const up = rank > 0 ? cluster.map_shared_rank(sm, rank - 1) : sm;
  uint32_t* const dn = rank + 1 < C ? cluster.map_shared_rank(sm, rank + 1) : sm;
  const size_t plane = (size_t)A.rpc * P;  // words of one class of one chain
  auto row = [&](int c, int cls, int r) -> uint32_t* {
    uint32_t* b = r < r0 ? up + (size_t)(A.rpc - 1) * P : r >= r1 ? dn : sm + (size_t)(r - r0) * P;
    return b + (size_t)(c * 4 + cls) * plane;
  };
  const int n = A.n;
  constexpr int kPre = 2;
  uint4 pre[kPre];
  SvSub u = sv_sub_of(A.s0, n, r0, r1, A.stream);
  if (tid < (u.r_hi - u.r_lo + 1) * u.words)
    for (int q = 0; q < kPre; ++q) pre[q] = sv_block(tid % u.words, u.r_lo + tid / u.words, q, u.c2, u.c3, A.seed);
  cluster.sync();
  for (int64_t s = A.s0; s < A.s0 + A.count; ++s) {
    const int items = (u.r_hi - u.r_lo + 1) * u.words;
    for (int it = tid; it < items; it += nt) {
      const int w = it % u.words, r = u.r_lo + it / u.words;
      const uint32_t imask = interior_mask(w, u.k_lo, u.k_hi);
      if (!imask) continue;
      const int rn = u.py ? r : r - 1, rs = u.py ? r + 1 : r;
      SvRows rows[NCH];
#pragma unroll
      for (int c = 0; c < NCH; ++c)
        rows[c] = {row(c, u.cls, r), row(c, u.cls ^ 1, r), row(c, u.cls ^ 2, rn), row(c, u.cls ^ 2, rs),
                   row(c, u.cls ^ 3, rn), row(c, u.cls ^ 3, rs)};
      if (it == tid)
        sv_update_word<NCH, kPre>(rows, w + 1, u.px, u.py, imask, (uint32_t)w, (uint32_t)r, A.leaf, A.seed, u.c2, u.c3, pre);
      else
        sv_update_word<NCH>(rows, w + 1, u.px, u.py, imask, (uint32_t)w, (uint32_t)r, A.leaf, A.seed, u.c2, u.c3);
    }
    // the next sub-sweep's first draws do not depend on the state: compute them while the
    // other CTAs of the cluster reach the barrier
    cluster_arrive_release();
    u = sv_sub_of(s + 1, n, r0, r1, A.stream);
    if (s + 1 < A.s0 + A.count && tid < (u.r_hi - u.r_lo + 1) * u.words)
      for (int q = 0; q < kPre; ++q) pre[q] = sv_block(tid % u.words, u.r_lo + tid / u.words, q, u.c2, u.c3, A.seed);
    cluster_wait_acquire();
  }
  for (int i = tid; i < NCH * 4 * own * P; i += nt) {
    const int p = i % P, lr = (i / P) % own, cc = i / (P * own);
    A.base[(size_t)(cc >> 2) * A.chain_words + (size_t)(cc & 3) * A.class_words + (size_t)(r0 + lr) * P + p] =
        sm[((size_t)cc * A.rpc + lr) * P + p];
  }
}

// OR of (top ^ bottom) over all words of the two chains.
__global__ void k_sv_diff(const uint32_t* a, const uint32_t* b, size_t words, uint32_t* flag) {
  uint32_t acc = 0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += (size_t)gridDim.x * blockDim.x)
    acc |= a[i] ^ b[i];
  acc = __reduce_or_sync(0xffffffffu, acc);
  if ((threadIdx.x & 31) == 0 && acc) atomicOr(flag, 1u);
}

void fill_launch(SvLaunch& L, const SvGeom& G, int64_t s) {
  L.px = (int)(s & 1);
  L.py = (int)((s >> 1) & 1);
  L.s = s;
  const int n = G.n;
  L.r_lo = L.py ? 0 : 1;
  const int r_hi = (n - 1 - L.py) / 2;
  L.rows = r_hi - L.r_lo + 1;
  L.k_lo = L.px ? 0 : 1;
  L.k_hi = (n - 1 - L.px) / 2;
  L.words = L.k_hi / 32 + 1;
}

}  // namespace

// ---- host side ------------------------------------------------------------------------

std::vector<uint32_t> sv_thresholds_host(double a, double b, double c) {
  std::vector<uint32_t> T(9);
  for (int k1 = 0; k1 < 3; ++k1)
    for (int k2 = 0; k2 < 3; ++k2) {
      double wp = 1.0, wm = 1.0;
      for (int i = 0; i < 2; ++i) wp *= i < k1 ? c : a, wm *= i < 2 - k1 ? c : a;
      for (int i = 0; i < 2; ++i) wp *= i < k2 ? c : b, wm *= i < 2 - k2 ? c : b;
      const double scaled = std::floor(wp / (wp + wm) * 4294967296.0);
      T[3 * k1 + k2] = scaled >= 4294967295.0 ? 0xffffffffu : (uint32_t)scaled;
    }
  return T;
}

// Checks |dh| = 1 across every edge; returns false otherwise.
bool sv_valid_heights(const int32_t* h, int n) {
  const int L = n + 1;
  for (int y = 0; y <= n; ++y)
    for (int x = 0; x <= n; ++x) {
      const int v = h[(size_t)y * L + x];
      if (x < n && std::abs(h[(size_t)y * L + x + 1] - v) != 1) return false;
      if (y < n && std::abs(h[(size_t)(y + 1) * L + x] - v) != 1) return false;
    }
  return true;
}

void sv_pack(const int32_t* h, const SvGeom& G, uint32_t* out) {
  const int n = G.n, L = n + 1, o = h[0] & 1;
  std::fill(out, out + G.chain_words, 0u);
  for (int y = 0; y <= n; ++y)
    for (int x = 0; x <= n; ++x) {
      const int v = h[(size_t)y * L + x] - o, p = (x + y) & 1;
      const uint32_t sigma = (uint32_t)(((v - p) >> 1) & 1);
      const int cls = (x & 1) | ((y & 1) << 1), r = y >> 1, k = x >> 1;
      out[(size_t)cls * G.class_words + (size_t)r * G.P + 1 + (k >> 5)] |= sigma << (k & 31);
    }
}

// Heights from the bits, anchored on the left column of the start heights (the boundary is
// never updated): along each row h moves by the step of +-1 that lands on the stored residue.
void sv_unpack(const uint32_t* bits, const SvGeom& G, const int32_t* start, int32_t* out) {
  const int n = G.n, L = n + 1, o = start[0] & 1;
  for (int y = 0; y <= n; ++y) {
    int prev = start[(size_t)y * L];
    out[(size_t)y * L] = prev;
    for (int x = 1; x <= n; ++x) {
      const int cls = (x & 1) | ((y & 1) << 1), r = y >> 1, k = x >> 1;
      const uint32_t sigma = (bits[(size_t)cls * G.class_words + (size_t)r * G.P + 1 + (k >> 5)] >> (k & 31)) & 1u;
      const int residue = (((x + y) & 1) + 2 * (int)sigma + o) & 3;
      const int up = prev + 1;
      prev = ((up & 3) == residue) ? up : prev - 1;
      out[(size_t)y * L + x] = prev;
    }
  }
}

namespace {

struct SvDevice {
  uint32_t* chains = nullptr;
  uint32_t* flag = nullptr;
  ~SvDevice() {
    if (chains) cudaFree(chains);
    if (flag) cudaFree(flag);
  }
};

rt_status sv_check_common(int32_t n, const double* abc, double* a, double* b, double* c) {
  if (n < 2 || n > 65534) return fail(RT_ERR_INVALID_ARGUMENT, "six-vertex: n must be in [2, 65534]");
  *a = abc ? abc[0] : 1.0;
  *b = abc ? abc[1] : 1.0;
  *c = abc ? abc[2] : 1.0;
  for (double v : {*a, *b, *c})
    if (!(v > 0.0) || !std::isfinite(v)) return fail(RT_ERR_INVALID_ARGUMENT, "six-vertex: weights must be finite and > 0");
  return RT_OK;
}

rt_status sv_check_device() {
  int devs = 0;
  if (cudaGetDeviceCount(&devs) != cudaSuccess || devs == 0) {
    cudaGetLastError();
    return fail(RT_ERR_CUDA, "no CUDA device: the sweep has no CPU fallback");
  }
  return RT_OK;
}

struct SvClusterPlan {
  bool ok = false;
  int C = 0, rpc = 0, threads = 0;
  size_t smem = 0;
};

template <int NCH>
SvClusterPlan sv_cluster_plan_for(const SvGeom& G) {
  SvClusterPlan best;
  const int words = (G.n / 2) / 32 + 1;
  for (int cmax : {16, 8}) {
    SvClusterPlan p;
    p.rpc = (G.R + cmax - 1) / cmax;
    p.C = (G.R + p.rpc - 1) / p.rpc;
    p.smem = (size_t)NCH * 4 * p.rpc * G.P * sizeof(uint32_t);
    if (p.smem > 200 * 1024) continue;
    p.threads = std::min(sv_cluster_max_threads<NCH>(), std::max(64, (p.rpc * words + 31) / 32 * 32));
    auto kern = k_sv_cluster<NCH>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p.smem) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(p.C);
    cfg.blockDim = dim3(p.threads);
    cfg.dynamicSmemBytes = p.smem;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = p.C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, kern, &cfg) != cudaSuccess || clusters < 1) {
      cudaGetLastError();
      continue;
    }
    p.ok = true;
    return p;
  }
  return best;
}

SvClusterPlan sv_cluster_plan(const SvGeom& G, int chains) {
  return chains == 1 ? sv_cluster_plan_for<1>(G) : sv_cluster_plan_for<2>(G);
}

// Per-CTA work above which the whole-GPU per-sub-sweep kernels are faster than one cluster.
constexpr int kSvClusterMaxItems = 256;

bool sv_use_cluster(const SvGeom& G, const SvClusterPlan& p, int engine) {
  if (engine == 1 || !p.ok) return false;
  if (engine == 2) return true;
  return (int64_t)p.rpc * ((G.n / 2) / 32 + 1) <= kSvClusterMaxItems;
}

// Sub-sweeps [s0, s0 + count) on `chains` (1 or 2) chains stored back to back at dev;
// returns the kernel launches, or -1 when engine 2 was asked for and no cluster fits.
int64_t sv_run(uint32_t* dev, int chains, const SvGeom& G, const std::vector<uint32_t>& T, uint64_t seed,
               uint32_t stream, int64_t s0, int64_t count, cudaStream_t st, int engine) {
  const SvClusterPlan plan = engine == 1 ? SvClusterPlan{} : sv_cluster_plan(G, chains);
  if (engine == 2 && !plan.ok) return -1;
  int64_t launches = 0;
  if (sv_use_cluster(G, plan, engine)) {
    SvClusterArgs A{};
    A.base = dev;
    A.chain_words = G.chain_words;
    A.class_words = G.class_words;
    A.P = G.P;
    A.n = G.n;
    A.R = G.R;
    A.rpc = plan.rpc;
    sv_leaves(T.data(), A.leaf);
    A.seed = seed;
    A.stream = stream;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(plan.C);
    cfg.blockDim = dim3(plan.threads);
    cfg.dynamicSmemBytes = plan.smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = plan.C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    constexpr int64_t kChunk = 8192;  // sub-sweeps per launch
    for (int64_t done = 0; done < count; done += kChunk) {
      A.s0 = s0 + done;
      A.count = std::min(kChunk, count - done);
      if (chains == 1)
        cudaLaunchKernelEx(&cfg, k_sv_cluster<1>, A);
      else
        cudaLaunchKernelEx(&cfg, k_sv_cluster<2>, A);
      ++launches;
    }
    return launches;
  }
  SvLaunch L{};
  L.base = dev;
  L.chain_words = G.chain_words;
  L.class_words = G.class_words;
  L.P = G.P;
  L.n = G.n;
  sv_leaves(T.data(), L.leaf);
  L.seed = seed;
  L.stream = stream;
  for (int64_t s = s0; s < s0 + count; ++s) {
    fill_launch(L, G, s);
    const int threads = L.words * L.rows;
    if (threads <= 0) continue;
    pdl_launch(k_sv_sub, dim3((threads + 127) / 128, chains), dim3(128), st, L);
    ++launches;
  }
  return launches;
}

int64_t sv_interior_points(int n) { return (int64_t)(n - 1) * (n - 1); }

}  // namespace
}  // namespace rt

using namespace rt;

extern "C" {

RT_API rt_status rt_sv_thresholds(double a, double b, double c, uint32_t* out9) {
  clear_error();
  if (!out9) return fail(RT_ERR_INVALID_ARGUMENT, "six-vertex thresholds: NULL output");
  if (!(a > 0 && b > 0 && c > 0) || !std::isfinite(a) || !std::isfinite(b) || !std::isfinite(c))
    return fail(RT_ERR_INVALID_ARGUMENT, "six-vertex: weights must be finite and > 0");
  const std::vector<uint32_t> T = sv_thresholds_host(a, b, c);
  std::memcpy(out9, T.data(), 9 * sizeof(uint32_t));
  return RT_OK;
}

RT_API rt_status rt_sv_dwbc_height(int32_t n, int32_t top, int32_t* out) {
  clear_error();
  if (n < 1 || !out) return fail(RT_ERR_INVALID_ARGUMENT, "six-vertex dwbc: n >= 1 and an output of (n+1)^2");
  const int L = n + 1;
  for (int y = 0; y <= n; ++y)
    for (int x = 0; x <= n; ++x) out[(size_t)y * L + x] = top ? std::min(x + y, 2 * n - x - y) : std::abs(x - y);
  return RT_OK;
}

RT_API rt_status rt_sv_height_to_asm(const int32_t* h, int32_t n, int32_t* out) {
  clear_error();
  if (n < 1 || !h || !out) return fail(RT_ERR_INVALID_ARGUMENT, "six-vertex height_to_asm: bad arguments");
  if (!sv_valid_heights(h, n)) return fail(RT_ERR_INVALID_ARGUMENT, "six-vertex: not a height function (|dh| != 1)");
  const int L = n + 1;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      const int nw = h[(size_t)i * L + j], ne = h[(size_t)i * L + j + 1];
      const int sw = h[(size_t)(i + 1) * L + j], se = h[(size_t)(i + 1) * L + j + 1];
      out[(size_t)i * n + j] = (ne + sw - nw - se) / 2;
    }
  return RT_OK;
}

RT_API rt_status rt_sv_asm_to_height(const int32_t* a, int32_t n, int32_t* out) {
  clear_error();
  if (n < 1 || !a || !out) return fail(RT_ERR_INVALID_ARGUMENT, "six-vertex asm_to_height: bad arguments");
  const int L = n + 1;
  // h(y, x) = x + y - 2 * sum_{i < y, j < x} a(i, j)
  std::vector<int64_t> S((size_t)L * L, 0);
  for (int y = 1; y <= n; ++y)
    for (int x = 1; x <= n; ++x)
      S[(size_t)y * L + x] = a[(size_t)(y - 1) * n + x - 1] + S[(size_t)(y - 1) * L + x] + S[(size_t)y * L + x - 1] -
                             S[(size_t)(y - 1) * L + x - 1];
  for (int y = 0; y <= n; ++y)
    for (int x = 0; x <= n; ++x) out[(size_t)y * L + x] = (int32_t)(x + y - 2 * S[(size_t)y * L + x]);
  if (!sv_valid_heights(out, n)) return fail(RT_ERR_INVALID_ARGUMENT, "six-vertex: not an alternating sign matrix");
  for (int k = 0; k <= n; ++k)
    if (out[(size_t)n * L + k] != n - k || out[(size_t)k * L + n] != n - k)
      return fail(RT_ERR_INVALID_ARGUMENT, "six-vertex: not an alternating sign matrix (row or column sums)");
  return RT_OK;
}

RT_API rt_status rt_sv_walk(int32_t* h, int32_t n, int64_t sweeps, int64_t seed, const double* abc,
                            const rt_walk_opts* opts, rt_cftp_stats* stats) {
  clear_error();
  rt_walk_opts o;
  rt_walk_opts_default(&o);
  o.rng_mode = RT_RNG_FAST;
  if (opts) o = *opts;
  if (!h || sweeps < 0) return fail(RT_ERR_INVALID_ARGUMENT, "six-vertex walk: NULL heights or negative sweeps");
  if (o.rng_mode != RT_RNG_FAST)
    return fail(RT_ERR_INVALID_ARGUMENT, "six-vertex walk: only the fast (Philox) random mode exists for this model");
  if (o.fast_stream >= 65536u) return fail(RT_ERR_INVALID_ARGUMENT, "fast_stream must be < 65536");
  double a, b, c;
  if (rt_status st = sv_check_common(n, abc, &a, &b, &c)) return st;
  if (!sv_valid_heights(h, n)) return fail(RT_ERR_INVALID_ARGUMENT, "six-vertex: not a height function (|dh| != 1)");
  if (rt_status st = sv_check_device()) return st;
  const SvGeom G = sv_geom(n);
  const std::vector<uint32_t> T = sv_thresholds_host(a, b, c);
  cudaStream_t st = (cudaStream_t)o.cuda_stream;
  SvDevice dev;
  if (cudaMalloc(&dev.chains, G.chain_words * sizeof(uint32_t)) != cudaSuccess) {
    cudaGetLastError();
    return fail(RT_ERR_OUT_OF_MEMORY, "six-vertex walk: device allocation failed");
  }
  std::vector<uint32_t> bits(G.chain_words);
  sv_pack(h, G, bits.data());
  cudaMemcpyAsync(dev.chains, bits.data(), bits.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, st);
  const int64_t launches = sv_run(dev.chains, 1, G, T, (uint64_t)seed, o.fast_stream, 0, 4 * sweeps, st, o.engine);
  if (launches < 0) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return fail(RT_ERR_INVALID_ARGUMENT, "six-vertex walk: no thread-block cluster holds this size (engine 2)");
  }
  cudaEventRecord(e1, st);
  cudaMemcpyAsync(bits.data(), dev.chains, bits.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
  const cudaError_t err = cudaStreamSynchronize(st);
  float ms = 0.f;
  if (err == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (err != cudaSuccess) return fail(RT_ERR_CUDA, std::string("six-vertex walk: ") + cudaGetErrorString(err));
  std::vector<int32_t> start(h, h + (size_t)(n + 1) * (n + 1));
  sv_unpack(bits.data(), G, start.data(), h);
  if (stats) {
    std::memset(stats, 0, sizeof *stats);
    stats->attempts = 1;
    stats->total_steps = 4 * sweeps;
    stats->final_steps = 4 * sweeps;
    stats->flip_attempts = sv_interior_points(n) * sweeps;
    stats->seconds = ms * 1e-3;
  }
  return RT_OK;
}

RT_API rt_status rt_sv_cftp(const int32_t* hmax, const int32_t* hmin, int32_t n, int64_t seed, int64_t first_sweeps,
                            int32_t max_attempts, const double* abc, const rt_walk_opts* opts, int32_t* out,
                            rt_cftp_stats* stats) {
  clear_error();
  rt_walk_opts o;
  rt_walk_opts_default(&o);
  o.rng_mode = RT_RNG_FAST;
  if (opts) o = *opts;
  if (!hmax || !hmin || !out || first_sweeps < 1 || max_attempts < 1)
    return fail(RT_ERR_INVALID_ARGUMENT, "six-vertex cftp: bad arguments");
  if (o.rng_mode != RT_RNG_FAST)
    return fail(RT_ERR_INVALID_ARGUMENT, "six-vertex cftp: only the fast (Philox) random mode exists for this model");
  if (o.fast_stream >= 65536u) return fail(RT_ERR_INVALID_ARGUMENT, "fast_stream must be < 65536");
  double a, b, c;
  if (rt_status st = sv_check_common(n, abc, &a, &b, &c)) return st;
  if (c < a || c < b)
    return fail(RT_ERR_INVALID_ARGUMENT, "six-vertex cftp: the heat-bath coupling is monotone only for c >= max(a, b)");
  if (!sv_valid_heights(hmax, n) || !sv_valid_heights(hmin, n))
    return fail(RT_ERR_INVALID_ARGUMENT, "six-vertex: not a height function (|dh| != 1)");
  const int L = n + 1;
  for (int y = 0; y <= n; ++y)
    for (int x = 0; x <= n; ++x) {
      const bool edge = y == 0 || x == 0 || y == n || x == n;
      const int32_t u = hmax[(size_t)y * L + x], v = hmin[(size_t)y * L + x];
      if ((edge && u != v) || u < v)
        return fail(RT_ERR_INVALID_ARGUMENT, "six-vertex cftp: hmax must dominate hmin with the same boundary");
    }
  if (rt_status st = sv_check_device()) return st;
  const SvGeom G = sv_geom(n);
  const std::vector<uint32_t> T = sv_thresholds_host(a, b, c);
  cudaStream_t st = (cudaStream_t)o.cuda_stream;
  SvDevice dev;
  if (cudaMalloc(&dev.chains, 2 * G.chain_words * sizeof(uint32_t)) != cudaSuccess ||
      cudaMalloc(&dev.flag, sizeof(uint32_t)) != cudaSuccess) {
    cudaGetLastError();
    return fail(RT_ERR_OUT_OF_MEMORY, "six-vertex cftp: device allocation failed");
  }
  std::vector<uint32_t> start(2 * G.chain_words);
  sv_pack(hmax, G, start.data());
  sv_pack(hmin, G, start.data() + G.chain_words);
  if (stats) std::memset(stats, 0, sizeof *stats);
  float total_ms = 0.f;
  int64_t Tsw = first_sweeps, total_sub = 0;
  for (int attempt = 1; attempt <= max_attempts; ++attempt, Tsw *= 2) {
    if (Tsw > ((int64_t)1 << 44)) break;
    cudaMemcpyAsync(dev.chains, start.data(), start.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(dev.flag, 0, sizeof(uint32_t), st);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    if (sv_run(dev.chains, 2, G, T, (uint64_t)seed, o.fast_stream, -4 * Tsw, 4 * Tsw, st, o.engine) < 0) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return fail(RT_ERR_INVALID_ARGUMENT, "six-vertex cftp: no thread-block cluster holds this size (engine 2)");
    }
    cudaEventRecord(e1, st);
    k_sv_diff<<<64, 256, 0, st>>>(dev.chains, dev.chains + G.chain_words, G.chain_words, dev.flag);
    uint32_t differ = 1;
    cudaMemcpyAsync(&differ, dev.flag, sizeof differ, cudaMemcpyDeviceToHost, st);
    const cudaError_t err = cudaStreamSynchronize(st);
    float ms = 0.f;
    if (err == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (err != cudaSuccess) return fail(RT_ERR_CUDA, std::string("six-vertex cftp: ") + cudaGetErrorString(err));
    total_ms += ms;
    total_sub += 4 * Tsw;
    if (stats) {
      stats->attempts = attempt;
      stats->total_steps = total_sub;
      stats->flip_attempts += 2 * sv_interior_points(n) * Tsw;
      stats->seconds = total_ms * 1e-3;
    }
    if (!differ) {
      std::vector<uint32_t> bits(G.chain_words);
      cudaMemcpy(bits.data(), dev.chains, bits.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost);
      sv_unpack(bits.data(), G, hmax, out);
      if (stats) stats->final_steps = 4 * Tsw;
      return RT_OK;
    }
  }
  // not coalesced: out holds the top chain of the last attempt
  std::vector<uint32_t> bits(G.chain_words);
  if (cudaMemcpy(bits.data(), dev.chains, bits.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost) == cudaSuccess)
    sv_unpack(bits.data(), G, hmax, out);
  return fail(RT_ERR_NOT_COALESCED, "six-vertex cftp: chains did not coalesce within max_attempts");
}

}  // extern "C"
