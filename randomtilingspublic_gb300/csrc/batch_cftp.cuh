// Device pieces shared by the batched CFTP kernels: the one-CTA-per-instance kernel
// (batch_cftp.cu) and the thread-block-cluster kernel for instances that do not fit one CTA
// (batch_cluster.cu).  The half-sweep is split into its two phases over a range of rows, so
// that a CTA holding a strip of rows of an instance runs exactly the per-site operations the
// one-CTA kernel runs on the whole instance: the same draws, the same rule, the same rebuild.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "rng.cuh"
#include "rt_internal.h"

namespace rt {

// One instance as the kernels see it.  Colour arrays are N rows x P bytes (P a multiple of
// 16), ncol of them per chain (2 dominoes, 3 lozenges); tmax / tmin / out are ncol
// consecutive arrays at these byte offsets of the launch's tiling buffer.
struct DevInstance {
  int32_t model, N, P, cols;  // cols: last site column + 1 of the colour arrays (N/2 - 1 or N/3)
  uint64_t seed;
  uint32_t stream;
  int32_t max_attempts;
  int64_t first_sweeps;
  int64_t off_max, off_min, off_out;  // byte offsets into the tiling buffer
  uint32_t lo_up[4], w_up[4], lo_dn[4], w_dn[4];  // domino rule intervals (fast scale)
  int32_t attempts;                                // outputs
  int64_t final_half_sweeps;
};

// Rows whose sites flip: dominoes [1, N-1) (the update kernels start at row 1,
// dominokernel.cl:6-7), lozenges every row (the rotation runs on all rows,
// lozengekernel.cl:12-13; the rebuild on rows [1, N-1), lozengekernel.cl:43).
__host__ __device__ inline int flip_row_lo(const DevInstance& in) { return in.model == 0 ? 1 : 0; }
__host__ __device__ inline int flip_row_hi(const DevInstance& in) { return in.model == 0 ? in.N - 1 : in.N; }

template <int kThreads>
__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = threadIdx.x < kThreads / 32 ? red[threadIdx.x] : 0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) red[0] = v;
  }
  __syncthreads();
  const uint32_t r = red[0];
  __syncthreads();
  return r;
}

__device__ __forceinline__ uint8_t dm_flip_b(uint32_t e, uint32_t u, uint32_t lo_up, uint32_t w_up, uint32_t lo_dn,
                                             uint32_t w_dn) {
  if (e == 3u) return (u - lo_up) < w_up ? 12 : 3;
  if (e == 12u) return (u - lo_dn) < w_dn ? 3 : 12;
  return (uint8_t)e;
}

// A CTA's view of the chains it holds: chain c, colour k starts at sm + (c * ncol + k) *
// plane, and its first stored row is row s0 of the instance (P bytes a row).
struct RowView {
  uint8_t* sm;
  size_t plane;
  int s0;
  __device__ __forceinline__ uint8_t* row(int c, int ncol, int k, int i, int P) const {
    return sm + (size_t)(c * ncol + k) * plane + (size_t)(i - s0) * P;
  }
};

// Domino flips of colour t on rows [f0, f1) of both chains with the fast draws of half-sweep
// h: every thread takes (row, column quad) units, one 32-bit word per chain.  A word of row
// send_up (send_dn) is also stored at the same place of the CTA above (below) - the `up` /
// `dn` views - which holds that row as its halo; -1: no such row.
template <int kThreads>
__device__ void dm_flip_rows(const RowView& v, const DevInstance& in, int t, int64_t h, int f0, int f1,
                             const RowView* up, int send_up, const RowView* dn, int send_dn) {
  const int P = in.P, cols = in.cols - 1;  // sites m in [1, cols]
  const int quads = cols / 4 + 1;
  for (int k = threadIdx.x; k < (f1 - f0) * quads; k += kThreads) {
    const int i = f0 + k / quads, q = k - (i - f0) * quads;
    const int c = (i & 1) | (t << 1);
    const uint32_t lo_up = in.lo_up[c], w_up = in.w_up[c], lo_dn = in.lo_dn[c], w_dn = in.w_dn[c];
    const uint4 r = fast_quad(in.seed, in.stream, h, (uint32_t)i, (uint32_t)q);
    const uint32_t rr[4] = {r.x, r.y, r.z, r.w};
    for (int ch = 0; ch < 2; ++ch) {
      uint32_t* word = reinterpret_cast<uint32_t*>(v.row(ch, 2, t, i, P)) + q;
      const uint32_t e4 = *word;
      uint32_t n4 = e4;
#pragma unroll
      for (int k4 = 0; k4 < 4; ++k4) {
        const int m = 4 * q + k4;
        if (m < 1 || m > cols) continue;
        const uint32_t e = (e4 >> (8 * k4)) & 0xffu;
        n4 ^= (e ^ dm_flip_b(e, rr[k4], lo_up, w_up, lo_dn, w_dn)) << (8 * k4);
      }
      if (n4 != e4) *word = n4;
      if (i == send_up) reinterpret_cast<uint32_t*>(up->row(ch, 2, t, i, P))[q] = n4;
      if (i == send_dn) reinterpret_cast<uint32_t*>(dn->row(ch, 2, t, i, P))[q] = n4;
    }
  }
}

// Rebuild of the passive colour 1 - t on rows [b0, b1) of both chains from the active rows
// i - 1, i, i + 1 (dominokernel.cl:22-31 semantics): four passive sites per word from whole
// words of the active rows (funnel shifts for the one-column offsets), keeping the columns
// outside [1, cols].
template <int kThreads>
__device__ void dm_rebuild_rows(const RowView& v, const DevInstance& in, int t, int b0, int b1) {
  const int P = in.P, cols = in.cols - 1;
  const int words = P / 4;
  for (int k = threadIdx.x; k < 2 * (b1 - b0) * words; k += kThreads) {
    const int rc = k / words, w = k - rc * words;
    const int ch = rc & 1, i = b0 + (rc >> 1);
    uint32_t keep = 0;  // columns outside [1, cols] keep their value
#pragma unroll
    for (int k4 = 0; k4 < 4; ++k4) {
      const int m = 4 * w + k4;
      if (m < 1 || m > cols) keep |= 0xffu << (8 * k4);
    }
    if (keep == 0xffffffffu) continue;
    const uint32_t* A = reinterpret_cast<const uint32_t*>(v.row(ch, 2, t, i, P));
    uint32_t* Pw = reinterpret_cast<uint32_t*>(v.row(ch, 2, 1 - t, i, P)) + w;
    const uint32_t cur = A[w], up = A[w - words], dn = A[w + words];
    uint32_t left, right;  // active neighbours at columns m, m+1 when i + t is odd, else m-1, m
    if ((i + t) & 1) {
      left = cur;
      right = __funnelshift_r(cur, w + 1 < words ? A[w + 1] : 0u, 8);
    } else {
      left = __funnelshift_l(w > 0 ? A[w - 1] : 0u, cur, 8);
      right = cur;
    }
    const uint32_t val = ((up >> 1) & 0x01010101u) | ((dn & 0x01010101u) << 1) | ((left & 0x08080808u) >> 1) |
                         ((right & 0x04040404u) << 1);
    *Pw = (val & ~keep) | (*Pw & keep);
  }
}

// Lozenge rotation 25 <-> 38 of colour r on rows [f0, f1) of both chains with the fast draws
// of step h (lozengekernel.cl:107-125 semantics); halo rows sent as in dm_flip_rows.
template <int kThreads>
__device__ void lz_rotate_rows(const RowView& v, const DevInstance& in, int r, int64_t h, uint32_t c4, uint32_t c8,
                               int f0, int f1, const RowView* up, int send_up, const RowView* dn, int send_dn) {
  const int P = in.P, M = in.cols;
  const int quads = (M + 3) / 4;
  for (int k = threadIdx.x; k < (f1 - f0) * quads; k += kThreads) {
    const int i = f0 + k / quads, q = k - (i - f0) * quads;
    const uint4 d = fast_quad(in.seed, in.stream, h, (uint32_t)i, (uint32_t)q);
    const uint32_t uu[4] = {d.x, d.y, d.z, d.w};
    for (int ch = 0; ch < 2; ++ch) {
      uint32_t* word = reinterpret_cast<uint32_t*>(v.row(ch, 3, r, i, P)) + q;
      const uint32_t e4 = *word;
      uint32_t n4 = e4;
#pragma unroll
      for (int k4 = 0; k4 < 4; ++k4) {
        if (4 * q + k4 >= M) break;
        const uint32_t e = (e4 >> (8 * k4)) & 0xffu;
        uint32_t n = e;
        if (e == 25u && uu[k4] < c4) n = 38;
        else if (e == 38u && uu[k4] >= c4 && uu[k4] < c8) n = 25;
        n4 ^= (e ^ n) << (8 * k4);
      }
      if (n4 != e4) *word = n4;
      if (i == send_up) reinterpret_cast<uint32_t*>(up->row(ch, 3, r, i, P))[q] = n4;
      if (i == send_dn) reinterpret_cast<uint32_t*>(dn->row(ch, 3, r, i, P))[q] = n4;
    }
  }
}

// Rebuild of the two other lozenge colours on rows [b0, b1) (b0 >= 1, b1 <= N - 1) of both
// chains from the rotated colour r's rows i - 1, i, i + 1: (chain, row, word of four
// vertices) units, keeping the columns outside [1, M-2].
template <int kThreads>
__device__ void lz_rebuild_rows(const RowView& v, const DevInstance& in, int r, int b0, int b1) {
  const int P = in.P, M = in.cols;
  const int words = P / 4;
  for (int k = threadIdx.x; k < 2 * (b1 - b0) * words; k += kThreads) {
    const int rc = k / words, w = k - rc * words;
    const int ch = rc & 1, i = b0 + (rc >> 1);
    uint32_t keep = 0;
#pragma unroll
    for (int k4 = 0; k4 < 4; ++k4) {
      const int j = 4 * w + k4;
      if (j < 1 || j > M - 2) keep |= 0xffu << (8 * k4);
    }
    if (keep == 0xffffffffu) continue;
    const int im = i % 3;
    const bool p2 = im == (2 * r + 1) % 3, p4 = im == (2 * r + 2) % 3, p8 = im == (2 * r) % 3;
    const uint32_t* up = reinterpret_cast<const uint32_t*>(v.row(ch, 3, r, i - 1, P));
    const uint32_t* mid = up + words;
    const uint32_t* dn = mid + words;
    uint32_t* T2 = reinterpret_cast<uint32_t*>(v.row(ch, 3, (r + 1) % 3, i, P)) + w;
    uint32_t* T3 = reinterpret_cast<uint32_t*>(v.row(ch, 3, (r + 2) % 3, i, P)) + w;
    const uint32_t u0 = up[w], m0 = mid[w], d0 = dn[w];
    const uint32_t u_r = __funnelshift_r(u0, w + 1 < words ? up[w + 1] : 0u, 8);
    const uint32_t m_r = __funnelshift_r(m0, w + 1 < words ? mid[w + 1] : 0u, 8);
    const uint32_t m_l = __funnelshift_l(w > 0 ? mid[w - 1] : 0u, m0, 8);
    const uint32_t d_l = __funnelshift_l(w > 0 ? dn[w - 1] : 0u, d0, 8);
    const uint32_t a2 = p2 ? u_r : u0, a4 = p4 ? m_l : m0, a8 = p8 ? m_r : m0, a16 = p2 ? d_l : d0;
    const uint32_t b2 = ((a2 & 0x10101010u) >> 3) | ((a4 & 0x08080808u) >> 1) | ((d0 & 0x01010101u) << 5);
    const uint32_t b3 = ((u0 & 0x20202020u) >> 5) | ((a8 & 0x04040404u) << 1) | ((a16 & 0x02020202u) << 3);
    const uint32_t t2 = *T2, t3 = *T3;
    *T2 = (((t2 & ~0x26262626u) | b2) & ~keep) | (t2 & keep);
    *T3 = (((t3 & ~0x19191919u) | b3) & ~keep) | (t3 & keep);
  }
}

// Thread-block-cluster instances (batch_cluster.cu): instances too large for one CTA's shared
// memory, each held by a cluster of C CTAs (C <= 16), CTA k holding a strip of rows with one
// halo row above and below.
struct ClusterGroup {
  int C = 0;                // CTAs per cluster
  size_t smem = 0;          // dynamic shared memory per CTA
  int clusters = 0;         // clusters launched
  std::vector<int> members; // indices into the launch's cluster instance list
};
// Rows each CTA of a C-CTA cluster flips, and the shared memory a CTA needs: both chains,
// every colour, its rows plus the halo row on each side.
__host__ __device__ inline int cluster_rows_per_cta(const DevInstance& d, int C) {
  return (flip_row_hi(d) - flip_row_lo(d) + C - 1) / C;
}
__host__ __device__ inline size_t cluster_plane_bytes(const DevInstance& d, int C) {
  return (size_t)(cluster_rows_per_cta(d, C) + 2) * d.P;
}
inline size_t cluster_smem_bytes(const DevInstance& d, int C) {
  return (size_t)2 * (d.model == 0 ? 2 : 3) * cluster_plane_bytes(d, C);
}
// Smallest cluster size (2..16) whose CTAs hold the instance within smem_limit; 0: none.
int cluster_size_for(const DevInstance& d, size_t smem_limit);
// Launches one group's kernel on stream s: d_inst points at the group's instances (count of
// them, contiguous), d_queue at a zeroed counter.  Returns the launch status.
rt_status launch_cluster_group(const ClusterGroup& g, DevInstance* d_inst, int count, uint8_t* d_tilings,
                               unsigned* d_queue, uint32_t lz_c4, uint32_t lz_c8, cudaStream_t s);
// Clusters of C CTAs with smem bytes each that can be resident at once (0 when none).
int cluster_capacity(int C, size_t smem);

}  // namespace rt
