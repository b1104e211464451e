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

// Bit 7 of each byte of x set where that byte equals the matching byte of 0xbbbbbbbb; every
// byte of x and b below 0x80, so that the additions carry into no other byte.
__device__ __forceinline__ uint32_t bytes_equal(uint32_t x, uint32_t bbbb) {
  return ~((x ^ bbbb) + 0x7f7f7f7fu) & 0x80808080u;
}
__device__ __forceinline__ uint32_t byte_bit(bool p, int k) { return p ? 0x80u << (8 * k) : 0u; }

// Walks the (row, column unit) pairs of rows [r0, r1), `units` units a row, the thread's
// first pair then every kThreads-th, with the division done once.
template <int kThreads>
struct UnitWalk {
  int i, q, di, dq, units, r1;
  __device__ __forceinline__ UnitWalk(int r0, int r1_, int units_) : units(units_), r1(r1_) {
    const int t = (int)threadIdx.x;
    i = r0 + t / units;
    q = t - (t / units) * units;
    di = kThreads / units;
    dq = kThreads - di * units;
  }
  __device__ __forceinline__ bool more() const { return i < r1; }
  __device__ __forceinline__ void next() {
    i += di;
    q += dq;
    if (q >= units) {
      q -= units;
      ++i;
    }
  }
};

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
// h: every thread takes (row, column quad) units, one 32-bit word of four sites per chain.  A
// site m in [1, cols] holding 3 becomes 12 when (u - lo_up) < w_up, one holding 12 becomes 3
// when (u - lo_dn) < w_dn, with the intervals of its colour class (i & 1) | (t << 1)
// (dominokernelCFTPtwoperiodic.cl semantics); both are an XOR with 15, taken for the four
// bytes of a word at once.  A word of row send_up (send_dn) is also stored at the same place
// of the CTA above (below) - the `up` / `dn` views - which holds that row as its halo; -1:
// no such row.
template <int kThreads>
__device__ void dm_flip_rows(const RowView& v, const DevInstance& in, int t, int64_t h, int f0, int f1,
                             const RowView* up, int send_up, const RowView* dn, int send_dn) {
  const int P = in.P, cols = in.cols - 1;  // sites m in [1, cols]
  const int quads = cols / 4 + 1;
  const int c0 = t << 1;
  const uint32_t lu[2] = {in.lo_up[c0], in.lo_up[c0 | 1]}, wu[2] = {in.w_up[c0], in.w_up[c0 | 1]};
  const uint32_t ld[2] = {in.lo_dn[c0], in.lo_dn[c0 | 1]}, wd[2] = {in.w_dn[c0], in.w_dn[c0 | 1]};
  for (UnitWalk<kThreads> u(f0, f1, quads); u.more(); u.next()) {
    const int i = u.i, q = u.q, odd = i & 1;
    const uint32_t lo_up = odd ? lu[1] : lu[0], w_up = odd ? wu[1] : wu[0];
    const uint32_t lo_dn = odd ? ld[1] : ld[0], w_dn = odd ? wd[1] : wd[0];
    const uint4 r = fast_quad(in.seed, in.stream, h, (uint32_t)i, (uint32_t)q);
    uint32_t valid = 0x80808080u;  // bytes of sites m = 4q + k in [1, cols]
    if (q == 0) valid = 0x80808000u;
    const int over = 4 * q + 3 - cols;
    if (over > 0) valid &= 0x80808080u >> (8 * over);
    const uint32_t acc_up = (byte_bit(r.x - lo_up < w_up, 0) | byte_bit(r.y - lo_up < w_up, 1) |
                             byte_bit(r.z - lo_up < w_up, 2) | byte_bit(r.w - lo_up < w_up, 3)) & valid;
    const uint32_t acc_dn = (byte_bit(r.x - lo_dn < w_dn, 0) | byte_bit(r.y - lo_dn < w_dn, 1) |
                             byte_bit(r.z - lo_dn < w_dn, 2) | byte_bit(r.w - lo_dn < w_dn, 3)) & valid;
#pragma unroll
    for (int ch = 0; ch < 2; ++ch) {
      uint32_t* word = reinterpret_cast<uint32_t*>(v.row(ch, 2, t, i, P)) + q;
      const uint32_t e4 = *word;
      const uint32_t f = (bytes_equal(e4, 0x03030303u) & acc_up) | (bytes_equal(e4, 0x0c0c0c0cu) & acc_dn);
      const uint32_t n4 = e4 ^ ((f >> 7) * 15u);
      if (n4 != e4) *word = n4;
      if (i == send_up) reinterpret_cast<uint32_t*>(up->row(ch, 2, t, i, P))[q] = n4;
      if (i == send_dn) reinterpret_cast<uint32_t*>(dn->row(ch, 2, t, i, P))[q] = n4;
    }
  }
}

// Bytes of word w (columns 4w .. 4w + 3) outside [lo, hi]: 0xff in each.
__device__ __forceinline__ uint32_t keep_bytes(int w, int lo, int hi) {
  uint32_t keep = 0;
  const int below = lo - 4 * w;  // bytes under column lo
  if (below >= 4) return 0xffffffffu;
  if (below > 0) keep = 0xffffffffu >> (8 * (4 - below));
  const int over = 4 * w + 3 - hi;  // bytes above column hi
  if (over >= 4) return 0xffffffffu;
  if (over > 0) keep |= 0xffffffffu << (8 * (4 - over));
  return keep;
}

// Rebuild of the passive colour 1 - t on rows [b0, b1) of both chains from the active rows
// i - 1, i, i + 1 (dominokernel.cl:22-31 semantics): four passive sites per word from whole
// words of the active rows (funnel shifts for the one-column offsets), keeping the columns
// outside [1, cols].  Units are (row, word) pairs, both chains in each.
template <int kThreads>
__device__ void dm_rebuild_rows(const RowView& v, const DevInstance& in, int t, int b0, int b1) {
  const int P = in.P, cols = in.cols - 1;
  const int words = P / 4;
  for (UnitWalk<kThreads> u(b0, b1, words); u.more(); u.next()) {
    const int i = u.i, w = u.q;
    const uint32_t keep = keep_bytes(w, 1, cols);
    if (keep == 0xffffffffu) continue;
#pragma unroll
    for (int ch = 0; ch < 2; ++ch) {
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
}

// Lozenge rotation 25 <-> 38 of colour r on rows [f0, f1) of both chains with the fast draws
// of step h (lozengekernel.cl:107-125 semantics): a vertex holding 25 becomes 38 when
// u < c4, one holding 38 becomes 25 when c4 <= u < c8; both are an XOR with 63, taken for
// the four vertices of a word at once.  Halo rows sent as in dm_flip_rows.
template <int kThreads>
__device__ void lz_rotate_rows(const RowView& v, const DevInstance& in, int r, int64_t h, uint32_t c4, uint32_t c8,
                               int f0, int f1, const RowView* up, int send_up, const RowView* dn, int send_dn) {
  const int P = in.P, M = in.cols;
  const int quads = (M + 3) / 4;
  const uint32_t span = c8 - c4;
  for (UnitWalk<kThreads> u(f0, f1, quads); u.more(); u.next()) {
    const int i = u.i, q = u.q;
    const uint4 d = fast_quad(in.seed, in.stream, h, (uint32_t)i, (uint32_t)q);
    uint32_t valid = 0x80808080u;  // vertices j = 4q + k below M
    const int over = 4 * q + 4 - M;
    if (over > 0) valid = 0x80808080u >> (8 * over);
    const uint32_t acc25 = (byte_bit(d.x < c4, 0) | byte_bit(d.y < c4, 1) | byte_bit(d.z < c4, 2) |
                            byte_bit(d.w < c4, 3)) & valid;
    const uint32_t acc38 = (byte_bit(d.x - c4 < span, 0) | byte_bit(d.y - c4 < span, 1) |
                            byte_bit(d.z - c4 < span, 2) | byte_bit(d.w - c4 < span, 3)) & valid;
#pragma unroll
    for (int ch = 0; ch < 2; ++ch) {
      uint32_t* word = reinterpret_cast<uint32_t*>(v.row(ch, 3, r, i, P)) + q;
      const uint32_t e4 = *word;
      const uint32_t f = (bytes_equal(e4, 0x19191919u) & acc25) | (bytes_equal(e4, 0x26262626u) & acc38);
      const uint32_t n4 = e4 ^ ((f >> 7) * 63u);
      if (n4 != e4) *word = n4;
      if (i == send_up) reinterpret_cast<uint32_t*>(up->row(ch, 3, r, i, P))[q] = n4;
      if (i == send_dn) reinterpret_cast<uint32_t*>(dn->row(ch, 3, r, i, P))[q] = n4;
    }
  }
}

// Rebuild of the two other lozenge colours on rows [b0, b1) (b0 >= 1, b1 <= N - 1) of both
// chains from the rotated colour r's rows i - 1, i, i + 1: (row, word of four vertices)
// units, both chains in each, keeping the columns outside [1, M-2].
template <int kThreads>
__device__ void lz_rebuild_rows(const RowView& v, const DevInstance& in, int r, int b0, int b1) {
  const int P = in.P, M = in.cols;
  const int words = P / 4;
  for (UnitWalk<kThreads> u(b0, b1, words); u.more(); u.next()) {
    const int i = u.i, w = u.q;
    const uint32_t keep = keep_bytes(w, 1, M - 2);
    if (keep == 0xffffffffu) continue;
    const int im = i % 3;
    const bool p2 = im == (2 * r + 1) % 3, p4 = im == (2 * r + 2) % 3, p8 = im == (2 * r) % 3;
#pragma unroll
    for (int ch = 0; ch < 2; ++ch) {
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
