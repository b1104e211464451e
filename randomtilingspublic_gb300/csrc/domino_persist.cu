// Resident persistent engine of the domino sweep.
//
// One cooperative launch runs many half-sweeps.  CTA b owns a band of colour-array rows
// [r0, r1) and keeps, in shared memory, rows r0-1 .. r1 of both colours of every swept chain
// over a 4-byte-aligned column window that contains every site of the band that can change
// (see dm_plan_partition).  Its flip candidates ("units": one site per unit in TinyMT mode,
// a column quad in fast mode) are dealt round-robin to its threads, whose TinyMT generator
// states stay in registers for the whole launch.  Each half-sweep:
//   1. flip: every unit draws and tests its site of the rotated colour t in every chain,
//      the units of the band's first and last rows first;
//   2. publish (two communication warps, while the workers flip the interior): the band's
//      first and last rows of colour t go to a double-buffered exchange slot in global
//      memory as 64-bit words that carry their half-sweep tag beside the data;
//   3. wait: the same warps poll the neighbours' rows until every word carries the tag
//      (bounded; on expiry an error code is set and every CTA leaves its loop) and copy
//      them into the halo rows;
//   4. rebuild: the passive colour of the band's first and last rows (the interior is kept
//      current by XOR updates from each flip, or rebuilt in full for general inputs).
// Only generators of flip candidates are advanced: the others never influence a flip, so
// the tilings are identical to the per-half-sweep kernels (and to the reference).  The
// rebuild is restricted to the window, which is exact when the loaded tilings are
// consistent (both endpoints of every edge agree); other inputs use the per-half-sweep path.
#include <cooperative_groups.h>
#include <cuda/atomic>
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "domino_persist.h"
#include "domino_sweep.h"
#include "rng.cuh"

namespace rt {

namespace {

constexpr int kThreads = kPersistThreads;
constexpr int kCommWarps = 2;  // warp 0 trades rows with the band above, warp 1 with the band below
constexpr int kWorkers = kThreads - 32 * kCommWarps;
constexpr uint32_t kNoUnit = 0xffffffffu;

// Byte-parallel flip of NCH coupled chains of one site (one byte per chain in x, bytes
// <= 15): a byte equal to 3 becomes 12 when up is all-ones, a byte equal to 12 becomes 3
// when dn is, both by XOR with 15.  Byte b equals v exactly when bit 4 of (b ^ v) + 15 is
// clear (the sum stays below 32, so no carry crosses a byte).
__device__ __forceinline__ uint32_t flip_bytes(uint32_t x, uint32_t up, uint32_t dn, uint32_t bytes_mask) {
  const uint32_t ne3 = (x ^ 0x03030303u) + 0x0f0f0f0fu, ne12 = (x ^ 0x0c0c0c0cu) + 0x0f0f0f0fu;
  const uint32_t hit = ((~ne3 & up) | (~ne12 & dn)) & 0x10101010u & bytes_mask;
  return x ^ ((hit >> 4) * 15u);
}

__device__ __forceinline__ void workers_sync() { asm volatile("bar.sync 1, %0;" ::"r"(kWorkers) : "memory"); }

// Shared memory: two colour planes, each R rows (band rows plus one halo row above and
// below) of Wb = W * NCH bytes; cell x of a row holds its NCH chains in consecutive bytes.
template <int NCH>
struct Planes {
  uint8_t* p;
  int R, Wb;
  __device__ uint8_t* row(int t, int ri) const { return p + ((size_t)t * R + ri) * Wb; }
};

// Rebuilds the passive colour 1-t of band row ri (colour-array row i) from the active
// colour t: bit 1 from the site above (its bit 2), bit 2 from below (its bit 1), bit 4 from
// the left active neighbour (its 8), bit 8 from the right one (its 4); left/right are
// columns m-1/m or m/m+1 by the parity of i+t.  Word w holds 4/NCH cells x NCH chains.
template <int NCH>
__device__ __forceinline__ void rebuild_word(const Planes<NCH>& pl, int t, int ri, int i, int w, int words, int wlo,
                                             int cols) {
  const uint32_t* A0 = reinterpret_cast<const uint32_t*>(pl.row(t, ri - 1));
  const uint32_t* A1 = reinterpret_cast<const uint32_t*>(pl.row(t, ri));
  const uint32_t* A2 = reinterpret_cast<const uint32_t*>(pl.row(t, ri + 1));
  uint32_t* Pw = reinterpret_cast<uint32_t*>(pl.row(1 - t, ri));
  const uint32_t cur = A1[w];
  uint32_t left, right;
  if ((i + t) & 1) {
    const uint32_t next = w + 1 < words ? A1[w + 1] : 0u;
    left = cur;
    right = __funnelshift_rc(cur, next, 8 * NCH);
  } else {
    const uint32_t prev = w > 0 ? A1[w - 1] : 0u;
    left = __funnelshift_lc(prev, cur, 8 * NCH);
    right = cur;
  }
  const uint32_t v = ((A0[w] >> 1) & 0x01010101u) | ((A2[w] & 0x01010101u) << 1) | ((left & 0x08080808u) >> 1) |
                     ((right & 0x04040404u) << 1);
  // Kept as they are: the window's first and last cell (they never change and lack a
  // neighbour here) and columns outside [1, cols], which the reference never rebuilds.
  constexpr int kCells = 4 / NCH;
  constexpr uint32_t kCellMask = NCH == 4 ? 0xffffffffu : ((1u << (8 * NCH)) - 1u);
  uint32_t keep = 0;
  const int c0 = wlo + kCells * w;
#pragma unroll
  for (int k = 0; k < kCells; ++k) {
    const int c = c0 + k;
    const bool edge = (w == 0 && k == 0) || (w == words - 1 && k == kCells - 1);
    if (edge || c < 1 || c > cols) keep |= kCellMask << (8 * NCH * k);
  }
  Pw[w] = (v & ~keep) | (Pw[w] & keep);
}

// XORs mask into the byte(s) of chain-interleaved cell offset off of a plane (atomically:
// two flips in one half-sweep can touch the same word).
__device__ __forceinline__ void xor_cell(uint8_t* plane, uint32_t off, uint32_t mask) {
  atomicXor(reinterpret_cast<unsigned*>(plane + (off & ~3u)), mask << (8 * (off & 3u)));
}

// Per-CTA constants kept in shared memory, so that neither role pins them in registers.
struct BandCtx {
  PersistArgs a;
  DmBand band;
  int R, W, Wb, words, vecs, rows, boundary_slots, abort;
  uint4 rule[4];
};

template <int NCH>
__device__ __forceinline__ Planes<NCH> planes_of(uint8_t* smem, const BandCtx& c, int K, bool need_where) {
  return Planes<NCH>{smem + (size_t)K * kThreads * 4 * (need_where ? 2 : 1), c.R, c.Wb};
}

// Exchange words: the 4 data bytes and a tag (the half-sweep count h + 1) in one 64-bit
// element, which is single-copy atomic, so a reader that sees the tag sees the data with it.
// Accesses are 16-byte vectors of two such elements (each element stays atomic on its own):
// every exchange row starts on a 32-byte boundary (P, wlo and whi are multiples of 16 cells).
__device__ __forceinline__ void st_tagged2(uint64_t* p, uint64_t a, uint64_t b) {
  asm volatile("st.relaxed.gpu.global.v2.u64 [%0], {%1, %2};" ::"l"(p), "l"(a), "l"(b) : "memory");
}
__device__ __forceinline__ void ld_tagged2(const uint64_t* p, uint64_t& a, uint64_t& b) {
  asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(a), "=l"(b) : "l"(p) : "memory");
}

// Exchange slot h & 1 of band b holds [2 rows][P x chains / 4 words] (see PersistArgs::xbuf):
// row 0 is the band's first row (read by the band above), row 1 its last (read below).
template <int NCH>
__device__ __forceinline__ uint64_t* exchange_row(const BandCtx& c, int h, int band, int which) {
  const size_t row_words = (size_t)c.a.P * NCH / 4;
  return reinterpret_cast<uint64_t*>(c.a.xbuf) + (((size_t)(h & 1) * c.a.nbands + band) * 2 + which) * row_words;
}

// Publishes the band's first and last rows of colour t for half-sweep h, one 16-byte
// vector (four data words) per thread of the whole CTA, right after the boundary flips.
template <int NCH>
__device__ __forceinline__ void publish_rows(const BandCtx& c, const Planes<NCH>& pl, int t, int h) {
  if ((int)blockIdx.x + 1 == c.a.silent_band_plus1) return;  // test hook: the neighbours' waits run out
  const int n4 = c.words >> 2;
  const uint64_t tag = (uint64_t)(uint32_t)(h + 1) << 32;
  for (int q = threadIdx.x; q < 2 * n4; q += blockDim.x) {
    const int which = q >= n4 ? 1 : 0, qq = q - which * n4;
    const uint4 d = reinterpret_cast<const uint4*>(pl.row(t, which == 0 ? 1 : c.R - 2))[qq];
    uint64_t* g = exchange_row<NCH>(c, h, blockIdx.x, which) + (size_t)c.band.wlo * NCH / 4 + 4 * qq;
    st_tagged2(g, tag | d.x, tag | d.y);
    st_tagged2(g + 2, tag | d.z, tag | d.w);
  }
}

// Unit c of the band -> colour-array row i and unit column u (site column in TinyMT mode,
// column quad in fast mode): the first row, the last row, then the rows between.
__device__ __forceinline__ void decode_unit(const BandCtx& c, int k, int& i, int& u) {
  const DmBand& b = c.band;
  if (k < b.nb_first) {
    i = b.r0;
  } else if (k < b.nb_boundary) {
    i = b.r1 - 1;
  } else {
    int lo = b.r0 + 1, hi = b.r1 - 2;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (c.a.row_prefix[mid] <= k) lo = mid;
      else hi = mid - 1;
    }
    i = lo;
  }
  u = c.a.row_lo[i] + (k - c.a.row_prefix[i]);
}

// Worker warps (1..31): flips, sparse passive updates or the interior rebuild, and the
// rebuild of the band's boundary rows.
template <int kMode, int K, bool kParams, int NCH, bool kSparse>
__device__ __noinline__ void worker_role(uint8_t* smem, BandCtx& c) {
  constexpr bool kNeedWhere = (kMode != RT_RNG_TINYMT) || kParams;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, wt = tid - 32 * kCommWarps;
  const int wwarp = warp - kCommWarps;  // worker warp index
  uint32_t* s_unit = reinterpret_cast<uint32_t*>(smem);
  uint32_t* s_where = s_unit + K * kThreads;
  const Planes<NCH> pl = planes_of<NCH>(smem, c, K, kNeedWhere);
  uint4 st[K];
#pragma unroll
  for (int s = 0; s < K; ++s) {
    s_unit[s * kThreads + tid] = kNoUnit;
    st[s] = make_uint4(0, 0, 0, 0);
    const int k = wt + s * kWorkers;
    if (k < c.band.units) {
      int i, u;
      decode_unit(c, k, i, u);
      const int ri = i - c.band.r0 + 1;
      const int m0 = kMode == RT_RNG_TINYMT ? u : 4 * u;
      uint32_t valid = 0;
      if (kMode != RT_RNG_TINYMT) {
#pragma unroll
        for (int k4 = 0; k4 < 4; ++k4)
          if (m0 + k4 >= 1 && m0 + k4 <= c.a.cols) valid |= 1u << k4;
      }
      s_unit[s * kThreads + tid] =
          (uint32_t)(ri * c.Wb + (m0 - c.band.wlo) * NCH) | (valid << 24) | ((uint32_t)(i & 1) << 31);
      if (kNeedWhere) s_where[s * kThreads + tid] = ((uint32_t)i << 16) | (uint32_t)u;
      if (kMode == RT_RNG_TINYMT) st[s] = c.a.tmt[(int64_t)(i - 1) * c.a.cols + (u - 1)];
    }
  }
  __syncthreads();  // init

  // Toggles, in the passive colour 1-t, the bit of the edge shared with the flipped site at
  // unit offset pk: bit 2 of the site above, bit 1 below, bit 8 of the passive site to its
  // left and bit 4 of the one to its right (columns m-1/m or m/m+1 by the parity of i+t);
  // ones has 0x01 in the byte of each chain that flipped.
  uint8_t* plane_act = pl.row(0, 0);  // set per half-sweep
  uint8_t* plane_pas = pl.row(1, 0);
  const uint4* rule_t = c.rule;
  auto passive_xor = [&](uint32_t pk, int t, uint32_t ones) {
    uint8_t* pp = plane_pas;
    const uint32_t off = pk & 0xffffffu, wb = (uint32_t)c.Wb;
    const int odd = (int)((pk >> 31) ^ (uint32_t)t) & 1;
    xor_cell(pp, off - wb, ones << 1);
    xor_cell(pp, off + wb, ones);
    xor_cell(pp, odd ? off - NCH : off, ones << 3);
    xor_cell(pp, odd ? off : off + NCH, ones << 2);
  };
  auto flip_cell = [&](uint8_t* q, uint32_t pk, int t, uint32_t r, const uint4& rl) {
    const uint32_t upm = (r - rl.x) < rl.y ? 0xffffffffu : 0u, dnm = (r - rl.z) < rl.w ? 0xffffffffu : 0u;
    uint32_t x, y;
    if (NCH == 1) {
      x = *q;
      y = flip_bytes(x, upm, dnm, 0xffu);
      if (y != x) *q = (uint8_t)y;
    } else if (NCH == 2) {
      uint16_t* q2 = reinterpret_cast<uint16_t*>(q);
      x = *q2;
      y = flip_bytes(x, upm, dnm, 0xffffu);
      if (y != x) *q2 = (uint16_t)y;
    } else {
      uint32_t* q4 = reinterpret_cast<uint32_t*>(q);
      x = *q4;
      y = flip_bytes(x, upm, dnm, 0xffffffffu);
      if (y != x) *q4 = y;
    }
    if (kSparse && y != x) passive_xor(pk, t, (x ^ y) & 0x01010101u);
  };
  auto flip_unit = [&](int s, int t, int h) {
    const uint32_t pk = s_unit[s * kThreads + tid];
    if (pk == kNoUnit) return;
    const uint4 rl = rule_t[pk >> 31];
    uint8_t* q = plane_act + (pk & 0xffffffu);
    if (kMode == RT_RNG_TINYMT) {
      uint32_t m1 = kTmtMat1, m2 = kTmtMat2, tm = kTmtTmat;
      if (kParams) {
        const uint32_t wh = s_where[s * kThreads + tid];
        const uint4 p = __ldg(&c.a.tmt_params[(int64_t)((wh >> 16) - 1) * c.a.cols + ((wh & 0xffffu) - 1)]);
        m1 = p.x; m2 = p.y; tm = p.z;
      }
      flip_cell(q, pk, t, tmt_next_u23(st[s], m1, m2, tm), rl);
    } else {
      const uint32_t wh = s_where[s * kThreads + tid];
      const uint4 r4 = fast_quad(c.a.fast_seed, c.a.fast_stream, c.a.h0 + h, wh >> 16, wh & 0xffffu);
      const uint32_t rr[4] = {r4.x, r4.y, r4.z, r4.w};
      const uint32_t valid = (pk >> 24) & 0xfu;
#pragma unroll
      for (int k4 = 0; k4 < 4; ++k4)
        if ((valid >> k4) & 1u) flip_cell(q + k4 * NCH, pk + k4 * NCH, t, rr[k4], rl);
    }
  };

  const int nsteps = (int)c.a.steps, par0 = (int)(c.a.h0 & 1);
  // The colour of half-sweep h + 1 is loaded during half-sweep h, off the critical path.
  int colour_next = (kMode == RT_RNG_TINYMT && nsteps > 0) ? c.a.colours[0] : 0;
  for (int h = 0; h < nsteps; ++h) {
    const int t = (kMode == RT_RNG_TINYMT) ? (colour_next ? 1 : 0) : (((par0 ^ h) & 1) ? 0 : 1);
    if (kMode == RT_RNG_TINYMT && h + 1 < nsteps) colour_next = c.a.colours[h + 1];
    const int bslots = c.boundary_slots;
    plane_act = pl.row(t, 0);
    plane_pas = pl.row(1 - t, 0);
    rule_t = c.rule + 2 * t;
#pragma unroll
    for (int s = 0; s < K; ++s)
      if (s < bslots) flip_unit(s, t, h);
    __syncthreads();  // #1: boundary rows final
    publish_rows<NCH>(c, pl, t, h);
#pragma unroll
    for (int s = 0; s < K; ++s)
      if (s >= bslots) flip_unit(s, t, h);
    if (!kSparse) {
      workers_sync();
      const int rows = c.rows, words = c.words;
      for (int r = wwarp + 1; r <= rows - 2; r += kWorkers / 32) {
        for (int w = lane; w < words; w += 32)
          rebuild_word<NCH>(pl, t, r + 1, c.band.r0 + r, w, words, c.band.wlo, c.a.cols);
      }
    }
    __syncthreads();  // #3: flips done, halo rows in place
    if (c.abort) break;
    {
      // All worker threads share the rebuild of the band's first and last rows.
      const int rows = c.rows, words = c.words, nrow = rows > 1 ? 2 : 1;
      for (int k = wt; k < nrow * words; k += kWorkers) {
        const int which = k >= words ? 1 : 0, w = k - which * words;
        const int rr = which == 0 ? 0 : rows - 1;
        rebuild_word<NCH>(pl, t, rr + 1, c.band.r0 + rr, w, words, c.band.wlo, c.a.cols);
      }
    }
    __syncthreads();  // #4
  }
  if (kMode == RT_RNG_TINYMT) {
#pragma unroll
    for (int s = 0; s < K; ++s) {
      if (s_unit[s * kThreads + tid] == kNoUnit) continue;
      int i, u;
      decode_unit(c, wt + s * kWorkers, i, u);
      c.a.tmt[(int64_t)(i - 1) * c.a.cols + (u - 1)] = st[s];
    }
  }
}

// Reads n tagged words (n even, src 16-byte aligned) into dst, polling until each carries
// tag want.  Each lane issues kBatch word pairs before it waits, so that one memory round
// trip covers a batch (576 words per warp), and every retry re-issues all pairs of the
// batch still pending at once: a row that arrives late then costs one more round trip, not
// one per word.  (Serial per-word polling turned a small delay of one band into a delay of
// several microseconds for its neighbour, which locked adjacent bands into alternating slow
// half-sweeps.)  Returns false when the wait gave up (bounded) or another CTA reported
// failure.
__device__ bool read_tagged(const uint64_t* src, uint32_t* dst, int n, uint32_t want, int* error, long max_spin) {
  constexpr int kBatch = 9;
  const int lane = threadIdx.x & 31, n2 = n >> 1;
  cuda::atomic_ref<int, cuda::thread_scope_device> err(*error);
  uint2* dst2 = reinterpret_cast<uint2*>(dst);
  for (int base = lane; base < n2; base += 32 * kBatch) {
    uint64_t v[2 * kBatch];
    uint32_t pending = 0;
#pragma unroll
    for (int j = 0; j < kBatch; ++j) {
      const int q = base + 32 * j;
      if (q < n2) {
        ld_tagged2(src + 2 * q, v[2 * j], v[2 * j + 1]);
        pending |= 1u << j;
      }
    }
    long it = 0;
    for (;;) {
#pragma unroll
      for (int j = 0; j < kBatch; ++j) {
        if (((pending >> j) & 1u) && (uint32_t)(v[2 * j] >> 32) == want && (uint32_t)(v[2 * j + 1] >> 32) == want) {
          dst2[base + 32 * j] = make_uint2((uint32_t)v[2 * j], (uint32_t)v[2 * j + 1]);
          pending &= ~(1u << j);
        }
      }
      if (pending == 0) break;
      if ((++it & 255) == 0 && err.load(cuda::memory_order_relaxed) != 0) return false;
      if (it > max_spin) {
        int zero = 0;
        err.compare_exchange_strong(zero, 1, cuda::memory_order_relaxed);
        return false;
      }
#pragma unroll
      for (int j = 0; j < kBatch; ++j)
        if ((pending >> j) & 1u) ld_tagged2(src + 2 * (base + 32 * j), v[2 * j], v[2 * j + 1]);
    }
  }
  return true;
}

// Warps 0 and 1: after their share of the publication of the band's boundary rows, each
// reads the facing boundary row of one neighbour (warp 0 the last row of the band above,
// warp 1 the first row of the band below) into its halo row while the workers flip the
// interior.
template <int kMode, int K, bool kParams, int NCH>
__device__ __noinline__ void comm_role(uint8_t* smem, BandCtx& c) {
  constexpr bool kNeedWhere = (kMode != RT_RNG_TINYMT) || kParams;
  const int lane = threadIdx.x & 31, which = threadIdx.x >> 5;  // 0: upper side, 1: lower side
  const int b = blockIdx.x, nb_band = which == 0 ? b - 1 : b + 1;
  const Planes<NCH> pl = planes_of<NCH>(smem, c, K, kNeedWhere);
  __syncthreads();  // init
  const int nsteps = (int)c.a.steps, par0 = (int)(c.a.h0 & 1);
  const bool has_nb = nb_band >= 0 && nb_band < c.a.nbands;
  int lo = 0, hi = 0;
  if (has_nb) {
    lo = max(c.band.wlo, c.a.bands[nb_band].wlo);
    hi = min(c.band.whi, c.a.bands[nb_band].whi);
  }
  const int n_in = hi > lo ? (hi - lo) * NCH / 4 : 0;
  int colour_next = (kMode == RT_RNG_TINYMT && nsteps > 0) ? c.a.colours[0] : 0;
  for (int h = 0; h < nsteps; ++h) {
    const int t = (kMode == RT_RNG_TINYMT) ? (colour_next ? 1 : 0) : (((par0 ^ h) & 1) ? 0 : 1);
    if (kMode == RT_RNG_TINYMT && h + 1 < nsteps) colour_next = c.a.colours[h + 1];
    __syncthreads();  // #1
    publish_rows<NCH>(c, pl, t, h);
    int ok = 1;
    if (has_nb) {
      const uint64_t* g = exchange_row<NCH>(c, h, nb_band, 1 - which) + (size_t)lo * NCH / 4;
      uint32_t* d = reinterpret_cast<uint32_t*>(pl.row(t, which == 0 ? 0 : c.R - 1) + (lo - c.band.wlo) * NCH);
      ok = read_tagged(g, d, n_in, (uint32_t)(h + 1), c.a.error, c.a.max_spin) ? 1 : 0;
    }
    ok = __all_sync(0xffffffffu, ok);
    if (!ok && lane == 0) c.abort = 1;
    __syncthreads();  // #3
    if (c.abort) break;
    __syncthreads();  // #4
  }
}

// kSparse: the passive colour is kept current by XOR updates from each flip (a flip toggles
// all four edge bits of its site, so each of its four passive neighbours toggles the one bit
// of the shared edge), and only the band's first and last rows are rebuilt in full, after
// the neighbours' rows arrive.  Exact for consistent tilings.  Without kSparse every window
// word is rebuilt each half-sweep, which reproduces the reference for any input.
template <int kMode, int K, bool kParams, int NCH, bool kSparse>
__global__ void __launch_bounds__(kThreads, 1) k_persist(PersistArgs a) {
  extern __shared__ __align__(16) uint8_t smem_raw[];
  __shared__ BandCtx c;
  constexpr bool kNeedWhere = (kMode != RT_RNG_TINYMT) || kParams;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    c.a = a;
    c.band = a.bands[blockIdx.x];
    c.R = c.band.r1 - c.band.r0 + 2;
    c.W = c.band.whi - c.band.wlo;
    c.Wb = c.W * NCH;
    c.words = c.Wb / 4;
    c.vecs = c.Wb / 16;
    c.rows = c.R - 2;
    c.boundary_slots = (c.band.nb_boundary + kWorkers - 1) / kWorkers;
    c.abort = 0;
  }
  if (tid < 4) c.rule[tid] = make_uint4(a.rule.lo_up[tid], a.rule.w_up[tid], a.rule.lo_dn[tid], a.rule.w_dn[tid]);
  __syncthreads();
  const Planes<NCH> pl = planes_of<NCH>(smem_raw, c, K, kNeedWhere);
  const int R = c.R, W = c.W, r0 = c.band.r0, wlo = c.band.wlo;
  // Load rows r0-1 .. r1 of both colours, interleaving the chains.
  for (int rr = warp; rr < 2 * R; rr += kThreads / 32) {
    const int t = rr / R, ri = rr - t * R;
    uint8_t* dst = pl.row(t, ri);
    const uint8_t* src = a.base + (size_t)t * a.colour_stride + (size_t)(r0 - 1 + ri) * a.P + wlo;
    for (int x = lane; x < W; x += 32) {
#pragma unroll
      for (int ch = 0; ch < NCH; ++ch) dst[x * NCH + ch] = src[(size_t)ch * a.chain_stride + x];
    }
  }
  if (warp < kCommWarps) comm_role<kMode, K, kParams, NCH>(smem_raw, c);
  else worker_role<kMode, K, kParams, NCH, kSparse>(smem_raw, c);
  __syncthreads();
  // Write back the band rows of both colours.
  const int rows = R - 2;
  for (int rr = warp; rr < 2 * rows; rr += kThreads / 32) {
    const int t = rr / rows, r = rr - t * rows;
    const uint8_t* src = pl.row(t, r + 1);
    uint8_t* dst = a.base + (size_t)t * a.colour_stride + (size_t)(r0 + r) * a.P + wlo;
    for (int x = lane; x < W; x += 32) {
#pragma unroll
      for (int ch = 0; ch < NCH; ++ch) dst[(size_t)ch * a.chain_stride + x] = src[x * NCH + ch];
    }
  }
}

template <int kMode, bool kParams, int NCH, bool kSparse>
void* kernel_for_k(int K) {
  switch (K) {
    case 1: return (void*)k_persist<kMode, 1, kParams, NCH, kSparse>;
    case 2: return (void*)k_persist<kMode, 2, kParams, NCH, kSparse>;
    case 4: return (void*)k_persist<kMode, 4, kParams, NCH, kSparse>;
    case 8: return (void*)k_persist<kMode, 8, kParams, NCH, kSparse>;
  }
  return nullptr;
}

template <int kMode, bool kParams, bool kSparse>
void* kernel_for(int K, int nch) {
  switch (nch) {
    case 1: return kernel_for_k<kMode, kParams, 1, kSparse>(K);
    case 2: return kernel_for_k<kMode, kParams, 2, kSparse>(K);
    case 4: return kSparse ? kernel_for_k<kMode, kParams, 4, kSparse>(K) : nullptr;
  }
  return nullptr;
}

}  // namespace

// ---------------------------------------------------------------------------------------
// Host: partition and launch
// ---------------------------------------------------------------------------------------

rt_status PersistPlan::build(const std::vector<uint8_t>& cand, int N, int P, int mode, int nch, int nbands_max,
                             size_t smem_limit) {
  const int H = N / 2, cols = H - 2, rows = N - 2;
  std::vector<int> lo(N, -1), hi(N, -1);  // candidate column range per row (cells)
  for (int i = 1; i <= rows; ++i)
    for (int m = 1; m <= cols; ++m)
      if (cand[(size_t)i * H + m]) {
        if (lo[i] < 0) lo[i] = m;
        hi[i] = m;
      }
  return build_from_rows(lo, hi, N, P, mode, nch, nbands_max, smem_limit);
}

rt_status PersistPlan::build_from_rows(const std::vector<int>& lo, const std::vector<int>& hi, int N, int P, int mode,
                                       int nch, int nbands_max, size_t smem_limit) {
  ok = false;
  why.clear();
  const int rows = N - 2;
  row_lo.assign(N, 0);
  row_cnt.assign(N, 0);
  row_prefix.assign(N + 1, 0);
  // Units per row: cells [lo, hi] (TinyMT) or quads [lo/4, hi/4] (fast).
  int64_t total = 0;
  for (int i = 1; i <= rows; ++i) {
    if (lo[i] < 0) continue;
    if (mode == RT_RNG_TINYMT) {
      row_lo[i] = lo[i];
      row_cnt[i] = hi[i] - lo[i] + 1;
    } else {
      row_lo[i] = lo[i] >> 2;
      row_cnt[i] = (hi[i] >> 2) - (lo[i] >> 2) + 1;
    }
    total += row_cnt[i];
  }
  if (total == 0) {
    why = "no flip candidates";
    return RT_OK;
  }
  // Bands: rows 1 .. N-2 split so that each band holds about total / G units.
  const int G = std::max(1, std::min(nbands_max, rows));
  bands.clear();
  int r = 1;
  int64_t acc = 0;
  for (int g = 0; g < G && r <= rows; ++g) {
    DmBand bd{};
    bd.r0 = r;
    const int64_t target = (total * (g + 1)) / G;
    int units = 0;
    // Take rows while that brings the running total nearer the target (the split lands on
    // the row boundary closest to it); every band gets at least one row, the last the rest.
    while (r <= rows && (2 * acc + row_cnt[r] <= 2 * target || r == bd.r0 || g == G - 1)) {
      acc += row_cnt[r];
      units += row_cnt[r];
      ++r;
    }
    bd.r1 = r;
    bd.units = units;
    bands.push_back(bd);
  }
  if (r <= rows) {  // leftover rows go to the last band
    for (; r <= rows; ++r) bands.back().units += row_cnt[r];
    bands.back().r1 = rows + 1;
  }
  // Row prefix: unit index of the first unit of each row within its band, numbering the
  // band's first row, then its last row, then the rows between (the kernel flips and
  // publishes the boundary rows first).  Windows: 16-cell aligned.
  max_units = 0;
  smem_bytes = 0;
  for (DmBand& bd : bands) {
    int u = 0, wl = P, wh = 0;
    row_prefix[bd.r0] = 0;
    u = row_cnt[bd.r0];
    bd.nb_first = u;
    if (bd.r1 - 1 > bd.r0) {
      row_prefix[bd.r1 - 1] = u;
      u += row_cnt[bd.r1 - 1];
    }
    bd.nb_boundary = u;
    for (int i = bd.r0 + 1; i < bd.r1 - 1; ++i) {
      row_prefix[i] = u;
      u += row_cnt[i];
    }
    for (int i = bd.r0 - 1; i <= bd.r1; ++i) {
      if (i < 1 || i > rows || lo[i] < 0) continue;
      wl = std::min(wl, lo[i] - 2);
      wh = std::max(wh, hi[i] + 3);
    }
    if (wh <= wl) {  // band without candidates: any aligned window works
      wl = 0;
      wh = 16;
    }
    bd.wlo = std::max(0, wl) & ~15;
    bd.whi = std::min(P, (wh + 15) & ~15);
    max_units = std::max(max_units, bd.units);
    const size_t sb = (size_t)2 * nch * (bd.r1 - bd.r0 + 2) * (bd.whi - bd.wlo);
    smem_bytes = std::max(smem_bytes, sb);
  }
  K = 0;
  for (int k : {1, 2, 4, 8})
    if ((int64_t)k * kWorkers >= max_units) {
      K = k;
      break;
    }
  if (K == 0) {
    why = "too many flip candidates per band for register-resident generators";
    return RT_OK;
  }
  const bool need_where = mode != RT_RNG_TINYMT;  // a parameter table adds the same again (see prepare)
  smem_bytes += (size_t)K * kThreads * 4 * (need_where ? 2 : 1);
  if (smem_bytes > smem_limit) {
    why = "band window exceeds shared memory";
    return RT_OK;
  }
  ok = true;
  return RT_OK;
}

#define RT_CUDA_P(expr)                                                                 \
  do {                                                                                  \
    cudaError_t _e = (expr);                                                            \
    if (_e != cudaSuccess)                                                              \
      return fail(RT_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e));     \
  } while (0)

PersistEngine::~PersistEngine() {
  for (void* p : {(void*)d_bands, (void*)d_rows, (void*)d_xbuf, (void*)d_flags, (void*)d_colours}) dev_free(p, stream);
}

rt_status PersistEngine::prepare(DmSampler& s) {
  ready = false;
  int dev = 0, sms = 0, coop = 0;
  size_t smem_optin = 0;
  RT_CUDA_P(cudaGetDevice(&dev));
  RT_CUDA_P(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  RT_CUDA_P(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  int optin = 0;
  RT_CUDA_P(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  smem_optin = (size_t)optin - 1024;
  if (!coop) {
    plan.why = "device lacks cooperative launch";
    return RT_OK;
  }
  if (rt_status st = plan.build_from_rows(s.cand_lo, s.cand_hi, s.N, s.P, s.opts.rng_mode, s.active, sms, smem_optin))
    return st;
  if (!plan.ok) return RT_OK;
  const bool params = s.tmt_params != nullptr;
  if (s.active == 3) {
    plan.ok = false;
    plan.why = "three swept chains (the resident kernel takes 1, 2 or 4)";
    return RT_OK;
  }
  if (params && s.opts.rng_mode == RT_RNG_TINYMT) plan.smem_bytes += (size_t)plan.K * kThreads * 4;  // position table
  if (plan.smem_bytes > smem_optin) {
    plan.ok = false;
    plan.why = "band window exceeds shared memory";
    return RT_OK;
  }
  kernel = dm_persist_kernel_ptr(s.opts.rng_mode, plan.K, params, s.active, true);
  RT_CUDA_P(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)plan.smem_bytes));
  int per_sm = 0;
  RT_CUDA_P(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, plan.smem_bytes));
  if ((int64_t)per_sm * sms < (int64_t)plan.bands.size()) {
    plan.ok = false;
    plan.why = "bands cannot all be resident";
    return RT_OK;
  }
  // Device copies of the plan.
  // Pool allocations ordered on the sampler's stream (device_pool.cpp).
  stream = s.stream;
  for (void** p : {(void**)&d_bands, (void**)&d_rows, (void**)&d_xbuf, (void**)&d_flags}) {
    dev_free(*p, stream);
    *p = nullptr;
  }
  if (rt_status st = dev_alloc(&d_bands, plan.bands.size() * sizeof(DmBand), stream)) return st;
  if (rt_status st = dev_alloc(&d_rows, 3 * (size_t)(s.N + 1) * sizeof(int), stream)) return st;
  std::vector<int> rows_host(3 * (size_t)(s.N + 1), 0);
  std::copy(plan.row_lo.begin(), plan.row_lo.end(), rows_host.begin());
  std::copy(plan.row_prefix.begin(), plan.row_prefix.end(), rows_host.begin() + (s.N + 1));
  RT_CUDA_P(cudaMemcpyAsync(d_bands, plan.bands.data(), plan.bands.size() * sizeof(DmBand), cudaMemcpyHostToDevice,
                            stream));
  RT_CUDA_P(cudaMemcpyAsync(d_rows, rows_host.data(), rows_host.size() * sizeof(int), cudaMemcpyHostToDevice, stream));
  xbuf_bytes = dm_xbuf_bytes((int)plan.bands.size(), s.active, s.P);
  if (rt_status st = dev_alloc(&d_xbuf, xbuf_bytes, stream)) return st;
  if (rt_status st = dev_alloc(&d_flags, (plan.bands.size() + 1) * sizeof(unsigned), stream)) return st;
  nch = s.active;
  ready = true;
  return RT_OK;
}

rt_status PersistEngine::launch(DmSampler& s, const uint8_t* colours_host, int64_t steps, uint64_t fast_seed,
                                int64_t h0) {
  const int64_t chunk_max = 65536;  // bounds one launch to a fraction of a second
  for (int64_t done = 0; done < steps;) {
    const int64_t n = std::min(chunk_max, steps - done);
    PersistArgs a{};
    a.base = s.base;
    a.P = s.P;
    a.cols = s.N / 2 - 2;
    a.chain_stride = s.chain_stride;
    a.colour_stride = s.colour_stride;
    a.nch = s.active;
    a.tmt = s.tmt;
    a.tmt_params = s.tmt_params;
    a.bands = d_bands;
    a.nbands = (int)plan.bands.size();
    a.row_lo = d_rows;
    a.row_prefix = d_rows + (s.N + 1);
    a.rule = s.rule;
    a.xbuf = d_xbuf;
    a.flags = d_flags;
    a.error = reinterpret_cast<int*>(d_flags + plan.bands.size());
    a.max_spin = s.test_max_spin > 0 ? s.test_max_spin : 1L << 22;
    a.silent_band_plus1 = s.test_silent_band + 1;
    a.steps = n;
    a.h0 = h0 + done;
    a.fast_seed = fast_seed;
    a.fast_stream = s.opts.fast_stream;
    if (s.opts.rng_mode == RT_RNG_TINYMT) {
      if (colours_cap < n) {
        dev_free(d_colours, s.stream);
        d_colours = nullptr;
        if (rt_status st = dev_alloc(&d_colours, (size_t)n, s.stream)) return st;
        colours_cap = n;
      }
      RT_CUDA_P(cudaMemcpyAsync(d_colours, colours_host + done, (size_t)n, cudaMemcpyHostToDevice, s.stream));
      a.colours = d_colours;
    }
    RT_CUDA_P(cudaMemsetAsync(d_flags, 0, (plan.bands.size() + 1) * sizeof(unsigned), s.stream));
    RT_CUDA_P(cudaMemsetAsync(d_xbuf, 0, xbuf_bytes, s.stream));  // no stale tags
    void* args[] = {&a};
    RT_CUDA_P(cudaLaunchCooperativeKernel(kernel, dim3((unsigned)plan.bands.size()), dim3(kThreads), args,
                                          plan.smem_bytes, s.stream));
    s.launches++;
    pending_error_check = true;
    done += n;
  }
  return RT_OK;
}

rt_status PersistEngine::check_error(DmSampler& s) {
  if (!pending_error_check) return RT_OK;
  int err = 0;
  RT_CUDA_P(cudaMemcpyAsync(&err, d_flags + plan.bands.size(), sizeof(int), cudaMemcpyDeviceToHost, s.stream));
  RT_CUDA_P(cudaStreamSynchronize(s.stream));
  pending_error_check = false;
  if (err) return fail(RT_ERR_TIMEOUT, "persistent sweep: a band wait gave up (neighbour never published)");
  return RT_OK;
}

}  // namespace rt

namespace rt {

size_t dm_xbuf_bytes(int nbands, int nch, int P) { return (size_t)2 * nbands * 2 * nch * P * 2; }

void* dm_persist_kernel_ptr(int mode, int K, bool params, int nch, bool sparse) {
  if (!sparse) return mode == RT_RNG_TINYMT ? kernel_for<RT_RNG_TINYMT, false, false>(K, nch)
                                            : kernel_for<RT_RNG_FAST, false, false>(K, nch);
  if (mode == RT_RNG_TINYMT)
    return params ? kernel_for<RT_RNG_TINYMT, true, true>(K, nch) : kernel_for<RT_RNG_TINYMT, false, true>(K, nch);
  return kernel_for<RT_RNG_FAST, false, true>(K, nch);
}

}  // namespace rt
