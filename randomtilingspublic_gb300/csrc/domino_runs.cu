// Run-resident engine of the domino sweep.
//
// A flip of a site of colour t (3 <-> 12) changes that site and, through the rebuild, the
// passive colour 1 - t; it never changes another site of colour t.  So consecutive
// half-sweeps of the same colour (a "run": in TinyMT mode the colours come from mt19937 and
// repeat half of the time) need neither the passive colour nor any data of another band, and
// the passive colour need only be rebuilt, once, where the colour switches.  The reference
// rebuilds it after every half-sweep (UpdateTilesKernel, dominokernel.cl:22-31); the sites
// of the active colour, which alone decide the flips, are the same either way.
//
// One cooperative launch; CTA b owns a band of colour-array rows [r0, r1) and keeps rows
// r0-1 .. r1 of both colours of every swept chain in shared memory over a column window.
// Its threads own column quads (cells 4q .. 4q+3 of one row, all chains: 4 * NCH bytes), K
// per thread, with the TinyMT generators of their cells in registers.  Per run of colour t:
//   1. after a barrier (run j > 0): where the colour switched, each thread rebuilds its quads'
//      colour t from colour 1 - t (rows above and below, and one neighbour cell in the row),
//      taking the row beyond the band from the neighbour band's published quads;
//   2. it flips each quad L times (L the run's length) in registers: 4 draws and, per 32-bit
//      word of chains, three logic ops on byte masks (which bytes can flip, which hold
//      state 3), no shared-memory traffic and no barrier;
//   3. it stores the quads, and the quads of the band's first and last rows are published
//      to the neighbour bands as tagged 64-bit words (data and tag in one single-copy-atomic
//      element, so no fence or flag is needed).
// Quads that read a neighbour's row are processed before the other quads of their thread,
// so that a band publishes its boundary rows early in each run and the neighbours' next run
// finds them in place: the exchange latency hides behind a whole run of work.  After the
// last run the passive colour is rebuilt once more, so both colours leave the launch
// consistent.  Every wait is bounded: on expiry the error word is set, all CTAs leave the
// loop at the next barrier and the host returns RT_ERR_TIMEOUT.  Exact for consistent
// tilings (both endpoints of every edge agree), as the windows assume.
//
// Coupling from the past runs in the same launch (RunArgs::attempts): each attempt resets
// the two chains from the extremal tilings, runs its half-sweeps (TinyMT: the epochs of the
// reference's schedule, generators seeded in the kernel at each epoch), rebuilds, tests
// coalescence (a fused XOR and byte test of the two chains, one count per band, a grid
// barrier), and the next attempt doubles the look-back, until the chains agree.
#include <cuda/atomic>
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <list>
#include <mutex>
#include <string>
#include <vector>

#include "domino_runs.h"
#include "domino_sweep.h"
#include "rng.cuh"

namespace rt {

namespace {

constexpr int kThreads = kRunThreads;  // the largest CTA; a plan may use fewer threads

// One column quad of NCH interleaved chains: cell k of the quad is bytes [k NCH, (k+1) NCH).
template <int NCH>
struct Quad {
  uint32_t w[NCH];
};

template <int NCH>
__device__ __forceinline__ Quad<NCH> ld_quad(const uint8_t* p) {
  Quad<NCH> q;
  if constexpr (NCH == 1) {
    q.w[0] = *reinterpret_cast<const uint32_t*>(p);
  } else if constexpr (NCH == 2) {
    const uint2 v = *reinterpret_cast<const uint2*>(p);
    q.w[0] = v.x;
    q.w[1] = v.y;
  } else {
    const uint4 v = *reinterpret_cast<const uint4*>(p);
    q.w[0] = v.x;
    q.w[1] = v.y;
    q.w[2] = v.z;
    q.w[3] = v.w;
  }
  return q;
}

template <int NCH>
__device__ __forceinline__ void st_quad(uint8_t* p, const Quad<NCH>& q) {
  if constexpr (NCH == 1) {
    *reinterpret_cast<uint32_t*>(p) = q.w[0];
  } else if constexpr (NCH == 2) {
    *reinterpret_cast<uint2*>(p) = make_uint2(q.w[0], q.w[1]);
  } else {
    *reinterpret_cast<uint4*>(p) = make_uint4(q.w[0], q.w[1], q.w[2], q.w[3]);
  }
}

// Byte mask, within word j of a quad, of the cells in the 4-bit set `cells`.
template <int NCH>
__device__ __forceinline__ uint32_t cell_bytes(uint32_t cells, int j) {
  if constexpr (NCH == 1) {
    return ((cells * 0x00204081u) & 0x01010101u) * 0xffu;  // bit k -> byte k
  } else if constexpr (NCH == 2) {
    const uint32_t x = (cells >> (2 * j)) & 3u;
    return ((x * 0x00008001u) & 0x00010001u) * 0xffffu;  // bit 0 -> low half, bit 1 -> high half
  } else {
    return 0u - ((cells >> j) & 1u);
  }
}

// Byte mask of word j of a quad from per-cell masks x[k] (all-ones or zero): the bytes of
// cell k take x[k]'s bytes (a byte permute for 2 or 4 chains).
template <int NCH>
__device__ __forceinline__ uint32_t cell_word_mask(const uint32_t (&x)[4], int j) {
  if constexpr (NCH == 1) {
    return __byte_perm(__byte_perm(x[0], x[1], 0x3340u), __byte_perm(x[2], x[3], 0x4033u), 0x7610u);
  } else if constexpr (NCH == 2) {
    return __byte_perm(x[2 * j], x[2 * j + 1], 0x7610u);  // cell 2j in bytes 0-1, 2j+1 in 2-3
  } else {
    return x[j];
  }
}

// The colour-(1 - tf) quad of a row rebuilt from colour tf (dominokernel.cl:22-31): a site
// takes its up edge from the site above's down edge (bit 2 -> 1), its down edge from below's
// up edge (1 -> 2), and its horizontal edges from the colour-tf sites left (8 -> 4) and right
// (4 -> 8) of it, at columns m, m+1 when i + tf is odd and m-1, m otherwise.  cur is the
// quad's own colour-tf cells; the cell one column over comes from the word just after (odd)
// or just before (even) the quad.
template <int NCH>
__device__ __forceinline__ Quad<NCH> rebuild_quad(const uint8_t* pf, uint32_t off, bool odd, const Quad<NCH>& above,
                                                  const Quad<NCH>& below) {
  const Quad<NCH> cur = ld_quad<NCH>(pf + off);
  constexpr int kCell = 8 * NCH;
  // x[1 .. NCH] the quad's words; x[0] the word before it, x[NCH + 1] the word after it.
  uint32_t x[NCH + 2];
#pragma unroll
  for (int j = 0; j < NCH; ++j) x[j + 1] = cur.w[j];
  if (odd) {
    x[0] = 0;
    x[NCH + 1] = *reinterpret_cast<const uint32_t*>(pf + off + 4 * NCH);
  } else {
    x[0] = *reinterpret_cast<const uint32_t*>(pf + off - 4);
    x[NCH + 1] = 0;
  }
  Quad<NCH> v;
#pragma unroll
  for (int j = 0; j < NCH; ++j) {
    const uint32_t left = odd ? x[j + 1] : __funnelshift_lc(x[j], x[j + 1], kCell);
    const uint32_t right = odd ? __funnelshift_rc(x[j + 1], x[j + 2], kCell) : x[j + 1];
    v.w[j] = ((above.w[j] >> 1) & 0x01010101u) | ((below.w[j] & 0x01010101u) << 1) | ((left & 0x08080808u) >> 1) |
             ((right & 0x04040404u) << 1);
  }
  return v;
}

// Exchange words: 4 data bytes and a 32-bit tag in one 64-bit element (single-copy atomic:
// a reader that sees the tag sees the data).  A quad is NCH such elements, 8 NCH bytes,
// aligned to 8 NCH bytes; vector accesses keep each element atomic on its own.
template <int NCH>
__device__ __forceinline__ void publish_quad(uint64_t* g, uint32_t tag, const Quad<NCH>& q) {
  const uint64_t t = (uint64_t)tag << 32;
  if constexpr (NCH == 1) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(g), "l"(t | q.w[0]) : "memory");
  } else {
#pragma unroll
    for (int j = 0; j < NCH; j += 2)
      asm volatile("st.relaxed.gpu.global.v2.u64 [%0], {%1, %2};" ::"l"(g + j), "l"(t | q.w[j]), "l"(t | q.w[j + 1])
                   : "memory");
  }
}

template <int NCH>
__device__ __forceinline__ bool poll_quad(const uint64_t* g, uint32_t tag, Quad<NCH>& q) {
  uint64_t v[NCH];
  if constexpr (NCH == 1) {
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v[0]) : "l"(g) : "memory");
  } else {
#pragma unroll
    for (int j = 0; j < NCH; j += 2)
      asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(v[j]), "=l"(v[j + 1]) : "l"(g + j) : "memory");
  }
  bool ok = true;
#pragma unroll
  for (int j = 0; j < NCH; ++j) {
    ok = ok && (uint32_t)(v[j] >> 32) == tag;
    q.w[j] = (uint32_t)v[j];
  }
  return ok;
}

// Waits (bounded) until the neighbour's quad carries `tag`.  False when the wait gave up or
// another CTA reported failure; the error word is then set.
template <int NCH>
__device__ bool wait_quad(const uint64_t* g, uint32_t tag, Quad<NCH>& q, int* error, long max_spin) {
  if (poll_quad<NCH>(g, tag, q)) return true;
  cuda::atomic_ref<int, cuda::thread_scope_device> err(*error);
  for (long it = 1;; ++it) {
    if (poll_quad<NCH>(g, tag, q)) return true;
    if ((it & 255) == 0 && err.load(cuda::memory_order_relaxed) != 0) return false;
    if (it > max_spin) {
      int zero = 0;
      err.compare_exchange_strong(zero, 1, cuda::memory_order_relaxed);
      return false;
    }
  }
}

struct RunCtx {
  RunArgs a;
  RunBand band;
  int R, W, Wb, plane_bytes;
  uint4 rule[4];  // c = (i & 1) | (t << 1): {lo_up, w_up, lo_dn, w_dn}
};

// Bounded grid-wide barrier number `gen` (0, 1, ...) of the launch, for the cooperative
// grid: thread 0 of each CTA arrives (release) and waits (acquire) until every CTA has.
// False when the wait gave up or another CTA reported failure.
__device__ bool grid_barrier(unsigned* bar, unsigned gen, int* error, long max_spin) {
  bool ok = true;
  __syncthreads();
  if (threadIdx.x == 0) {
    cuda::atomic_ref<unsigned, cuda::thread_scope_device> b(*bar);
    cuda::atomic_ref<int, cuda::thread_scope_device> err(*error);
    b.fetch_add(1u, cuda::memory_order_release);
    const unsigned target = (gen + 1) * gridDim.x;
    for (long it = 0; b.load(cuda::memory_order_acquire) < target; ++it) {
      if ((it & 255) == 0 && err.load(cuda::memory_order_relaxed) != 0) {
        ok = false;
        break;
      }
      if (it > max_spin) {
        int zero = 0;
        err.compare_exchange_strong(zero, 1, cuda::memory_order_relaxed);
        ok = false;
        break;
      }
    }
  }
  return __syncthreads_or(ok ? 0 : 1) == 0;
}

template <int kMode, int K, bool kParams, int NCH>
__global__ void __launch_bounds__(kThreads, 1) k_runs(RunArgs a) {
  extern __shared__ __align__(16) uint8_t planes[];  // [colour][R rows][Wb bytes]
  __shared__ RunCtx c;
  __shared__ unsigned long long s_diff;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nthr = (int)blockDim.x;
  if (tid == 0) {
    c.a = a;
    c.band = a.bands[blockIdx.x];
    c.R = c.band.r1 - c.band.r0 + 2;
    c.W = c.band.whi - c.band.wlo;
    c.Wb = c.W * NCH;
    c.plane_bytes = c.R * c.Wb;
  }
  if (tid < 4) c.rule[tid] = make_uint4(a.rule.lo_up[tid], a.rule.w_up[tid], a.rule.lo_dn[tid], a.rule.w_dn[tid]);
  __syncthreads();
  // Rows r0-1 .. r1 of both colours of the chains at `base`, chains interleaved cell by cell.
  auto load_band = [&](const uint8_t* base) {
    const int R = c.R, W = c.W, r0 = c.band.r0, wlo = c.band.wlo;
    for (int rr = warp; rr < 2 * R; rr += nthr / 32) {
      const int t = rr / R, ri = rr - t * R;
      uint8_t* dst = planes + t * c.plane_bytes + ri * c.Wb;
      const uint8_t* src = base + (size_t)t * a.colour_stride + (size_t)(r0 - 1 + ri) * a.P + wlo;
      for (int x = lane; x < W; x += 32) {
#pragma unroll
        for (int ch = 0; ch < NCH; ++ch) dst[x * NCH + ch] = src[(size_t)ch * a.chain_stride + x];
      }
    }
  };
  const bool cftp = a.attempts > 0;
  if (!cftp) load_band(a.base);
  // This thread's quads and, in TinyMT mode, the generators of their candidate cells
  // (loaded, or seeded in the kernel at the start of each epoch of a CFTP attempt).
  const size_t sbase = (size_t)blockIdx.x * K * nthr + tid;
  uint32_t meta[K], where[K];
  uint4 st[K][4];
#pragma unroll
  for (int s = 0; s < K; ++s) {
    meta[s] = a.slot_meta[sbase + (size_t)s * nthr];
    where[s] = a.slot_where[sbase + (size_t)s * nthr];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      st[s][k] = make_uint4(0, 0, 0, 0);
      if (kMode == RT_RNG_TINYMT && !cftp && ((meta[s] >> (kQuadValidShift + k)) & 1u)) {
        const int i = (int)(where[s] >> 16), m = 4 * (int)(where[s] & 0xffffu) + k;
        st[s][k] = a.tmt[(int64_t)(i - 1) * a.cols + (m - 1)];
      }
    }
  }
  __syncthreads();  // planes loaded

  const int b = blockIdx.x;
  const size_t row_words = (size_t)a.P / 4 * NCH;  // tagged words per exchange row
  auto exchange = [&](uint32_t tag, int band, int which, uint32_t q) -> uint64_t* {
    return a.xbuf + (((size_t)(tag & 1u) * a.nbands + band) * 2 + which) * row_words + (size_t)q * NCH;
  };
  const bool silent = b + 1 == a.silent_band_plus1;  // test hook: publishes nothing
  bool failed = false;

  // Colour tf's quad s rebuilt into colour 1 - tf, the rows beyond the band taken from the
  // neighbours' publications `tag`.
  auto rebuilt = [&](uint32_t m, uint32_t wh, int tf, uint32_t tag) -> Quad<NCH> {
    const uint8_t* pf = planes + tf * c.plane_bytes;
    const uint32_t off = m & kQuadOffMask;
    Quad<NCH> above = ld_quad<NCH>(pf + off - c.Wb), below = ld_quad<NCH>(pf + off + c.Wb);
    const uint32_t q = wh & 0xffffu;
    if ((m & kQuadHaloUp) && !failed && !wait_quad<NCH>(exchange(tag, b - 1, 1, q), tag, above, a.error, a.max_spin))
      failed = true;
    if ((m & kQuadHaloDn) && !failed && !wait_quad<NCH>(exchange(tag, b + 1, 0, q), tag, below, a.error, a.max_spin))
      failed = true;
    Quad<NCH> v = rebuild_quad<NCH>(pf, off, ((m & kQuadOdd) != 0) != (tf != 0), above, below);
    const uint32_t keep = (m >> kQuadKeepShift) & 15u;
    if (keep) {
      const Quad<NCH> old = ld_quad<NCH>(planes + (1 - tf) * c.plane_bytes + off);
#pragma unroll
      for (int j = 0; j < NCH; ++j) {
        const uint32_t km = cell_bytes<NCH>(keep, j);
        v.w[j] = (v.w[j] & ~km) | (old.w[j] & km);
      }
    }
    return v;
  };

  // Waits for the neighbours' publications `tag` of quad s without using them.  A quad may
  // overwrite its exchange slot (publication tag + 2 replaces tag) only once the neighbour
  // that reads it has moved on, which its own publication tag + 1 shows; a run that keeps its
  // colour reads no neighbour row, but must still see that publication.
  auto flow_wait = [&](uint32_t m, uint32_t wh, uint32_t tag) {
    Quad<NCH> x;
    const uint32_t q = wh & 0xffffu;
    if ((m & kQuadHaloUp) && !failed && !wait_quad<NCH>(exchange(tag, b - 1, 1, q), tag, x, a.error, a.max_spin))
      failed = true;
    if ((m & kQuadHaloDn) && !failed && !wait_quad<NCH>(exchange(tag, b + 1, 0, q), tag, x, a.error, a.max_spin))
      failed = true;
  };

  // InitTinyMT for an epoch (tinymt.clh:183-203, as k_tmt_seed): generator (i-1) cols + (m-1)
  // seeded seed + that index, with its own parameters when a table is loaded.
  auto reseed = [&](int s, uint32_t seed) {
    const uint32_t m = meta[s], wh = where[s];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (!((m >> (kQuadValidShift + k)) & 1u)) continue;
      const int i = (int)(wh >> 16), col = 4 * (int)(wh & 0xffffu) + k;
      const int64_t g = (int64_t)(i - 1) * a.cols + (col - 1);
      uint32_t m1 = kTmtMat1, m2 = kTmtMat2, tm = kTmtTmat;
      if (kParams) {
        const uint4 p = __ldg(&a.tmt_params[g]);
        m1 = p.x;
        m2 = p.y;
        tm = p.z;
      }
      st[s][k] = tmt_seed(seed + (uint32_t)g, m1, m2, tm);
    }
  };

  // One run of colour t and length L on slot s: load (the run continues the colour of the
  // previous one, or starts the segment when first) or rebuild from the other colour, L flips
  // starting at half-sweep h (fast-mode key), store, publish under tag.
  auto run_slot = [&](int s, bool first, bool load, int t, int L, int64_t h, uint32_t tag) {
    const uint32_t m = meta[s], wh = where[s];
    const uint32_t off = m & kQuadOffMask;
    uint8_t* pa = planes + t * c.plane_bytes;
    if (load && !first) flow_wait(m, wh, tag - 1);
    Quad<NCH> w = load ? ld_quad<NCH>(pa + off) : rebuilt(m, wh, 1 - t, tag - 1);
    const uint32_t valid = (m >> kQuadValidShift) & 15u;
    if (valid) {
      const uint4 rl = c.rule[((m & kQuadOdd) ? 1 : 0) | (t << 1)];
      // Per word, the bytes that can flip (state 3 or 12; a flippable site is an interior
      // vertex, so a cell without a candidate has none) and those in state 3.  A flip only
      // toggles 3 <-> 12, so within the run the quad is tracked by its state-3 bytes and
      // written back once: a byte flipped an odd number of times is XORed with 15.  Every
      // generator of the quad advances each half-sweep, branch-free: those of cells without a
      // candidate are never read back or written out.
      uint32_t flippable[NCH], three[NCH], three0[NCH];
#pragma unroll
      for (int jj = 0; jj < NCH; ++jj) {
        const uint32_t x = w.w[jj];
        const uint32_t is3 = (~((x ^ 0x03030303u) + 0x0f0f0f0fu) & 0x10101010u) >> 4;
        const uint32_t is12 = (~((x ^ 0x0c0c0c0cu) + 0x0f0f0f0fu) & 0x10101010u) >> 4;
        three[jj] = three0[jj] = is3 * 0xffu;
        flippable[jj] = (is3 | is12) * 0xffu;
      }
      for (int hh = 0; hh < L; ++hh) {
        uint32_t r[4];
        if (kMode == RT_RNG_TINYMT) {
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            if (kParams) {  // per-generator parameters, reloaded (L1) to spare registers
              const int i = (int)(wh >> 16), col = 4 * (int)(wh & 0xffffu) + k;
              const uint4 p = ((valid >> k) & 1u) ? __ldg(&a.tmt_params[(int64_t)(i - 1) * a.cols + (col - 1)])
                                                  : make_uint4(kTmtMat1, kTmtMat2, kTmtTmat, 0);
              r[k] = tmt_next_u23_mad(st[s][k], p.x, p.y, p.z);
            } else {
              r[k] = tmt_next_u23_mad(st[s][k], kTmtMat1, kTmtMat2, kTmtTmat);
            }
          }
        } else {
          const uint4 r4 = fast_quad(a.fast_seed, a.fast_stream, h + hh, wh >> 16, wh & 0xffffu);
          r[0] = r4.x;
          r[1] = r4.y;
          r[2] = r4.z;
          r[3] = r4.w;
        }
        // Per cell, all-ones where the draw accepts the up (3 -> 12) or down (12 -> 3) move.
        uint32_t up[4], dn[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          up[k] = (r[k] - rl.x) < rl.y ? 0xffffffffu : 0u;
          dn[k] = (r[k] - rl.z) < rl.w ? 0xffffffffu : 0u;
        }
        // A byte flips where it is 3 and the up move is accepted, or 12 and the down move is.
#pragma unroll
        for (int jj = 0; jj < NCH; ++jj) {
          const uint32_t u = cell_word_mask<NCH>(up, jj), d = cell_word_mask<NCH>(dn, jj) & flippable[jj];
          three[jj] ^= (three[jj] & u) | (~three[jj] & d);
        }
      }
#pragma unroll
      for (int jj = 0; jj < NCH; ++jj) w.w[jj] ^= (three[jj] ^ three0[jj]) & 0x0f0f0f0fu;
    }
    st_quad<NCH>(pa + off, w);
    if (!silent) {
      if (m & kQuadPubUp) publish_quad<NCH>(exchange(tag, b, 0, wh & 0xffffu), tag, w);
      if (m & kQuadPubDn) publish_quad<NCH>(exchange(tag, b, 1, wh & 0xffffu), tag, w);
    }
  };

  constexpr uint32_t kHalo = kQuadHaloUp | kQuadHaloDn;
  bool aborted = false, coalesced = false;
  uint32_t tag0 = 0;  // run j of a segment publishes tag0 + j + 1; tags only grow in a launch
  const int n_att = cftp ? a.attempts : 1;
  int att = 0;
  for (; att < n_att; ++att) {
    // The attempt's segment: an explicit run list (TinyMT; bit 30 of a run starts an epoch,
    // whose generators are seeded from the next epoch seed) or, in fast mode, nruns
    // alternating half-sweeps from h_start.
    int64_t nruns = a.nruns, h_start = a.h0;
    int run_off = 0, seed_off = 0;
    if (cftp) {
      if (kMode == RT_RNG_TINYMT) {
        const int4 d = a.attempt_desc[att];
        run_off = d.x;
        nruns = d.y;
        seed_off = d.z;
      } else {
        nruns = a.first_half << (a.attempt0 + att);
        h_start = -nruns;
      }
      load_band(a.start_base);
      __syncthreads();
    }
    int64_t h = h_start;
    int t_last = -1;
    for (int64_t j = 0; j < nruns; ++j) {
      int t, L;
      bool epoch = false;
      if (kMode == RT_RNG_TINYMT) {
        const uint32_t run = __ldg(&a.runs[run_off + j]);
        t = (int)(run >> 31);
        L = (int)(run & 0x3fffffffu);
        epoch = (run >> 30) & 1u;
      } else {
        t = (h & 1) ? 0 : 1;
        L = 1;
      }
      const uint32_t tag = tag0 + (uint32_t)j + 1u;
      if (j > 0 && __syncthreads_or(failed ? 1 : 0)) {
        aborted = true;
        break;
      }
      if (kMode == RT_RNG_TINYMT && epoch) {
        const uint32_t seed = __ldg(&a.epoch_seeds[seed_off++]);
#pragma unroll
        for (int s = 0; s < K; ++s)
          if (meta[s] & kQuadPresent) reseed(s, seed);
      }
      // A run rebuilds its colour only where the colour switches: an epoch boundary can split
      // one colour into two runs, and the passive colour is stale inside such a stretch.
      const bool load = j == 0 || t == t_last;
      // The band's boundary quads first: they publish this run's rows early, so the
      // neighbours' next run finds them in place, and they read rows the neighbours published
      // early in the previous run.  Then the interior quads.
      if (j > 0) {
#pragma unroll
        for (int s = 0; s < K; ++s)
          if ((meta[s] & kQuadPresent) && (meta[s] & kHalo)) run_slot(s, false, load, t, L, h, tag);
      }
#pragma unroll
      for (int s = 0; s < K; ++s)
        if ((meta[s] & kQuadPresent) && (j == 0 || !(meta[s] & kHalo))) run_slot(s, j == 0, load, t, L, h, tag);
      h += L;
      t_last = t;
    }
    // The passive colour of the last run, rebuilt from its active one.
    if (__syncthreads_or(failed ? 1 : 0)) aborted = true;
    if (!aborted && t_last >= 0) {
      const uint32_t tag = tag0 + (uint32_t)nruns;
#pragma unroll
      for (int pass = 0; pass < 2; ++pass) {
#pragma unroll
        for (int s = 0; s < K; ++s) {
          const uint32_t m = meta[s];
          if (!(m & kQuadPresent) || ((m & kHalo) != 0) != (pass == 1)) continue;
          const Quad<NCH> v = rebuilt(m, where[s], t_last, tag);
          st_quad<NCH>(planes + (1 - t_last) * c.plane_bytes + (m & kQuadOffMask), v);
        }
      }
    }
    tag0 += (uint32_t)nruns;
    if (__syncthreads_or(failed ? 1 : 0)) aborted = true;
    if (aborted || !cftp) break;
    // Coalescence: does any cell of the band rows differ between chain 0 and chain 1 (byte
    // pairs of each cell, both colours)?  Fused XOR and byte test per 32-bit word; one count
    // per band that differs, summed over the grid, then a grid barrier.
    uint32_t differ = 0;
    if (NCH == 2) {
      const int words = c.Wb / 4, rows = c.R - 2;
      for (int k = tid; k < 2 * rows * words; k += nthr) {
        const int t = k / (rows * words), rem = k - t * rows * words, r = rem / words, w = rem - r * words;
        const uint32_t x = *reinterpret_cast<const uint32_t*>(planes + t * c.plane_bytes + (r + 1) * c.Wb + 4 * w);
        const uint32_t d = (x ^ (x >> 8)) & 0x000f000fu;
        differ |= (d + 0x000f000fu) & 0x00100010u;
      }
    }
    const int band_differs = __syncthreads_or(differ != 0 ? 1 : 0);
    if (tid == 0) {
      if (band_differs) atomicAdd(&a.diff[att], 1ull);
      s_diff = 0;
    }
    if (!grid_barrier(a.grid_bar, (unsigned)att, a.error, a.max_spin)) {
      aborted = true;
      break;
    }
    if (tid == 0)
      s_diff = cuda::atomic_ref<unsigned long long, cuda::thread_scope_device>(a.diff[att]).load(
          cuda::memory_order_relaxed);
    __syncthreads();
    if (s_diff == 0) {
      coalesced = true;
      ++att;
      break;
    }
  }
  __syncthreads();
  {
    // Band rows of both colours back to the chains.
    const int rows = c.R - 2, W = c.W, r0 = c.band.r0, wlo = c.band.wlo;
    for (int rr = warp; rr < 2 * rows; rr += nthr / 32) {
      const int t = rr / rows, r = rr - t * rows;
      const uint8_t* src = planes + t * c.plane_bytes + (r + 1) * c.Wb;
      uint8_t* dst = a.base + (size_t)t * a.colour_stride + (size_t)(r0 + r) * a.P + wlo;
      for (int x = lane; x < W; x += 32) {
#pragma unroll
        for (int ch = 0; ch < NCH; ++ch) dst[(size_t)ch * a.chain_stride + x] = src[x * NCH + ch];
      }
    }
  }
  if (kMode == RT_RNG_TINYMT) {
#pragma unroll
    for (int s = 0; s < K; ++s) {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (!((meta[s] >> (kQuadValidShift + k)) & 1u)) continue;
        const int i = (int)(where[s] >> 16), m = 4 * (int)(where[s] & 0xffffu) + k;
        a.tmt[(int64_t)(i - 1) * a.cols + (m - 1)] = st[s][k];
      }
    }
  }
  if (cftp && b == 0 && tid == 0) {
    a.result[0] = att;  // attempts run
    a.result[1] = coalesced ? 1 : 0;
  }
}

template <int kMode, bool kParams, int NCH>
void* kernel_for_k(int K) {
  switch (K) {
    case 1: return (void*)k_runs<kMode, 1, kParams, NCH>;
    case 2: return (void*)k_runs<kMode, 2, kParams, NCH>;
    case 4:
      if constexpr (kMode == RT_RNG_FAST) return (void*)k_runs<kMode, 4, kParams, NCH>;
      return nullptr;
  }
  return nullptr;
}

template <int kMode, bool kParams>
void* kernel_for(int K, int nch) {
  switch (nch) {
    case 1: return kernel_for_k<kMode, kParams, 1>(K);
    case 2: return kernel_for_k<kMode, kParams, 2>(K);
    case 4: return kernel_for_k<kMode, kParams, 4>(K);
  }
  return nullptr;
}

}  // namespace

void* dm_runs_kernel_ptr(int mode, int K, bool params, int nch) {
  if (mode == RT_RNG_TINYMT)
    return params ? kernel_for<RT_RNG_TINYMT, true>(K, nch) : kernel_for<RT_RNG_TINYMT, false>(K, nch);
  if (mode == RT_RNG_FAST && !params) return kernel_for<RT_RNG_FAST, false>(K, nch);
  return nullptr;
}

// ---------------------------------------------------------------------------------------
// Host: plan and launch
// ---------------------------------------------------------------------------------------

rt_status RunPlan::build(const std::vector<int>& lo, const std::vector<int>& hi, int N, int P, int mode, int nch,
                         int nbands_max, size_t smem_limit, int k_max, int threads_per_band) {
  ok = false;
  why.clear();
  bands.clear();
  meta.clear();
  where.clear();
  nslot = 0;
  quads = draw_cells = 0;
  threads = threads_per_band;
  if (threads < 32 || threads > kThreads || threads % 32) {
    why = "threads per band must be a multiple of 32 in [32, 1024]";
    return RT_OK;
  }
  const int rows = N - 2, cols = N / 2 - 2;
  auto has = [&](int i) { return i >= 1 && i <= rows && lo[i] >= 0; };
  // Quads of each row: every cell of the row that can change, in either colour - the
  // candidates and their passive neighbours (the cell left and right of a candidate of the
  // row, the same column of a candidate in the row above or below) - within [1, cols].
  std::vector<int> qlo(N, 0), qhi(N, -1), cnt(N, 0);
  int64_t total = 0;
  for (int i = 1; i <= rows; ++i) {
    int x0 = INT_MAX, x1 = INT_MIN;
    if (has(i)) {
      x0 = lo[i] - 1;
      x1 = hi[i] + 1;
    }
    for (int d : {-1, 1})
      if (has(i + d)) {
        x0 = std::min(x0, lo[i + d]);
        x1 = std::max(x1, hi[i + d]);
      }
    x0 = std::max(x0, 1);
    x1 = std::min(x1, cols);
    if (x0 > x1) continue;
    qlo[i] = x0 >> 2;
    qhi[i] = x1 >> 2;
    cnt[i] = qhi[i] - qlo[i] + 1;
    total += cnt[i];
  }
  if (total == 0) {
    why = "no flip candidates";
    return RT_OK;
  }
  // Bands: rows split so that each holds about total / G quads.
  const int G = std::max(1, std::min(nbands_max, rows));
  {
    int r = 1;
    int64_t acc = 0;
    for (int g = 0; g < G && r <= rows; ++g) {
      RunBand bd{};
      bd.r0 = r;
      const int64_t target = (total * (g + 1)) / G;
      while (r <= rows && (2 * acc + cnt[r] <= 2 * target || r == bd.r0 || g == G - 1)) acc += cnt[r++];
      bd.r1 = r;
      bands.push_back(bd);
    }
    if (r <= rows) bands.back().r1 = rows + 1;
  }
  const int nb = (int)bands.size();
  auto in_row = [&](int i, int q) { return i >= 1 && i <= rows && cnt[i] > 0 && q >= qlo[i] && q <= qhi[i]; };
  // Per band: window, quads and their descriptors.
  struct QuadDesc {
    uint32_t meta, where;
  };
  std::vector<std::vector<QuadDesc>> inner(nb), edge(nb);
  size_t max_quads = 0;
  smem_bytes = 0;
  for (int g = 0; g < nb; ++g) {
    RunBand& bd = bands[g];
    int q0 = INT_MAX, q1 = INT_MIN;
    for (int i = bd.r0; i < bd.r1; ++i)
      if (cnt[i] > 0) {
        q0 = std::min(q0, qlo[i]);
        q1 = std::max(q1, qhi[i]);
      }
    if (q0 > q1) {
      bd.wlo = 0;
      bd.whi = std::min(P, 16);
    } else {
      bd.wlo = std::max(0, 4 * q0 - 1) & ~15;         // holds the cell left of the first quad
      bd.whi = std::min(P, (4 * q1 + 5 + 15) & ~15);  // and the cell right of the last
    }
    const int R = bd.r1 - bd.r0 + 2, W = bd.whi - bd.wlo;
    const size_t sb = (size_t)2 * nch * R * W;
    smem_bytes = std::max(smem_bytes, sb);
    if ((size_t)R * W * nch > kQuadOffMask) {
      why = "band plane exceeds the quad descriptor's offset range";
      return RT_OK;
    }
    for (int i = bd.r0; i < bd.r1; ++i) {
      for (int q = qlo[i]; cnt[i] > 0 && q <= qhi[i]; ++q) {
        uint32_t valid = 0, keep = 0;
        for (int k = 0; k < 4; ++k) {
          const int m = 4 * q + k;
          if (has(i) && m >= lo[i] && m <= hi[i]) valid |= 1u << k;
          if (m < 1 || m > cols) keep |= 1u << k;
        }
        uint32_t flags = kQuadPresent;
        if (i == bd.r0 && g > 0 && in_row(i - 1, q)) flags |= kQuadHaloUp | kQuadPubUp;
        if (i == bd.r1 - 1 && g < nb - 1 && in_row(i + 1, q)) flags |= kQuadHaloDn | kQuadPubDn;
        const uint32_t off = (uint32_t)((i - bd.r0 + 1) * W * nch + (4 * q - bd.wlo) * nch);
        const uint32_t mt =
            flags | off | ((i & 1) ? kQuadOdd : 0u) | (valid << kQuadValidShift) | (keep << kQuadKeepShift);
        const QuadDesc d{mt, ((uint32_t)i << 16) | (uint32_t)q};
        (flags & (kQuadHaloUp | kQuadHaloDn) ? edge[g] : inner[g]).push_back(d);
        draw_cells += __builtin_popcount(valid);
        ++quads;
      }
    }
    max_quads = std::max(max_quads, inner[g].size() + edge[g].size());
    if (edge[g].size() > (size_t)threads) {
      why = "more boundary quads than threads";
      return RT_OK;
    }
  }
  K = 0;
  for (int k : {1, 2, 4})
    if (k <= k_max && (size_t)k * threads >= max_quads) {
      K = k;
      break;
    }
  if (K == 0) {
    why = "too many quads per band for register-resident generators";
    return RT_OK;
  }
  if (smem_bytes > smem_limit) {
    why = "band window exceeds shared memory";
    return RT_OK;
  }
  // Slots: a band's boundary quads go to the last slot of its first threads (each such
  // thread processes them before its other quads); the rest fill the slots in order.
  meta.assign((size_t)nb * K * threads, 0u);
  where.assign((size_t)nb * K * threads, 0u);
  for (int g = 0; g < nb; ++g) {
    const size_t base = (size_t)g * K * threads;
    const int ne = (int)edge[g].size();
    for (int t = 0; t < ne; ++t) {
      meta[base + (size_t)(K - 1) * threads + t] = edge[g][t].meta;
      where[base + (size_t)(K - 1) * threads + t] = edge[g][t].where;
    }
    size_t k = 0;
    for (int s = 0; s < K && k < inner[g].size(); ++s)
      for (int t = (s == K - 1 ? ne : 0); t < threads && k < inner[g].size(); ++t, ++k) {
        meta[base + (size_t)s * threads + t] = inner[g][k].meta;
        where[base + (size_t)s * threads + t] = inner[g][k].where;
      }
    if (k < inner[g].size()) {
      why = "quads do not fit the slots";
      return RT_OK;
    }
  }
  nslot = meta.size();
  ok = true;
  return RT_OK;
}

#define RT_CUDA_R(expr)                                                                 \
  do {                                                                                  \
    cudaError_t _e = (expr);                                                            \
    if (_e != cudaSuccess)                                                              \
      return fail(RT_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e));     \
  } while (0)

RunEngine::~RunEngine() {
  for (void* p : {(void*)d_xbuf, (void*)d_error, (void*)d_runs, (void*)d_diff, (void*)d_epoch}) dev_free(p, stream);
}

RunDevPlan::~RunDevPlan() {
  if (d_bands) cudaFree(d_bands);
  if (d_meta) cudaFree(d_meta);
}

namespace {

// Plans of recent domains: building one is O(quads) host work (milliseconds at order 1024)
// plus a few MB of descriptors to upload, while a CFTP or walk call creates a fresh sampler
// for the same domain every time.  Keyed by everything the plan depends on.
struct PlanKey {
  int dev, N, P, mode, nch, nbands, threads, k_max;
  size_t smem_limit;
  std::vector<int> lo, hi;
  bool operator==(const PlanKey& o) const {
    return dev == o.dev && N == o.N && P == o.P && mode == o.mode && nch == o.nch && nbands == o.nbands &&
           threads == o.threads && k_max == o.k_max && smem_limit == o.smem_limit && lo == o.lo && hi == o.hi;
  }
};
struct PlanEntry {
  PlanKey key;
  RunPlan plan;  // without slot tables
  std::shared_ptr<RunDevPlan> dev;
};
std::mutex g_plan_mu;
std::list<PlanEntry>* g_plans = new std::list<PlanEntry>();  // never destroyed: no CUDA calls at exit
constexpr size_t kPlanCacheEntries = 8;

// The cached device tables are still those of the current context (a cudaDeviceReset
// invalidates them).
bool dev_plan_valid(const RunDevPlan& d) {
  cudaPointerAttributes at{};
  const bool ok = cudaPointerGetAttributes(&at, d.d_meta) == cudaSuccess && at.type == cudaMemoryTypeDevice;
  cudaGetLastError();
  return ok;
}

}  // namespace

rt_status RunEngine::prepare(DmSampler& s) {
  ready = false;
  int dev_id = 0, sms = 0, coop = 0, optin = 0;
  RT_CUDA_R(cudaGetDevice(&dev_id));
  RT_CUDA_R(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev_id));
  RT_CUDA_R(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev_id));
  RT_CUDA_R(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev_id));
  if (!coop) {
    plan.why = "device lacks cooperative launch";
    return RT_OK;
  }
  const bool params = s.tmt_params != nullptr;
  if (s.active != 1 && s.active != 2 && s.active != 4) {
    plan.ok = false;
    plan.why = "the run kernel takes 1, 2 or 4 swept chains";
    return RT_OK;
  }
  if (s.opts.rng_mode != RT_RNG_TINYMT && s.opts.rng_mode != RT_RNG_FAST) {
    plan.ok = false;
    plan.why = "TinyMT or fast mode only";
    return RT_OK;
  }
  const int k_max = s.opts.rng_mode == RT_RNG_TINYMT ? 2 : 4;
  bands_asked = s.eff_bands;
  threads_asked = s.eff_threads;
  const int nbands = s.eff_bands > 0 ? std::min(s.eff_bands, sms) : sms;
  const int threads = s.eff_threads > 0 ? s.eff_threads : kThreads;
  PlanKey key{dev_id, s.N, s.P, s.opts.rng_mode, s.active, nbands, threads, k_max, (size_t)optin - 1024,
              s.cand_lo, s.cand_hi};
  {
    std::lock_guard<std::mutex> lock(g_plan_mu);
    for (auto it = g_plans->begin(); it != g_plans->end(); ++it) {
      if (!(it->key == key)) continue;
      if (!dev_plan_valid(*it->dev)) {
        g_plans->erase(it);
        break;
      }
      plan = it->plan;
      dev = it->dev;
      g_plans->splice(g_plans->begin(), *g_plans, it);  // most recent first
      break;
    }
  }
  if (!dev) {
    if (rt_status st = plan.build(s.cand_lo, s.cand_hi, s.N, s.P, s.opts.rng_mode, s.active, nbands,
                                  (size_t)optin - 1024, k_max, threads))
      return st;
    if (!plan.ok) return RT_OK;
    auto d = std::make_shared<RunDevPlan>();
    RT_CUDA_R(cudaMalloc(&d->d_bands, plan.bands.size() * sizeof(RunBand)));
    RT_CUDA_R(cudaMalloc(&d->d_meta, 2 * plan.nslot * sizeof(uint32_t)));
    RT_CUDA_R(cudaMemcpy(d->d_bands, plan.bands.data(), plan.bands.size() * sizeof(RunBand), cudaMemcpyHostToDevice));
    RT_CUDA_R(cudaMemcpy(d->d_meta, plan.meta.data(), plan.nslot * sizeof(uint32_t), cudaMemcpyHostToDevice));
    RT_CUDA_R(cudaMemcpy(d->d_meta + plan.nslot, plan.where.data(), plan.nslot * sizeof(uint32_t),
                         cudaMemcpyHostToDevice));
    plan.meta = std::vector<uint32_t>();
    plan.where = std::vector<uint32_t>();
    dev = d;
    std::lock_guard<std::mutex> lock(g_plan_mu);
    g_plans->push_front(PlanEntry{std::move(key), plan, d});
    if (g_plans->size() > kPlanCacheEntries) g_plans->pop_back();
  }
  d_bands = dev->d_bands;
  d_meta = dev->d_meta;
  kernel = dm_runs_kernel_ptr(s.opts.rng_mode, plan.K, params, s.active);
  if (!kernel) {
    plan.ok = false;
    plan.why = "no run kernel for this mode";
    return RT_OK;
  }
  RT_CUDA_R(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)plan.smem_bytes));
  int per_sm = 0;
  RT_CUDA_R(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, plan.threads, plan.smem_bytes));
  if ((int64_t)per_sm * sms < (int64_t)plan.bands.size()) {
    plan.ok = false;
    plan.why = "bands cannot all be resident";
    return RT_OK;
  }
  stream = s.stream;
  for (void** p : {(void**)&d_xbuf, (void**)&d_error}) {
    dev_free(*p, stream);
    *p = nullptr;
  }
  // Two parities x bands x two rows x P / 4 quads x nch tagged 8-byte words.
  xbuf_bytes = (size_t)2 * plan.bands.size() * 2 * (s.P / 4) * s.active * 8;
  if (rt_status st = dev_alloc(&d_xbuf, xbuf_bytes, stream)) return st;
  if (rt_status st = dev_alloc(&d_error, sizeof(int), stream)) return st;
  nch = s.active;
  ready = true;
  return RT_OK;
}

void append_runs(const uint8_t* colours, int64_t n, bool epoch, std::vector<uint32_t>* runs) {
  bool fresh = true;
  for (int64_t q = 0; q < n; ++q) {
    const uint32_t t = colours[q] ? 1u : 0u;
    if (!fresh && (runs->back() >> 31) == t && (runs->back() & 0x3fffffffu) < 0x3fffffffu) {
      runs->back() += 1;
    } else {
      runs->push_back((t << 31) | ((fresh && epoch) ? 1u << 30 : 0u) | 1u);
      fresh = false;
    }
  }
}

namespace {

// The launch arguments every run-kernel launch shares.
RunArgs run_args(const RunEngine& e, DmSampler& s) {
  RunArgs a{};
  a.base = s.base;
  a.P = s.P;
  a.cols = s.N / 2 - 2;
  a.nch = s.active;
  a.nbands = (int)e.plan.bands.size();
  a.K = e.plan.K;
  a.chain_stride = s.chain_stride;
  a.colour_stride = s.colour_stride;
  a.tmt = s.tmt;
  a.tmt_params = s.tmt_params;
  a.bands = e.d_bands;
  a.slot_meta = e.d_meta;
  a.slot_where = e.d_meta + e.plan.nslot;
  a.rule = s.rule;
  a.xbuf = e.d_xbuf;
  a.error = e.d_error;
  a.max_spin = s.test_max_spin > 0 ? s.test_max_spin : 1L << 22;
  a.silent_band_plus1 = s.test_silent_band + 1;
  a.fast_stream = s.opts.fast_stream;
  return a;
}

}  // namespace

rt_status RunEngine::launch(DmSampler& s, const uint8_t* colours_host, int64_t steps, uint64_t fast_seed,
                            int64_t h0) {
  const int64_t chunk_max = 65536;  // bounds one launch to a fraction of a second
  std::vector<uint32_t> runs;
  for (int64_t done = 0; done < steps;) {
    const int64_t n = std::min(chunk_max, steps - done);
    RunArgs a = run_args(*this, s);
    if (colours_host) {
      runs.clear();
      append_runs(colours_host + done, n, false, &runs);
      if (runs_cap < (int64_t)runs.size()) {
        dev_free(d_runs, s.stream);
        d_runs = nullptr;
        if (rt_status st = dev_alloc(&d_runs, runs.size() * sizeof(uint32_t), s.stream)) return st;
        runs_cap = (int64_t)runs.size();
      }
      RT_CUDA_R(
          cudaMemcpyAsync(d_runs, runs.data(), runs.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s.stream));
      a.runs = d_runs;
      a.nruns = (int64_t)runs.size();
    } else {
      a.nruns = n;  // fast mode: n alternating half-sweeps from h0 + done
    }
    a.h0 = h0 + done;
    a.fast_seed = fast_seed;
    RT_CUDA_R(cudaMemsetAsync(d_error, 0, sizeof(int), s.stream));
    RT_CUDA_R(cudaMemsetAsync(d_xbuf, 0, xbuf_bytes, s.stream));  // no stale tags
    void* args[] = {&a};
    RT_CUDA_R(cudaLaunchCooperativeKernel(kernel, dim3((unsigned)plan.bands.size()), dim3((unsigned)plan.threads),
                                          args, plan.smem_bytes, s.stream));
    s.launches++;
    pending_error_check = true;
    done += n;
  }
  return RT_OK;
}

rt_status RunEngine::cftp(DmSampler& s, int a0, int n, const std::vector<std::vector<Epoch>>& epochs,
                          int64_t first_sweeps, uint64_t fast_seed, int* attempts_run, bool* coalesced) {
  *attempts_run = 0;
  *coalesced = false;
  if (n < 1 || n > 40 || s.active != 2) return fail(RT_ERR_INVALID_ARGUMENT, "run-resident cftp: 1..40 attempts, 2 chains");
  RunArgs a = run_args(*this, s);
  const bool tmt = s.opts.rng_mode == RT_RNG_TINYMT;
  std::vector<uint32_t> runs, seeds;
  std::vector<int4> desc;
  if (tmt) {
    if ((int)epochs.size() < n) return fail(RT_ERR_INVALID_ARGUMENT, "run-resident cftp: epochs missing");
    for (int k = 0; k < n; ++k) {
      int4 d = make_int4((int)runs.size(), 0, (int)seeds.size(), 0);
      for (const Epoch& e : epochs[k]) {
        if (!e.colours || e.colours->empty()) continue;
        seeds.push_back(e.seed);
        append_runs(e.colours->data(), (int64_t)e.colours->size(), true, &runs);
      }
      d.y = (int)runs.size() - d.x;
      desc.push_back(d);
    }
    if (runs_cap < (int64_t)runs.size()) {
      dev_free(d_runs, s.stream);
      d_runs = nullptr;
      if (rt_status st = dev_alloc(&d_runs, runs.size() * sizeof(uint32_t), s.stream)) return st;
      runs_cap = (int64_t)runs.size();
    }
    const size_t desc_off = (seeds.size() * sizeof(uint32_t) + 15) / 16 * 16;
    const size_t eb = desc_off + desc.size() * sizeof(int4);
    if (epoch_cap < eb) {
      dev_free(d_epoch, s.stream);
      d_epoch = nullptr;
      if (rt_status st = dev_alloc(&d_epoch, eb, s.stream)) return st;
      epoch_cap = eb;
    }
    RT_CUDA_R(cudaMemcpyAsync(d_runs, runs.data(), runs.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s.stream));
    RT_CUDA_R(cudaMemcpyAsync(d_epoch, seeds.data(), seeds.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s.stream));
    RT_CUDA_R(cudaMemcpyAsync(reinterpret_cast<uint8_t*>(d_epoch) + desc_off, desc.data(), desc.size() * sizeof(int4),
                              cudaMemcpyHostToDevice, s.stream));
    a.runs = d_runs;
    a.epoch_seeds = d_epoch;
    a.attempt_desc = reinterpret_cast<const int4*>(reinterpret_cast<uint8_t*>(d_epoch) + desc_off);
  }
  if (!d_diff) {
    if (rt_status st = dev_alloc(&d_diff, 44 * sizeof(unsigned long long), s.stream)) return st;
  }
  a.attempts = n;
  a.attempt0 = a0;
  a.start_base = s.base + 2 * s.chain_stride;
  a.first_half = 2 * first_sweeps;
  a.fast_seed = fast_seed;
  a.diff = d_diff;
  a.grid_bar = reinterpret_cast<unsigned*>(d_diff + 40);
  a.result = reinterpret_cast<int*>(d_diff + 41);
  RT_CUDA_R(cudaMemsetAsync(d_error, 0, sizeof(int), s.stream));
  RT_CUDA_R(cudaMemsetAsync(d_xbuf, 0, xbuf_bytes, s.stream));
  RT_CUDA_R(cudaMemsetAsync(d_diff, 0, 44 * sizeof(unsigned long long), s.stream));
  void* args[] = {&a};
  RT_CUDA_R(cudaLaunchCooperativeKernel(kernel, dim3((unsigned)plan.bands.size()), dim3((unsigned)plan.threads), args,
                                        plan.smem_bytes, s.stream));
  s.launches++;
  int res[2] = {0, 0};
  RT_CUDA_R(cudaMemcpyAsync(res, d_diff + 41, sizeof res, cudaMemcpyDeviceToHost, s.stream));
  pending_error_check = true;
  if (rt_status st = check_error(s)) return st;  // synchronises the stream
  *attempts_run = res[0];
  *coalesced = res[1] != 0;
  return RT_OK;
}

rt_status RunEngine::check_error(DmSampler& s) {
  if (!pending_error_check) return RT_OK;
  int err = 0;
  RT_CUDA_R(cudaMemcpyAsync(&err, d_error, sizeof(int), cudaMemcpyDeviceToHost, s.stream));
  RT_CUDA_R(cudaStreamSynchronize(s.stream));
  pending_error_check = false;
  if (err) return fail(RT_ERR_TIMEOUT, "run-resident sweep: a band wait gave up (neighbour never published)");
  return RT_OK;
}

}  // namespace rt
