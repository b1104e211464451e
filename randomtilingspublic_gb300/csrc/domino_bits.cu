// Bit-plane engine of the domino sweep.
//
// The reference keeps one byte per lattice vertex (its four edge bits: 1 up, 2 down, 4 left,
// 8 right, DominoTiler.cpp:24-33), rotates the active colour and rebuilds the passive one from
// it after every half-sweep (dominokernel.cl:5-31).  Every lattice edge joins a black and a
// white vertex, so the tiling is fully described by one bit per edge; a rotation of colour t
// toggles the four edges of each flipped vertex, and no vertex of colour t shares an edge with
// another, so the passive colour needs no rebuild at all.  Here each colour-array row i holds
// four planes of 32-bit words, bit k of word w for cell m = 32 w + k:
//   VD_t(i)  the down edge of cell (i, m) of colour t (the up edge of cell (i+1, m), colour 1-t)
//   HE(i)    the lattice edge (i, 2m)-(i, 2m+1), HO(i) the edge (i, 2m+1)-(i, 2m+2)
// Cell (i, m) of colour t sits at lattice column 2m + o, o = (i + 1 - t) & 1; its edges are up
// VD_{1-t}(i-1), down VD_t(i), and left/right HE, HO (o = 1) or HO one cell to the left, HE
// (o = 0).  Its state is 3 (up and down) or 12 (left and right) exactly when it can flip.
//
// One cooperative launch, one CTA (band) per SM: the band's rows r0-1 .. r1 of every plane of
// every swept chain stay in shared memory for the whole launch (a few KB: 4 bits per cell and
// chain instead of 2 bytes).  A warp holds up to 16 words (slots) of rows of one parity; lane
// l keeps, for each slot, the TinyMT generator of cell 32 w + l in registers.  Per half-sweep
// each lane draws for its slots, and two warp ballots turn the 32 draws of a word into its
// up-move and down-move acceptance words; lane s keeps those of slot s and updates slot s's
// word with two logic operations per chain (state-3 and flippable masks, as the byte kernels
// track them).  Colour runs (consecutive half-sweeps of one colour, TinyMT mode) iterate in
// registers; the planes are read at the start of a run and the net toggles written back at its
// end.  Bands share the vertical-edge planes of their boundary rows: after every run a band
// publishes, for the words of its first and last rows, the running XOR of its own changes to
// those planes as tagged 64-bit words; the neighbour reads them where the colour switches (the
// plane it is about to read was last changed by the other band) and at the end of the launch.
// The boundary words sit in the first kPhaseA slots of the warps and are processed last in each
// run, after the interior words, so a publication has the neighbour's whole interior phase to
// travel before it is read.  Every wait is bounded (error word, RT_ERR_TIMEOUT on the host).  Exact for
// consistent tilings whose flip candidates all lie away from the unrebuilt border cells
// (rows 0 and N-1, columns m = 0 and m > N/2 - 2), where the reference's byte updates and the
// edge planes agree; the engine declines other inputs.
//
// Coupling from the past runs in one launch (BitArgs::attempts), as in the run kernel: reset,
// the attempt's epochs (generators seeded in the kernel), the coalescence test (planes of the
// two chains compared, one count per band, a grid barrier), look-back doubling.
#include <cuda/atomic>
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <list>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "domino_bits.h"
#include "domino_sweep.h"
#include "rng.cuh"

namespace rt {

namespace {

constexpr int K = kBitSlots;
constexpr int kPhaseA = 8;  // slots of the boundary phase of a run (the plan puts boundary words there)
constexpr int kMid = 12;     // the interior phase in two halves, the halo loads issued between
constexpr int kGroup = 16;  // slots whose draws interleave (a warp skips empty groups)
template <int V>
using Int = std::integral_constant<int, V>;

// Exchange element [word][colour][chain]: 32 data bits and a 32-bit tag in one 64-bit word
// (single-copy atomic: a reader that sees the tag sees the data).
template <int NCH>
__device__ __forceinline__ bool xb_poll(const uint64_t* g, uint32_t tag, uint32_t (&v)[NCH]) {
  uint64_t x[NCH];
  if constexpr (NCH == 1) {
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(x[0]) : "l"(g) : "memory");
  } else {
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(x[0]), "=l"(x[1]) : "l"(g) : "memory");
  }
  bool ok = true;
#pragma unroll
  for (int c = 0; c < NCH; ++c) {
    ok = ok && (uint32_t)(x[c] >> 32) == tag;
    v[c] = (uint32_t)x[c];
  }
  return ok;
}

// Waits (bounded) until the element carries `tag`.  False when the wait gave up or another
// CTA reported failure; the error word is then set.
template <int NCH>
__device__ bool xb_wait(const uint64_t* g, uint32_t tag, uint32_t (&v)[NCH], int* error, long max_spin) {
  if (xb_poll<NCH>(g, tag, v)) return true;
  cuda::atomic_ref<int, cuda::thread_scope_device> err(*error);
  for (long it = 1;; ++it) {
    if (xb_poll<NCH>(g, tag, v)) return true;
    if ((it & 255) == 0 && err.load(cuda::memory_order_relaxed) != 0) return false;
    if (it > max_spin) {
      int zero = 0;
      err.compare_exchange_strong(zero, 1, cuda::memory_order_relaxed);
      return false;
    }
  }
}

// Lane s keeps the ballots of slot s: a predicated select, never a branch (a divergent branch
// per slot and half-sweep would serialise the warp).
__device__ __forceinline__ void pick_if_lane(uint32_t& up, uint32_t& dn, uint32_t bu, uint32_t bd, int lane, int s) {
  asm("{\n\t.reg .pred p;\n\tsetp.eq.s32 p, %4, %5;\n\tselp.b32 %0, %2, %0, p;\n\tselp.b32 %1, %3, %1, p;\n\t}"
      : "+r"(up), "+r"(dn)
      : "r"(bu), "r"(bd), "r"(lane), "r"(s));
}

// Bounded grid-wide barrier number `gen` of the launch (thread 0 of each CTA arrives and
// waits); false when the wait gave up or another CTA reported failure.
__device__ bool bits_grid_barrier(unsigned* bar, unsigned gen, int* error, long max_spin) {
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

template <int NCH, bool kParams>
__global__ void __launch_bounds__(kBitMaxWarps * 32, 1) k_bits(BitArgs a) {
  extern __shared__ __align__(16) uint32_t sm[];
  __shared__ BitBand bd;
  __shared__ uint4 srule[4];
  __shared__ unsigned long long s_diff;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = (int)(blockDim.x >> 5);
  const int b = blockIdx.x;
  if (tid == 0) bd = a.bands[b];
  // Acceptance tests on the tempered word t0 (the draw is t0 >> 9): up when t0 < w_up 2^9,
  // down when t0 - lo_dn 2^9 < w_dn 2^9 (unsigned); the host admits only intervals for which
  // these products fit 32 bits and lo_up is 0, where the tests equal the reference's.
  if (tid < 4) srule[tid] = make_uint4(a.rule.w_up[tid] << 9, a.rule.lo_dn[tid] << 9, a.rule.w_dn[tid] << 9, 0u);
  __syncthreads();
  const int r0 = bd.r0, r1 = bd.r1, wlo = bd.wlo;
  const int R = r1 - r0 + 2, Wn = bd.whi - wlo + 2;
  // Shared memory: planes [R rows from r0-1][VD0, VD1, HE, HO][Wn words from wlo-1][NCH];
  // boundary deltas [own, received][up: row r0-1, down: row r1-1][colour][Wn][NCH]; slots.
  // (32-bit offsets into sm: the shared-memory addresses stay 32-bit.)
  uint32_t* const planes = sm;
  const int dlt_off = R * 4 * Wn * NCH;
  uint2* const sslot = reinterpret_cast<uint2*>(sm + dlt_off + 8 * Wn * NCH);
  auto PL = [&](int ri, int p, int wi) -> uint32_t* { return sm + ((ri * 4 + p) * Wn + wi) * NCH; };
  auto DL = [&](int kind, int side, int colour, int wi) -> uint32_t* {
    return sm + dlt_off + (((kind * 2 + side) * 2 + colour) * Wn + wi) * NCH;
  };
  for (int k = tid; k < nwarps * K; k += (int)blockDim.x) sslot[k] = a.slots[(size_t)b * nwarps * K + k];

  // The band's window of the chains at `src` as planes (one warp per row and word: lane l
  // reads cell 32 w + l of both colours), the deltas cleared.
  auto load_band = [&](const uint8_t* src) {
    for (int it = warp; it < R * Wn; it += nwarps) {
      const int ri = it / Wn, wi = it - ri * Wn;
      const int i = r0 - 1 + ri, w = wlo - 1 + wi, m = 32 * w + lane;
      const bool in = w >= 0 && m < a.P;
#pragma unroll
      for (int c = 0; c < NCH; ++c) {
        const uint8_t* row = src + (size_t)c * a.chain_stride + (size_t)i * a.P;
        const uint32_t b0 = in ? row[m] : 0u, b1 = in ? row[a.colour_stride + m] : 0u;
        const uint32_t bo = (i & 1) ? b1 : b0;  // the colour whose cells sit at odd lattice columns
        const uint32_t vd0 = __ballot_sync(~0u, (b0 >> 1) & 1u), vd1 = __ballot_sync(~0u, (b1 >> 1) & 1u);
        const uint32_t he = __ballot_sync(~0u, (bo >> 2) & 1u), ho = __ballot_sync(~0u, (bo >> 3) & 1u);
        if (lane == 0) {
          PL(ri, 0, wi)[c] = vd0;
          PL(ri, 1, wi)[c] = vd1;
          PL(ri, 2, wi)[c] = he;
          PL(ri, 3, wi)[c] = ho;
        }
      }
    }
    for (int k = tid; k < 8 * Wn * NCH; k += (int)blockDim.x) sm[dlt_off + k] = 0u;
  };
  const bool cftp = a.attempts > 0;
  if (!cftp) load_band(a.base);
  __syncthreads();  // slots (and planes) in place

  // This warp's slots: the first nK are present (the plan puts boundary words in the first
  // kPhaseA, which every run processes last); all have the row parity par.  Kept in shared
  // memory (nK << 8 | par << 16) and read once per run, like the loop state below: registers
  // go to the generators.
  __shared__ int s_warp[kBitMaxWarps];
  __shared__ int s_ctl[4];  // the segment's first run, runs, first epoch seed; tag0
  if (lane == 0) {
    int nK = 0;
    for (int s = 0; s < K; ++s)
      if (sslot[warp * K + s].y & kSlotPresent) nK = s + 1;
    s_warp[warp] = (nK << 8) | (int)((sslot[warp * K].x >> 16) & 1u) << 16;
  }
  if (tid == 0) s_ctl[3] = 0;
  volatile int* const ctl = s_ctl;
  // Generator of lane `lane` in slot s: number (i-1) cols + (m-1) of cell (i, m = 32 w + lane),
  // held when the cell lies in the row's candidate range.
  auto gen_index = [&](int s, bool* valid) -> int64_t {
    const uint2 e = sslot[warp * K + s];
    const int i = (int)(e.x >> 16), w = (int)(e.x & 0xffffu);
    const int blo = (int)((e.y >> 8) & 31u), bhi = (int)((e.y >> 16) & 31u);
    *valid = (e.y & kSlotPresent) && lane >= blo && lane <= bhi;
    return (int64_t)(i - 1) * a.cols + (32 * w + lane - 1);
  };
  uint4 gen[K];
#pragma unroll
  for (int s = 0; s < K; ++s) {
    gen[s] = make_uint4(0u, 0u, 0u, 0u);
    bool v;
    const int64_t g = gen_index(s, &v);
    if (!cftp && v) gen[s] = a.tmt[g];
  }
  // InitTinyMT for an epoch (tinymt.clh:183-203, as k_tmt_seed).
  auto reseed = [&](uint32_t seed) {
#pragma unroll
    for (int s = 0; s < K; ++s) {
      bool v;
      const int64_t g = gen_index(s, &v);
      if (!v) continue;
      uint32_t m1 = kTmtMat1, m2 = kTmtMat2, tm = kTmtTmat;
      if (kParams) {
        const uint4 p = __ldg(&a.tmt_params[g]);
        m1 = p.x;
        m2 = p.y;
        tm = p.z;
      }
      gen[s] = tmt_seed(seed + (uint32_t)g, m1, m2, tm);
    }
  };
  // Exchange element of word w, colour `colour`: publication `which` (0 up: a band's first
  // row, 1 down: its last row) of band `band` under tag.
  auto xel = [&](uint32_t tag, int band, int which, int w, int colour) -> uint64_t* {
    const unsigned idx =
        (((((unsigned)(tag & 1u) * a.nbands + band) * 2 + which) * a.xwords + w) * 2 + colour) * NCH;
    return a.xbuf + idx;
  };
  const bool silent = b + 1 == a.silent_band_plus1;  // test hook: publishes nothing
  bool failed = false;

  // Lane ℓ of a warp keeps the word of slot ℓ & 15, chain ℓ >> 4 (lanes 16-31 idle with one
  // chain), for the run's colour t: three (cells in state 3) and flip (cells that can flip).
  const int ws = lane & (K - 1), wc = NCH == 2 ? lane >> 4 : 0;
  const bool lane_ok = NCH == 2 || lane < K;
  // The word's planes for colour t, the halo plane patched first with the neighbour's
  // publication tag - 1 where `patch` asks for it (the colour switched), or only waited for
  // (`wait`: so that the slot it overwrites next has been read).
  // The exchange element a boundary word reads first (the band above's, else the band
  // below's), loaded ahead of use: the load's round trip overlaps other work.
  auto word_prefetch = [&](int t, uint32_t tag) -> uint64_t {
    const uint2 e = sslot[warp * K + ws];
    const int w = (int)(e.x & 0xffffu);
    if (!(e.y & (kSlotHaloUp | kSlotHaloDn))) return 0ull;
    const bool up = (e.y & kSlotHaloUp) != 0;
    uint64_t x;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];"
                 : "=l"(x)
                 : "l"(xel(tag - 1, up ? b - 1 : b + 1, up ? 1 : 0, w, up ? 1 - t : t) + wc)
                 : "memory");
    return x;
  };
  auto word_setup = [&](int t, bool patch, bool wait, uint32_t tag, uint64_t pf, uint32_t& three, uint32_t& flip) {
    const uint2 e = sslot[warp * K + ws];
    const int i = (int)(e.x >> 16), w = (int)(e.x & 0xffffu);
    const int ri = i - r0 + 1, wi = w - wlo + 1;
    if ((patch || wait) && (e.y & (kSlotHaloUp | kSlotHaloDn))) {
      const int pf_side = (e.y & kSlotHaloUp) ? 0 : 1;
#pragma unroll
      for (int side = 0; side < 2; ++side) {  // a one-row band can have both
        const bool up = side == 0;
        if (!(e.y & (up ? kSlotHaloUp : kSlotHaloDn)) || failed) continue;
        uint32_t v[1];
        if (side == pf_side && (uint32_t)(pf >> 32) == tag - 1) {
          v[0] = (uint32_t)pf;  // the prefetched element already carries the tag
        } else if (!xb_wait<1>(xel(tag - 1, up ? b - 1 : b + 1, up ? 1 : 0, w, up ? 1 - t : t) + wc, tag - 1, v,
                               a.error, a.max_spin)) {
          failed = true;
        }
        if (patch && !failed) {
          uint32_t* pl = up ? PL(ri - 1, 1 - t, wi) : PL(ri, t, wi);
          uint32_t* rc = up ? DL(1, 0, 1 - t, wi) : DL(1, 1, t, wi);
          pl[wc] ^= v[0] ^ rc[wc];
          rc[wc] = v[0];
        }
      }
    }
    const bool aligned = ((i + 1 - t) & 1) != 0;  // o = 1: left HE, right HO of the same word
    const uint32_t U = PL(ri - 1, 1 - t, wi)[wc], D = PL(ri, t, wi)[wc];
    const uint32_t* po = PL(ri, 3, wi);
    const uint32_t he = PL(ri, 2, wi)[wc];
    const uint32_t lft = aligned ? he : __funnelshift_l(po[wc - NCH], po[wc], 1);
    const uint32_t rgt = aligned ? po[wc] : he;
    // Flippable: up = down, left = right, up != left (states 3 and 12).
    flip = ~(U ^ D) & ~(lft ^ rgt) & (U ^ lft);
    three = U & flip;
  };
  // L half-sweeps of slots [S0, S1) (compile-time: their draws interleave), those from nK on
  // absent; lane ℓ's word takes slot ℓ & 15's acceptance words (zero for the other slots).
  // `first` runs after the draws of the first half-sweep and before their update (the
  // boundary phase sets its words up there, its halo loads overlapping those draws).
  auto draw_phase = [&](auto S0c, auto S1c, int nK, int L, uint4 rl, uint32_t& three, uint32_t& flip, auto first) {
    constexpr int S0 = decltype(S0c)::value, S1 = decltype(S1c)::value;
    for (int hh = 0; hh < L; ++hh) {
      uint32_t up_m = 0u, dn_m = 0u;
#pragma unroll
      for (int s = S0; s < S1; ++s) {
        if (s % kGroup == 0 && s >= nK) break;  // warp-uniform: the rest of the phase is empty
        uint32_t m1 = kTmtMat1, m2 = kTmtMat2, tm = kTmtTmat;
        if (kParams) {  // per-generator parameters, reloaded (L1) to spare registers
          bool v;
          const int64_t g = gen_index(s, &v);
          if (v) {
            const uint4 p = __ldg(&a.tmt_params[g]);
            m1 = p.x;
            m2 = p.y;
            tm = p.z;
          }
        }
        const uint32_t t0 = tmt_next_t0_mad(gen[s], m1, m2, tm);
        const uint32_t bu = __ballot_sync(~0u, t0 < rl.x);
        const uint32_t bdn = __ballot_sync(~0u, t0 - rl.y < rl.z);
        pick_if_lane(up_m, dn_m, bu, bdn, ws, s);
      }
      if (hh == 0) first();
      three ^= (three & up_m) | (~three & flip & dn_m);
    }
  };
  // A boundary word's net toggles of the run added to the band's own deltas, which are
  // published under tag (the planes are written back at the end of the run).
  auto word_publish = [&](int t, uint32_t tag, uint32_t three, uint32_t flip) {
    const uint2 e = sslot[warp * K + ws];
    if (!(e.y & (kSlotPubUp | kSlotPubDn))) return;
    const int i = (int)(e.x >> 16), w = (int)(e.x & 0xffffu);
    const int ri = i - r0 + 1, wi = w - wlo + 1;
    const uint32_t T = three ^ (PL(ri - 1, 1 - t, wi)[wc] & flip);  // cells flipped an odd number of times
    if (e.y & kSlotPubUp) DL(0, 0, 1 - t, wi)[wc] ^= T;
    if (e.y & kSlotPubDn) DL(0, 1, t, wi)[wc] ^= T;
    if (!silent) {
      const uint64_t tg = (uint64_t)tag << 32;
#pragma unroll
      for (int side = 0; side < 2; ++side) {  // a one-row band can publish both ways
        if (!(e.y & (side == 0 ? kSlotPubUp : kSlotPubDn))) continue;
#pragma unroll
        for (int colour = 0; colour < 2; ++colour) {
          uint64_t* g = xel(tag, b, side, w, colour) + wc;
          asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(g), "l"(tg | DL(0, side, colour, wi)[wc])
                       : "memory");
        }
      }
    }
  };
  // The run's net toggles of lane ℓ's word back to the planes.
  auto word_writeback = [&](int t, uint32_t three, uint32_t flip) {
    const uint2 e = sslot[warp * K + ws];
    const int i = (int)(e.x >> 16), w = (int)(e.x & 0xffffu);
    const int ri = i - r0 + 1, wi = w - wlo + 1;
    const bool aligned = ((i + 1 - t) & 1) != 0;
    uint32_t* pu = PL(ri - 1, 1 - t, wi) + wc;
    const uint32_t T = three ^ (*pu & flip);
    if (T != 0u) {
      *pu ^= T;
      PL(ri, t, wi)[wc] ^= T;
      PL(ri, 2, wi)[wc] ^= T;
      if (aligned) {
        PL(ri, 3, wi)[wc] ^= T;
      } else {  // left edges: bit k - 1 of this word's HO, bit 31 of the previous word's
        atomicXor(PL(ri, 3, wi) + wc, T >> 1);
        if (T & 1u) atomicXor(PL(ri, 3, wi - 1) + wc, T << 31);
      }
    }
  };
  bool aborted = false, coalesced = false;
  // Run j of a segment publishes tag0 + j + 1 (s_ctl[3]); tags only grow in a launch.
  const int n_att = cftp ? a.attempts : 1;
  int att = 0;
  for (; att < n_att; ++att) {
    __syncthreads();
    if (tid == 0) {
      if (cftp) {
        const int4 d = a.attempt_desc[att];
        s_ctl[0] = d.x;
        s_ctl[1] = d.y;
        s_ctl[2] = d.z;
      } else {
        s_ctl[0] = 0;
        s_ctl[1] = (int)a.nruns;
        s_ctl[2] = 0;
      }
    }
    if (cftp) load_band(a.start_base);
    __syncthreads();
    const int nruns = ctl[1];
    int t_last = -1;
    // Each run's descriptor is loaded one run ahead: its latency hides behind the run before.
    uint32_t run_next = nruns > 0 ? __ldg(&a.runs[ctl[0]]) : 0u;
    for (int j = 0; j < nruns; ++j) {
      const uint32_t run = run_next;
      if (j + 1 < nruns) run_next = __ldg(&a.runs[ctl[0] + j + 1]);
      const int t = (int)(run >> 31), L = (int)(run & 0x3fffffffu);
      const bool epoch = (run >> 30) & 1u;
      if (j > 0 && __syncthreads_or(failed ? 1 : 0)) {
        aborted = true;
        break;
      }
      if (epoch) {
        reseed(__ldg(&a.epoch_seeds[ctl[2]]));
        __syncthreads();
        if (tid == 0) s_ctl[2] = s_ctl[2] + 1;
      }
      const uint32_t tag = (uint32_t)ctl[3] + (uint32_t)j + 1u;
      const int wv = ((volatile int*)s_warp)[warp];
      const int nK = (wv >> 8) & 255, par = (wv >> 16) & 1;
      const uint4 rl = srule[par | (t << 1)];
      const bool pull = j > 0 && t != t_last, wait = j > 0 && !pull;
      const bool mine = lane_ok && ws < nK;
      uint32_t three = 0u, flip = 0u;  // lanes without a word update zeros, branch-free
      // Interior words first; between their two halves the boundary words (slots below
      // kPhaseA) load their halo elements, the neighbours' publications at the end of the
      // previous run, which have had the first half to arrive and load in the second.  (Boundary
      // words the plan could not fit below kPhaseA wait for theirs at once.)
      if (mine && ws >= kPhaseA) word_setup(t, pull, wait, tag, 0ull, three, flip);
      auto none = [] {};
      if (nK > kPhaseA) draw_phase(Int<kPhaseA>{}, Int<kMid>{}, nK, L, rl, three, flip, none);
      uint64_t pf = 0ull;
      if (mine && ws < kPhaseA && (pull || wait)) pf = word_prefetch(t, tag);
      if (nK > kMid) draw_phase(Int<kMid>{}, Int<K>{}, nK, L, rl, three, flip, none);
      auto boundary_setup = [&] {
        if (mine && ws < kPhaseA) word_setup(t, pull, wait, tag, pf, three, flip);
      };
      if (nK > 0) draw_phase(Int<0>{}, Int<kPhaseA>{}, nK, L, rl, three, flip, boundary_setup);
      if (mine) {
        word_publish(t, tag, three, flip);
        word_writeback(t, three, flip);
      }
      t_last = t;
    }
    if (__syncthreads_or(failed ? 1 : 0)) aborted = true;
    const uint32_t tag0 = (uint32_t)ctl[3];
    // The neighbours' last publications of every boundary word, so both boundary rows' planes
    // hold the final edges.
    if (!aborted && nruns > 0) {
      const uint32_t tag = tag0 + (uint32_t)nruns;
      const int nup = bd.fin1 - bd.fin0;
      for (int k = tid; k < bd.fin2 - bd.fin0 && !failed; k += (int)blockDim.x) {
        const bool up = k < nup;
        const int w = (int)a.fin[bd.fin0 + k], wi = w - wlo + 1;
#pragma unroll
        for (int colour = 0; colour < 2; ++colour) {
          uint32_t v[NCH];
          if (!xb_wait<NCH>(xel(tag, up ? b - 1 : b + 1, up ? 1 : 0, w, colour), tag, v, a.error, a.max_spin)) {
            failed = true;
            break;
          }
          uint32_t *pl = PL(up ? 0 : R - 2, colour, wi), *rc = DL(1, up ? 0 : 1, colour, wi);
#pragma unroll
          for (int c = 0; c < NCH; ++c) {
            pl[c] ^= v[c] ^ rc[c];
            rc[c] = v[c];
          }
        }
      }
    }
    if (__syncthreads_or(failed ? 1 : 0)) aborted = true;
    if (tid == 0) s_ctl[3] = (int)(tag0 + (uint32_t)nruns);
    if (aborted || !cftp) break;
    // Coalescence: does any plane word of the band's rows differ between the two chains?
    uint32_t differ = 0;
    if (NCH == 2) {
      const int cnt = (R - 2) * 4 * Wn;
      const uint32_t* p0 = planes + (size_t)4 * Wn * NCH;
      for (int k = tid; k < cnt; k += (int)blockDim.x) differ |= p0[2 * k] ^ p0[2 * k + 1];
    }
    const int band_differs = __syncthreads_or(differ != 0u ? 1 : 0);
    if (tid == 0) {
      if (band_differs) atomicAdd(&a.diff[att], 1ull);
      s_diff = 0;
    }
    if (!bits_grid_barrier(a.grid_bar, (unsigned)att, a.error, a.max_spin)) {
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
  // Band rows of both colours back to the chains as edge masks: cells m in [1, cols] of the
  // written words (the others keep their bytes, as the reference never rebuilds them).
  for (int it = warp; it < (R - 2) * (Wn - 2) * 2; it += nwarps) {
    const int t = it & 1, q = it >> 1;
    const int ri = 1 + q / (Wn - 2), wi = 1 + q % (Wn - 2);
    const int i = r0 - 1 + ri, w = wlo - 1 + wi, m = 32 * w + lane;
    if (m < 1 || m > a.cols || m >= a.P) continue;
    const bool aligned = ((i + 1 - t) & 1) != 0;
#pragma unroll
    for (int c = 0; c < NCH; ++c) {
      const uint32_t up = (PL(ri - 1, 1 - t, wi)[c] >> lane) & 1u, dn = (PL(ri, t, wi)[c] >> lane) & 1u;
      const uint32_t he = (PL(ri, 2, wi)[c] >> lane) & 1u;
      uint32_t lft, rgt;
      if (aligned) {
        lft = he;
        rgt = (PL(ri, 3, wi)[c] >> lane) & 1u;
      } else {
        lft = lane ? (PL(ri, 3, wi)[c] >> (lane - 1)) & 1u : PL(ri, 3, wi - 1)[c] >> 31;
        rgt = he;
      }
      a.base[(size_t)c * a.chain_stride + (size_t)t * a.colour_stride + (size_t)i * a.P + m] =
          (uint8_t)(up | (dn << 1) | (lft << 2) | (rgt << 3));
    }
  }
#pragma unroll
  for (int s = 0; s < K; ++s) {
    bool v;
    const int64_t g = gen_index(s, &v);
    if (v) a.tmt[g] = gen[s];
  }
  if (cftp && b == 0 && tid == 0) {
    a.result[0] = att;  // attempts run
    a.result[1] = coalesced ? 1 : 0;
  }
}

}  // namespace

void* dm_bits_kernel_ptr(bool params, int nch) {
  if (nch == 1) return params ? (void*)k_bits<1, true> : (void*)k_bits<1, false>;
  if (nch == 2) return params ? (void*)k_bits<2, true> : (void*)k_bits<2, false>;
  return nullptr;
}

// ---------------------------------------------------------------------------------------
// Host: plan and launch
// ---------------------------------------------------------------------------------------

rt_status BitPlan::build(const std::vector<int>& lo, const std::vector<int>& hi, int N, int P, int nch,
                         int nbands_max, size_t smem_limit) {
  ok = false;
  why.clear();
  bands.clear();
  slots.clear();
  fin.clear();
  words = draw_cells = 0;
  warps = 0;
  wn_max = 0;
  smem_bytes = 0;
  const int rows = N - 2, xw = (P + 31) / 32;
  if (xw > 0xffff || N > 0xffff) {
    why = "tiling too large for the slot descriptors";
    return RT_OK;
  }
  // Candidate words of each row.
  std::vector<int> wl(N + 1, 0), wh(N + 1, -1), cnt(N + 1, 0);
  auto has = [&](int i) { return i >= 1 && i <= rows && lo[i] >= 0; };
  int64_t total = 0;
  int cand_rows = 0;
  for (int i = 1; i <= rows; ++i)
    if (has(i)) {
      wl[i] = lo[i] / 32;
      wh[i] = hi[i] / 32;
      cnt[i] = wh[i] - wl[i] + 1;
      total += cnt[i];
      ++cand_rows;
    }
  if (total == 0) {
    why = "no flip candidates";
    return RT_OK;
  }
  // Bands: consecutive rows, at most G of them, each within kBitMaxWarps warps (the words of
  // each row parity fill their own warps); the largest band, which sets the pace, as small as
  // possible (binary search on its word count, bands filled greedily).
  const int G = std::max(1, std::min(nbands_max, cand_rows));
  auto warps_of = [](int64_t even, int64_t odd) { return (int)((even + K - 1) / K + (odd + K - 1) / K); };
  // Rows are taken in pairs, so a band's first and last rows have different parities and its
  // boundary words fill the warps of both parities.
  auto pack = [&](int64_t cap, std::vector<BitBand>* out) -> bool {
    out->clear();
    for (int r = 1; r <= rows;) {
      BitBand bb{};
      bb.r0 = r;
      int64_t par[2] = {0, 0};
      while (r <= rows) {
        const int take = std::min(2, rows - r + 1);
        int64_t p2[2] = {par[0], par[1]};
        for (int q = 0; q < take; ++q) p2[(r + q) & 1] += cnt[r + q];
        const bool over = p2[0] + p2[1] > cap || warps_of(p2[0], p2[1]) > kBitMaxWarps;
        if (over && r > bb.r0) break;
        if (warps_of(p2[0], p2[1]) > kBitMaxWarps) return false;  // one row pair alone is too wide
        par[0] = p2[0];
        par[1] = p2[1];
        r += take;
      }
      bb.r1 = r;
      out->push_back(bb);
      if ((int)out->size() > G) return false;
    }
    return true;
  };
  int64_t cap_lo = 1, cap_hi = total;
  if (!pack(cap_hi, &bands)) {
    why = "too many words for one band per SM with register-resident generators";
    return RT_OK;
  }
  while (cap_lo < cap_hi) {
    const int64_t mid = (cap_lo + cap_hi) / 2;
    if (pack(mid, &bands)) cap_hi = mid;
    else cap_lo = mid + 1;
  }
  if (!pack(cap_lo, &bands)) {
    why = "too many words for one band per SM with register-resident generators";
    return RT_OK;
  }
  const int nb = (int)bands.size();
  auto in_row = [&](int i, int w) { return has(i) && w >= wl[i] && w <= wh[i]; };
  // Slots per band: the words of each row parity dealt over that parity's warps, boundary
  // words first, so that each warp's boundary slots come first and spread over the warps.
  std::vector<std::vector<std::vector<uint2>>> per(nb);  // [band][warp] slots
  for (int g = 0; g < nb; ++g) {
    BitBand& bb = bands[g];
    int w0 = INT_MAX, w1 = INT_MIN;
    for (int i = std::max(1, bb.r0 - 1); i <= std::min(rows, bb.r1); ++i)
      if (has(i)) {
        w0 = std::min(w0, wl[i]);
        w1 = std::max(w1, wh[i]);
      }
    if (w0 > w1) {
      w0 = 0;
      w1 = 0;
    }
    bb.wlo = std::max(0, w0 - 1);
    bb.whi = std::min(xw, w1 + 2);
    wn_max = std::max(wn_max, bb.whi - bb.wlo + 2);
    std::vector<uint2> cls[2][2];  // [parity][boundary?]
    for (int i = bb.r0; i < bb.r1; ++i) {
      if (!has(i)) continue;
      for (int w = wl[i]; w <= wh[i]; ++w) {
        uint32_t f = kSlotPresent;
        if (i == bb.r0 && g > 0) {
          f |= kSlotPubUp;
          if (in_row(i - 1, w)) f |= kSlotHaloUp;
        }
        if (i == bb.r1 - 1 && g < nb - 1) {
          f |= kSlotPubDn;
          if (in_row(i + 1, w)) f |= kSlotHaloDn;
        }
        const int m0 = std::max(lo[i], 32 * w), m1 = std::min(hi[i], 32 * w + 31);
        f |= (uint32_t)(m0 - 32 * w) << 8 | (uint32_t)(m1 - 32 * w) << 16;
        draw_cells += m1 - m0 + 1;
        ++words;
        const bool edge = (f & (kSlotPubUp | kSlotPubDn | kSlotHaloUp | kSlotHaloDn)) != 0;
        cls[i & 1][edge ? 0 : 1].push_back(make_uint2(((uint32_t)i << 16) | (uint32_t)w, f));
      }
    }
    // Warps per parity class: enough for its words, and for its boundary words below kPhaseA
    // where that fits; the band's remaining warps (up to kBitMaxWarps) then go one at a time to
    // the class with the most words per warp, so that the work spreads over every warp.
    const size_t n[2] = {cls[0][0].size() + cls[0][1].size(), cls[1][0].size() + cls[1][1].size()};
    int cw[2];
    for (int p = 0; p < 2; ++p) cw[p] = (int)((n[p] + K - 1) / K);
    for (int p = 0; p < 2; ++p) {
      const int want = (int)((cls[p][0].size() + kPhaseA - 1) / kPhaseA);
      if (want > cw[p] && cw[0] + cw[1] + (want - cw[p]) <= kBitMaxWarps) cw[p] = want;
    }
    while (cw[0] + cw[1] < kBitMaxWarps) {
      int best = -1;
      for (int p = 0; p < 2; ++p)
        if (n[p] > (size_t)cw[p] && (best < 0 || n[p] * cw[best] > n[best] * cw[p])) best = p;
      if (best < 0) break;
      ++cw[best];
    }
    for (int p = 0; p < 2; ++p) {
      std::vector<uint2> list = cls[p][0];
      list.insert(list.end(), cls[p][1].begin(), cls[p][1].end());
      if (list.empty()) continue;
      const size_t first = per[g].size();
      per[g].resize(first + cw[p], std::vector<uint2>());
      for (size_t k = 0; k < list.size(); ++k) per[g][first + k % cw[p]].push_back(list[k]);
    }
    warps = std::max(warps, (int)per[g].size());
    // Final reads: the words of the row above the band (published down by the band above)
    // and of the row below it (published up by the band below).
    bb.fin0 = (int)fin.size();
    if (g > 0 && has(bb.r0 - 1))
      for (int w = wl[bb.r0 - 1]; w <= wh[bb.r0 - 1]; ++w) fin.push_back((uint32_t)w);
    bb.fin1 = (int)fin.size();
    if (g < nb - 1 && has(bb.r1))
      for (int w = wl[bb.r1]; w <= wh[bb.r1]; ++w) fin.push_back((uint32_t)w);
    bb.fin2 = (int)fin.size();
  }
  if (warps > kBitMaxWarps) {
    why = "too many words per band for register-resident generators";
    return RT_OK;
  }
  warps = std::max(warps, 1);
  slots.assign((size_t)nb * warps * K, make_uint2(0u, 0u));
  for (int g = 0; g < nb; ++g)
    for (size_t wp = 0; wp < per[g].size(); ++wp)
      for (size_t s = 0; s < per[g][wp].size(); ++s) slots[((size_t)g * warps + wp) * K + s] = per[g][wp][s];
  for (const BitBand& bb : bands) {
    const size_t R = (size_t)(bb.r1 - bb.r0 + 2), Wn = (size_t)(bb.whi - bb.wlo + 2);
    smem_bytes = std::max(smem_bytes, (R * 4 * Wn * nch + 8 * Wn * nch) * sizeof(uint32_t) +
                                          (size_t)warps * K * sizeof(uint2));
  }
  if (smem_bytes > smem_limit) {
    why = "band window exceeds shared memory";
    return RT_OK;
  }
  ok = true;
  return RT_OK;
}

#define RT_CUDA_B(expr)                                                                 \
  do {                                                                                  \
    cudaError_t _e = (expr);                                                            \
    if (_e != cudaSuccess)                                                              \
      return fail(RT_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e));     \
  } while (0)

BitEngine::~BitEngine() {
  for (void* p : {(void*)d_xbuf, (void*)d_error, (void*)d_runs, (void*)d_diff, (void*)d_epoch}) dev_free(p, stream);
}

BitDevPlan::~BitDevPlan() {
  if (d_bands) cudaFree(d_bands);
  if (d_slots) cudaFree(d_slots);
  if (d_fin) cudaFree(d_fin);
}

namespace {

// Plans of recent domains: building one is O(words) host work plus a few hundred KB of tables
// to upload (0.7 ms at order 1024), while a CFTP or walk call creates a fresh sampler for the
// same domain every time.  Keyed by everything the plan depends on.
struct BitPlanKey {
  int dev, N, P, nch, nbands;
  size_t smem_limit;
  std::vector<int> lo, hi;
  bool operator==(const BitPlanKey& o) const {
    return dev == o.dev && N == o.N && P == o.P && nch == o.nch && nbands == o.nbands && smem_limit == o.smem_limit &&
           lo == o.lo && hi == o.hi;
  }
};
struct BitPlanEntry {
  BitPlanKey key;
  BitPlan plan;  // without its tables
  std::shared_ptr<BitDevPlan> dev;
};
std::mutex g_bit_plan_mu;
std::list<BitPlanEntry>* g_bit_plans = new std::list<BitPlanEntry>();  // never destroyed: no CUDA calls at exit
constexpr size_t kBitPlanCacheEntries = 8;

// The cached tables are still those of the current context (a cudaDeviceReset invalidates them).
bool bit_dev_plan_valid(const BitDevPlan& d) {
  cudaPointerAttributes at{};
  const bool ok = cudaPointerGetAttributes(&at, d.d_slots) == cudaSuccess && at.type == cudaMemoryTypeDevice;
  cudaGetLastError();
  return ok;
}

}  // namespace

rt_status BitEngine::prepare(DmSampler& s) {
  ready = false;
  plan.ok = false;
  int dev_id = 0, sms = 0, coop = 0, optin = 0;
  RT_CUDA_B(cudaGetDevice(&dev_id));
  RT_CUDA_B(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev_id));
  RT_CUDA_B(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev_id));
  RT_CUDA_B(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev_id));
  if (!coop) {
    plan.why = "device lacks cooperative launch";
    return RT_OK;
  }
  if (s.opts.rng_mode != RT_RNG_TINYMT) {
    plan.why = "TinyMT mode only";
    return RT_OK;
  }
  if (s.active != 1 && s.active != 2) {
    plan.why = "the bit-plane kernel takes 1 or 2 swept chains";
    return RT_OK;
  }
  if (s.border_candidates) {
    plan.why = "a flip candidate borders the cells the reference never rebuilds";
    return RT_OK;
  }
  for (int c = 0; c < 4; ++c) {  // the kernel tests the tempered word against interval ends x 2^9
    const uint64_t lo_dn = s.rule.lo_dn[c], w_dn = s.rule.w_dn[c];
    if (s.rule.lo_up[c] != 0 || s.rule.w_up[c] >= (1u << 23) || w_dn >= (1u << 23) || lo_dn + w_dn > (1u << 23)) {
      plan.why = "rule intervals outside the bit-plane kernel's compare range";
      return RT_OK;
    }
  }
  const int nbands = s.eff_bands > 0 ? std::min(s.eff_bands, sms) : sms;
  stream = s.stream;
  BitPlanKey key{dev_id, s.N, s.P, s.active, nbands, (size_t)optin - 1024, s.cand_lo, s.cand_hi};
  dev.reset();
  {
    std::lock_guard<std::mutex> lock(g_bit_plan_mu);
    for (auto it = g_bit_plans->begin(); it != g_bit_plans->end(); ++it) {
      if (!(it->key == key)) continue;
      if (!bit_dev_plan_valid(*it->dev)) {
        g_bit_plans->erase(it);
        break;
      }
      plan = it->plan;
      dev = it->dev;
      g_bit_plans->splice(g_bit_plans->begin(), *g_bit_plans, it);  // most recent first
      break;
    }
  }
  if (!dev) {
    if (rt_status st = plan.build(s.cand_lo, s.cand_hi, s.N, s.P, s.active, nbands, (size_t)optin - 1024)) return st;
    if (!plan.ok) return RT_OK;
    auto d = std::make_shared<BitDevPlan>();
    const size_t nb = plan.bands.size(), nfin = std::max<size_t>(1, plan.fin.size());
    RT_CUDA_B(cudaMalloc(&d->d_bands, nb * sizeof(BitBand)));
    RT_CUDA_B(cudaMalloc(&d->d_slots, plan.slots.size() * sizeof(uint2)));
    RT_CUDA_B(cudaMalloc(&d->d_fin, nfin * sizeof(uint32_t)));
    RT_CUDA_B(cudaMemcpy(d->d_bands, plan.bands.data(), nb * sizeof(BitBand), cudaMemcpyHostToDevice));
    RT_CUDA_B(cudaMemcpy(d->d_slots, plan.slots.data(), plan.slots.size() * sizeof(uint2), cudaMemcpyHostToDevice));
    if (!plan.fin.empty())
      RT_CUDA_B(cudaMemcpy(d->d_fin, plan.fin.data(), plan.fin.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    plan.slots = std::vector<uint2>();
    plan.fin = std::vector<uint32_t>();
    dev = d;
    std::lock_guard<std::mutex> lock(g_bit_plan_mu);
    g_bit_plans->push_front(BitPlanEntry{std::move(key), plan, d});
    if (g_bit_plans->size() > kBitPlanCacheEntries) g_bit_plans->pop_back();
  }
  d_bands = dev->d_bands;
  d_slots = dev->d_slots;
  d_fin = dev->d_fin;
  kernel = dm_bits_kernel_ptr(s.tmt_params != nullptr, s.active);
  if (!kernel) {
    plan.ok = false;
    plan.why = "no bit-plane kernel for this chain count";
    return RT_OK;
  }
  RT_CUDA_B(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)plan.smem_bytes));
  int per_sm = 0;
  RT_CUDA_B(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, plan.warps * 32, plan.smem_bytes));
  if ((int64_t)per_sm * sms < (int64_t)plan.bands.size()) {
    plan.ok = false;
    plan.why = "bands cannot all be resident";
    return RT_OK;
  }
  for (void** p : {(void**)&d_xbuf, (void**)&d_error}) {
    dev_free(*p, stream);
    *p = nullptr;
  }
  const size_t nb = plan.bands.size();
  xwords = (s.P + 31) / 32 + 1;
  xbuf_bytes = (size_t)2 * nb * 2 * xwords * 2 * s.active * sizeof(uint64_t);
  if (rt_status st = dev_alloc(&d_xbuf, xbuf_bytes, stream)) return st;
  if (rt_status st = dev_alloc(&d_error, sizeof(int), stream)) return st;
  nch = s.active;
  ready = true;
  return RT_OK;
}

namespace {

BitArgs bit_args(const BitEngine& e, DmSampler& s) {
  BitArgs a{};
  a.base = s.base;
  a.N = s.N;
  a.P = s.P;
  a.cols = s.N / 2 - 2;
  a.nbands = (int)e.plan.bands.size();
  a.warps = e.plan.warps;
  a.wn_max = e.plan.wn_max;
  a.chain_stride = s.chain_stride;
  a.colour_stride = s.colour_stride;
  a.tmt = s.tmt;
  a.tmt_params = s.tmt_params;
  a.bands = e.d_bands;
  a.slots = e.d_slots;
  a.fin = e.d_fin;
  a.rule = s.rule;
  a.xbuf = e.d_xbuf;
  a.xwords = e.xwords;
  a.error = e.d_error;
  a.max_spin = s.test_max_spin > 0 ? s.test_max_spin : 1L << 22;
  a.silent_band_plus1 = s.test_silent_band + 1;
  return a;
}

}  // namespace

rt_status BitEngine::launch(DmSampler& s, const uint8_t* colours_host, int64_t steps) {
  const int64_t chunk_max = 65536;  // bounds one launch to a fraction of a second
  std::vector<uint32_t> runs;
  for (int64_t done = 0; done < steps;) {
    const int64_t n = std::min(chunk_max, steps - done);
    BitArgs a = bit_args(*this, s);
    runs.clear();
    append_runs(colours_host + done, n, false, &runs);
    if (runs_cap < (int64_t)runs.size()) {
      dev_free(d_runs, s.stream);
      d_runs = nullptr;
      if (rt_status st = dev_alloc(&d_runs, runs.size() * sizeof(uint32_t), s.stream)) return st;
      runs_cap = (int64_t)runs.size();
    }
    RT_CUDA_B(cudaMemcpyAsync(d_runs, runs.data(), runs.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s.stream));
    a.runs = d_runs;
    a.nruns = (int64_t)runs.size();
    RT_CUDA_B(cudaMemsetAsync(d_error, 0, sizeof(int), s.stream));
    RT_CUDA_B(cudaMemsetAsync(d_xbuf, 0, xbuf_bytes, s.stream));  // no stale tags
    void* args[] = {&a};
    RT_CUDA_B(cudaLaunchCooperativeKernel(kernel, dim3((unsigned)plan.bands.size()), dim3((unsigned)plan.warps * 32),
                                          args, plan.smem_bytes, s.stream));
    s.launches++;
    pending_error_check = true;
    done += n;
  }
  return RT_OK;
}

rt_status BitEngine::cftp(DmSampler& s, int n, const std::vector<std::vector<RunEngine::Epoch>>& epochs,
                          int* attempts_run, bool* coalesced) {
  *attempts_run = 0;
  *coalesced = false;
  if (n < 1 || n > 40 || s.active != 2) return fail(RT_ERR_INVALID_ARGUMENT, "bit-plane cftp: 1..40 attempts, 2 chains");
  if ((int)epochs.size() < n) return fail(RT_ERR_INVALID_ARGUMENT, "bit-plane cftp: epochs missing");
  BitArgs a = bit_args(*this, s);
  std::vector<uint32_t> runs, seeds;
  std::vector<int4> desc;
  for (int k = 0; k < n; ++k) {
    int4 d = make_int4((int)runs.size(), 0, (int)seeds.size(), 0);
    for (const RunEngine::Epoch& e : epochs[k]) {
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
  RT_CUDA_B(cudaMemcpyAsync(d_runs, runs.data(), runs.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s.stream));
  RT_CUDA_B(cudaMemcpyAsync(d_epoch, seeds.data(), seeds.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s.stream));
  RT_CUDA_B(cudaMemcpyAsync(reinterpret_cast<uint8_t*>(d_epoch) + desc_off, desc.data(), desc.size() * sizeof(int4),
                            cudaMemcpyHostToDevice, s.stream));
  a.runs = d_runs;
  a.epoch_seeds = d_epoch;
  a.attempt_desc = reinterpret_cast<const int4*>(reinterpret_cast<uint8_t*>(d_epoch) + desc_off);
  if (!d_diff) {
    if (rt_status st = dev_alloc(&d_diff, 44 * sizeof(unsigned long long), s.stream)) return st;
  }
  a.attempts = n;
  a.start_base = s.base + 2 * s.chain_stride;
  a.diff = d_diff;
  a.grid_bar = reinterpret_cast<unsigned*>(d_diff + 40);
  a.result = reinterpret_cast<int*>(d_diff + 41);
  RT_CUDA_B(cudaMemsetAsync(d_error, 0, sizeof(int), s.stream));
  RT_CUDA_B(cudaMemsetAsync(d_xbuf, 0, xbuf_bytes, s.stream));
  RT_CUDA_B(cudaMemsetAsync(d_diff, 0, 44 * sizeof(unsigned long long), s.stream));
  void* args[] = {&a};
  RT_CUDA_B(cudaLaunchCooperativeKernel(kernel, dim3((unsigned)plan.bands.size()), dim3((unsigned)plan.warps * 32), args,
                                        plan.smem_bytes, s.stream));
  s.launches++;
  int res[2] = {0, 0};
  RT_CUDA_B(cudaMemcpyAsync(res, d_diff + 41, sizeof res, cudaMemcpyDeviceToHost, s.stream));
  pending_error_check = true;
  if (rt_status st = check_error(s)) return st;  // synchronises the stream
  *attempts_run = res[0];
  *coalesced = res[1] != 0;
  return RT_OK;
}

rt_status BitEngine::check_error(DmSampler& s) {
  if (!pending_error_check) return RT_OK;
  int err = 0;
  RT_CUDA_B(cudaMemcpyAsync(&err, d_error, sizeof(int), cudaMemcpyDeviceToHost, s.stream));
  RT_CUDA_B(cudaStreamSynchronize(s.stream));
  pending_error_check = false;
  if (err) return fail(RT_ERR_TIMEOUT, "bit-plane sweep: a band wait gave up (neighbour never published)");
  return RT_OK;
}

}  // namespace rt
