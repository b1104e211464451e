// Resident persistent engine of the domino sweep.
//
// One cooperative launch runs many half-sweeps.  CTA b owns a band of colour-array rows
// [r0, r1) and keeps, in shared memory, rows r0-1 .. r1 of both colours of every swept chain
// over a 4-byte-aligned column window that contains every site of the band that can change
// (see dm_plan_partition).  Its flip candidates ("units": one site per unit in TinyMT mode,
// a column quad in fast mode) are dealt round-robin to its threads, whose TinyMT generator
// states stay in registers for the whole launch.  Each half-sweep:
//   1. flip: every unit draws and tests its site of the rotated colour t in every chain;
//   2. publish: the band's first and last rows of colour t go to a double-buffered exchange
//      slot in global memory, then a release store of the half-sweep count to the band flag;
//   3. wait: acquire-poll the two neighbour flags (bounded; on expiry an error code is set
//      and every CTA leaves its loop), copy their rows into the halo rows;
//   4. rebuild: the passive colour of the band, four sites per 32-bit word.
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

constexpr int kThreads = 1024;

__device__ __forceinline__ uint8_t flip_site(uint32_t e, uint32_t u, uint32_t lo_up, uint32_t w_up, uint32_t lo_dn,
                                             uint32_t w_dn) {
  if (e == 3u) return (u - lo_up) < w_up ? 12 : 3;
  if (e == 12u) return (u - lo_dn) < w_dn ? 3 : 12;
  return (uint8_t)e;
}

struct Smem {
  uint8_t* p;
  int R, W;  // rows (band + 2 halo), window bytes
  // byte of chain ch, colour t, colour-array row i (band-relative index ri = i - r0 + 1), window column x
  __device__ uint8_t* row(int ch, int t, int ri) const { return p + ((size_t)(ch * 2 + t) * R + ri) * W; }
};

// Waits until *flag >= target; returns false when the wait gave up or another CTA failed.
__device__ bool wait_flag(unsigned* flag, unsigned target, int* error, long max_spin) {
  cuda::atomic_ref<unsigned, cuda::thread_scope_device> f(*flag);
  cuda::atomic_ref<int, cuda::thread_scope_device> err(*error);
  long it = 0;
  while (f.load(cuda::memory_order_acquire) < target) {
    if ((++it & 255) == 0 && err.load(cuda::memory_order_relaxed) != 0) return false;
    if (it > max_spin) {
      int zero = 0;
      err.compare_exchange_strong(zero, 1, cuda::memory_order_relaxed);
      return false;
    }
    __nanosleep(64);
  }
  return true;
}

template <int kMode, int K, bool kParams>
__global__ void __launch_bounds__(kThreads, 1) k_persist(PersistArgs a) {
  extern __shared__ __align__(16) uint8_t smem_raw[];
  __shared__ int s_abort;
  const int b = blockIdx.x;
  const DmBand band = a.bands[b];
  const int nch = a.nch;
  const int R = band.r1 - band.r0 + 2, W = band.whi - band.wlo, words = W / 4;
  Smem sm{smem_raw, R, W};
  const int tid = threadIdx.x;

  // Load rows r0-1 .. r1 of both colours of every chain (window only).
  for (int idx = tid; idx < nch * 2 * R * words; idx += kThreads) {
    const int w = idx % words, rest = idx / words, ri = rest % R, ct = rest / R;
    const int ch = ct >> 1, t = ct & 1;
    const uint8_t* g = a.base + (size_t)ch * a.chain_stride + (size_t)t * a.colour_stride +
                       (size_t)(band.r0 - 1 + ri) * a.P + band.wlo;
    reinterpret_cast<uint32_t*>(sm.row(ch, t, ri))[w] = reinterpret_cast<const uint32_t*>(g)[w];
  }
  if (tid == 0) s_abort = 0;

  // This thread's units: list index tid + s * kThreads, rows enumerated in order.
  uint32_t pos[K];
  uint4 st[K];
#pragma unroll
  for (int s = 0; s < K; ++s) {
    const int c = tid + s * kThreads;
    pos[s] = 0xffffffffu;
    st[s] = make_uint4(0, 0, 0, 0);
    if (c < band.units) {
      // binary search the band's rows for the one holding unit c
      int lo = band.r0, hi = band.r1 - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (a.row_prefix[mid] <= c) lo = mid;
        else hi = mid - 1;
      }
      const int i = lo, u = a.row_lo[i] + (c - a.row_prefix[i]);
      pos[s] = ((uint32_t)i << 16) | (uint32_t)u;
      if (kMode == RT_RNG_TINYMT) st[s] = a.tmt[(int64_t)(i - 1) * a.cols + (u - 1)];
    }
  }
  __syncthreads();

  const int up = b - 1, dn = b + 1;
  const DmBand bu = up >= 0 ? a.bands[up] : band, bd = dn < a.nbands ? a.bands[dn] : band;
  for (int64_t h = 0; h < a.steps; ++h) {
    const int64_t hh = a.h0 + h;
    const int t = (kMode == RT_RNG_TINYMT) ? (a.colours[h] ? 1 : 0) : ((hh & 1) ? 0 : 1);
    // 1. flip
#pragma unroll
    for (int s = 0; s < K; ++s) {
      if (pos[s] == 0xffffffffu) continue;
      const int i = (int)(pos[s] >> 16), u = (int)(pos[s] & 0xffffu);
      const int c = (i & 1) | (t << 1);
      const uint32_t lo_up = a.rule.lo_up[c], w_up = a.rule.w_up[c], lo_dn = a.rule.lo_dn[c], w_dn = a.rule.w_dn[c];
      const int ri = i - band.r0 + 1;
      if (kMode == RT_RNG_TINYMT) {
        uint32_t m1 = kTmtMat1, m2 = kTmtMat2, tm = kTmtTmat;
        if (kParams) {
          const uint4 p = __ldg(&a.tmt_params[(int64_t)(i - 1) * a.cols + (u - 1)]);
          m1 = p.x; m2 = p.y; tm = p.z;
        }
        const uint32_t r = tmt_next_u23(st[s], m1, m2, tm);
        const int x = u - band.wlo;
        for (int ch = 0; ch < nch; ++ch) {
          uint8_t* q = sm.row(ch, t, ri) + x;
          const uint32_t e = *q;
          const uint8_t n = flip_site(e, r, lo_up, w_up, lo_dn, w_dn);
          if (n != e) *q = n;
        }
      } else {
        const uint4 r4 = fast_quad(a.fast_seed, a.fast_stream, hh, (uint32_t)i, (uint32_t)u);
        const uint32_t rr[4] = {r4.x, r4.y, r4.z, r4.w};
        for (int ch = 0; ch < nch; ++ch) {
          uint8_t* rowp = sm.row(ch, t, ri);
#pragma unroll
          for (int k4 = 0; k4 < 4; ++k4) {
            const int m = 4 * u + k4;
            if (m < 1 || m > a.cols) continue;
            uint8_t* q = rowp + (m - band.wlo);
            const uint32_t e = *q;
            const uint8_t n = flip_site(e, rr[k4], lo_up, w_up, lo_dn, w_dn);
            if (n != e) *q = n;
          }
        }
      }
    }
    __syncthreads();
    // 2. publish the band's first and last rows of colour t
    const int slot = (int)(h & 1);
    for (int idx = tid; idx < 2 * nch * words; idx += kThreads) {
      const int w = idx % words, rest = idx / words, ch = rest % nch, which = rest / nch;
      const int ri = which == 0 ? 1 : R - 2;
      uint8_t* g = a.xbuf + ((((size_t)slot * a.nbands + b) * 2 + which) * nch + ch) * a.P + band.wlo;
      __stcg(reinterpret_cast<uint32_t*>(g) + w, reinterpret_cast<const uint32_t*>(sm.row(ch, t, ri))[w]);
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) {
      cuda::atomic_ref<unsigned, cuda::thread_scope_device> f(a.flags[b]);
      f.store((unsigned)(h + 1), cuda::memory_order_release);
      bool ok = true;
      if (up >= 0) ok = wait_flag(&a.flags[up], (unsigned)(h + 1), a.error, a.max_spin);
      if (ok && dn < a.nbands) ok = wait_flag(&a.flags[dn], (unsigned)(h + 1), a.error, a.max_spin);
      s_abort = ok ? 0 : 1;
    }
    __syncthreads();
    if (s_abort) break;
    // 3. halo rows from the neighbours (the part inside both windows)
    {
      const int ulo = max(band.wlo, bu.wlo), uhi = min(band.whi, bu.whi);
      const int dlo = max(band.wlo, bd.wlo), dhi = min(band.whi, bd.whi);
      const int uw = up >= 0 ? max(0, (uhi - ulo) / 4) : 0, dw = dn < a.nbands ? max(0, (dhi - dlo) / 4) : 0;
      for (int idx = tid; idx < nch * (uw + dw); idx += kThreads) {
        const int ch = idx % nch, rest = idx / nch;
        const bool top = rest < uw;
        const int w = top ? rest : rest - uw;
        const int nb = top ? up : dn, which = top ? 1 : 0, col = (top ? ulo : dlo) + 4 * w;
        const uint8_t* g = a.xbuf + ((((size_t)slot * a.nbands + nb) * 2 + which) * nch + ch) * a.P + col;
        const uint32_t v = __ldcg(reinterpret_cast<const uint32_t*>(g));
        reinterpret_cast<uint32_t*>(sm.row(ch, t, top ? 0 : R - 1) + (col - band.wlo))[0] = v;
      }
    }
    __syncthreads();
    // 4. rebuild the passive colour 1-t of rows r0 .. r1-1: bit 1 from the site above (its
    //    bit 2), bit 2 from below (its bit 1), bit 4 from the left active neighbour (its 8),
    //    bit 8 from the right one (its 4); left/right are columns m-1/m or m/m+1 by (i+t).
    const int rows = R - 2;
    for (int idx = tid; idx < nch * rows * words; idx += kThreads) {
      const int w = idx % words, rest = idx / words, r = rest % rows, ch = rest / rows;
      const int ri = r + 1, i = band.r0 + r;
      const uint32_t* A0 = reinterpret_cast<const uint32_t*>(sm.row(ch, t, ri - 1));
      const uint32_t* A1 = reinterpret_cast<const uint32_t*>(sm.row(ch, t, ri));
      const uint32_t* A2 = reinterpret_cast<const uint32_t*>(sm.row(ch, t, ri + 1));
      uint32_t* Pw = reinterpret_cast<uint32_t*>(sm.row(ch, 1 - t, ri));
      const uint32_t cur = A1[w];
      const uint32_t prev = w > 0 ? A1[w - 1] : 0u, next = w + 1 < words ? A1[w + 1] : 0u;
      uint32_t left, right;
      if ((i + t) & 1) {  // left = m, right = m + 1
        left = cur;
        right = __funnelshift_r(cur, next, 8);
      } else {            // left = m - 1, right = m
        left = __funnelshift_l(prev, cur, 8);
        right = cur;
      }
      uint32_t v = ((A0[w] >> 1) & 0x01010101u) | ((A2[w] & 0x01010101u) << 1) | ((left & 0x08080808u) >> 1) |
                   ((right & 0x04040404u) << 1);
      // Kept as they are: the window's edge sites (they never change and lack a neighbour
      // here) and columns outside [1, cols], which the reference never rebuilds.
      uint32_t keep = 0;
      if (w == 0) keep |= 0x000000ffu;
      if (w == words - 1) keep |= 0xff000000u;
      const int c0 = band.wlo + 4 * w;
      if (c0 < 1) keep |= 0x000000ffu;
      if (c0 + 3 > a.cols) {
#pragma unroll
        for (int k4 = 0; k4 < 4; ++k4)
          if (c0 + k4 > a.cols) keep |= 0xffu << (8 * k4);
      }
      const uint32_t old = Pw[w];
      Pw[w] = (v & ~keep) | (old & keep);
    }
    __syncthreads();
  }

  // Write back the band rows of both colours and the generator states.
  for (int idx = tid; idx < nch * 2 * (R - 2) * words; idx += kThreads) {
    const int w = idx % words, rest = idx / words, r = rest % (R - 2), ct = rest / (R - 2);
    const int ch = ct >> 1, t = ct & 1;
    uint8_t* g = a.base + (size_t)ch * a.chain_stride + (size_t)t * a.colour_stride + (size_t)(band.r0 + r) * a.P +
                 band.wlo;
    reinterpret_cast<uint32_t*>(g)[w] = reinterpret_cast<const uint32_t*>(sm.row(ch, t, r + 1))[w];
  }
  if (kMode == RT_RNG_TINYMT) {
#pragma unroll
    for (int s = 0; s < K; ++s) {
      if (pos[s] == 0xffffffffu) continue;
      const int i = (int)(pos[s] >> 16), u = (int)(pos[s] & 0xffffu);
      a.tmt[(int64_t)(i - 1) * a.cols + (u - 1)] = st[s];
    }
  }
}

template <int kMode, bool kParams>
void* kernel_for(int K) {
  switch (K) {
    case 1: return (void*)k_persist<kMode, 1, kParams>;
    case 2: return (void*)k_persist<kMode, 2, kParams>;
    case 4: return (void*)k_persist<kMode, 4, kParams>;
    case 8: return (void*)k_persist<kMode, 8, kParams>;
  }
  return nullptr;
}

}  // namespace

// ---------------------------------------------------------------------------------------
// Host: partition and launch
// ---------------------------------------------------------------------------------------

bool dm_tiling_consistent(const int32_t* t, int N) {
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      const int32_t v = t[(size_t)i * N + j];
      if (i + 1 < N && ((v >> 1) & 1) != (t[(size_t)(i + 1) * N + j] & 1)) return false;
      if (j + 1 < N && ((v >> 3) & 1) != ((t[(size_t)i * N + j + 1] >> 2) & 1)) return false;
      if ((i == 0 && (v & 1)) || (i == N - 1 && (v & 2)) || (j == 0 && (v & 4)) || (j == N - 1 && (v & 8)))
        return false;
    }
  return true;
}

void dm_mark_candidates(const int32_t* t, int N, std::vector<uint8_t>& cand) {
  // Interior vertices (four covered squares), then the cells (i, m) holding one.
  const int M = N - 1, H = N / 2;
  std::vector<uint8_t> sq((size_t)M * M);
  for (int i = 0; i < M; ++i)
    for (int j = 0; j < M; ++j)
      sq[(size_t)i * M + j] = ((t[(size_t)i * N + j] & 10) != 0) || ((t[(size_t)(i + 1) * N + j + 1] & 5) != 0);
  if (cand.size() != (size_t)N * H) cand.assign((size_t)N * H, 0);
  for (int i = 1; i < M; ++i)
    for (int j = 1; j < M; ++j)
      if (sq[(size_t)(i - 1) * M + j - 1] && sq[(size_t)(i - 1) * M + j] && sq[(size_t)i * M + j - 1] &&
          sq[(size_t)i * M + j])
        cand[(size_t)i * H + j / 2] = 1;
}

rt_status PersistPlan::build(const std::vector<uint8_t>& cand, int N, int P, int mode, int nch, int nbands_max,
                             size_t smem_limit) {
  ok = false;
  why.clear();
  const int H = N / 2, cols = H - 2, rows = N - 2;
  row_lo.assign(N, 0);
  row_cnt.assign(N, 0);
  row_prefix.assign(N + 1, 0);
  std::vector<int> lo(N, -1), hi(N, -1);  // candidate column range per row (cells)
  for (int i = 1; i <= rows; ++i)
    for (int m = 1; m <= cols; ++m)
      if (cand[(size_t)i * H + m]) {
        if (lo[i] < 0) lo[i] = m;
        hi[i] = m;
      }
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
    while (r <= rows && (acc < target || r == bd.r0 || g == G - 1)) {
      if (acc >= target && r > bd.r0 && g < G - 1) break;
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
  // Row prefix (unit index of the first unit of each row within its band) and windows.
  max_units = 0;
  smem_bytes = 0;
  for (DmBand& bd : bands) {
    int u = 0, wl = P, wh = 0;
    for (int i = bd.r0; i < bd.r1; ++i) {
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
      wh = 4;
    }
    bd.wlo = std::max(0, wl) & ~3;
    bd.whi = std::min(P, (wh + 3) & ~3);
    max_units = std::max(max_units, bd.units);
    const size_t sb = (size_t)2 * nch * (bd.r1 - bd.r0 + 2) * (bd.whi - bd.wlo);
    smem_bytes = std::max(smem_bytes, sb);
  }
  K = 0;
  for (int k : {1, 2, 4, 8})
    if ((int64_t)k * kThreads >= max_units) {
      K = k;
      break;
    }
  if (K == 0) {
    why = "too many flip candidates per band for register-resident generators";
    return RT_OK;
  }
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
  if (d_bands) cudaFree(d_bands);
  if (d_rows) cudaFree(d_rows);
  if (d_xbuf) cudaFree(d_xbuf);
  if (d_flags) cudaFree(d_flags);
  if (d_colours) cudaFree(d_colours);
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
  if (rt_status st = plan.build(s.candidates, s.N, s.P, s.opts.rng_mode, s.active, sms, smem_optin)) return st;
  if (!plan.ok) return RT_OK;
  const bool params = s.tmt_params != nullptr;
  kernel = s.opts.rng_mode == RT_RNG_TINYMT
               ? (params ? kernel_for<RT_RNG_TINYMT, true>(plan.K) : kernel_for<RT_RNG_TINYMT, false>(plan.K))
               : kernel_for<RT_RNG_FAST, false>(plan.K);
  RT_CUDA_P(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)plan.smem_bytes));
  int per_sm = 0;
  RT_CUDA_P(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, plan.smem_bytes));
  if ((int64_t)per_sm * sms < (int64_t)plan.bands.size()) {
    plan.ok = false;
    plan.why = "bands cannot all be resident";
    return RT_OK;
  }
  // Device copies of the plan.
  if (d_bands) cudaFree(d_bands), d_bands = nullptr;
  if (d_rows) cudaFree(d_rows), d_rows = nullptr;
  if (d_xbuf) cudaFree(d_xbuf), d_xbuf = nullptr;
  if (d_flags) cudaFree(d_flags), d_flags = nullptr;
  RT_CUDA_P(cudaMalloc(&d_bands, plan.bands.size() * sizeof(DmBand)));
  RT_CUDA_P(cudaMalloc(&d_rows, 3 * (size_t)(s.N + 1) * sizeof(int)));
  std::vector<int> rows_host(3 * (size_t)(s.N + 1), 0);
  std::copy(plan.row_lo.begin(), plan.row_lo.end(), rows_host.begin());
  std::copy(plan.row_prefix.begin(), plan.row_prefix.end(), rows_host.begin() + (s.N + 1));
  RT_CUDA_P(cudaMemcpy(d_bands, plan.bands.data(), plan.bands.size() * sizeof(DmBand), cudaMemcpyHostToDevice));
  RT_CUDA_P(cudaMemcpy(d_rows, rows_host.data(), rows_host.size() * sizeof(int), cudaMemcpyHostToDevice));
  xbuf_bytes = (size_t)2 * plan.bands.size() * 2 * s.active * s.P;
  RT_CUDA_P(cudaMalloc(&d_xbuf, xbuf_bytes));
  RT_CUDA_P(cudaMalloc(&d_flags, (plan.bands.size() + 1) * sizeof(unsigned)));
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
    a.max_spin = 1L << 22;
    a.steps = n;
    a.h0 = h0 + done;
    a.fast_seed = fast_seed;
    a.fast_stream = s.opts.fast_stream;
    if (s.opts.rng_mode == RT_RNG_TINYMT) {
      if (colours_cap < n) {
        if (d_colours) cudaFree(d_colours);
        d_colours = nullptr;
        RT_CUDA_P(cudaMalloc(&d_colours, (size_t)n));
        colours_cap = n;
      }
      RT_CUDA_P(cudaMemcpyAsync(d_colours, colours_host + done, (size_t)n, cudaMemcpyHostToDevice, s.stream));
      a.colours = d_colours;
    }
    RT_CUDA_P(cudaMemsetAsync(d_flags, 0, (plan.bands.size() + 1) * sizeof(unsigned), s.stream));
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

void* dm_persist_kernel_ptr(int mode, int K, bool params) {
  if (mode == RT_RNG_TINYMT) return params ? kernel_for<RT_RNG_TINYMT, true>(K) : kernel_for<RT_RNG_TINYMT, false>(K);
  return kernel_for<RT_RNG_FAST, false>(K);
}

}  // namespace rt
