// The domino checkerboard sweep on the GPU: colour split/merge, per-half-sweep kernels,
// the sampler object behind the C ABI, and the walk / epoch / CFTP entry points.
//
// Device layout of one chain: two colour arrays, black (t = 1, (i + j) even) and white
// (t = 0), each N rows x P bytes (P = N/2 rounded up to 16; column m of row i holds vertex
// (i, 2m + ((i + 1 - t) & 1))), one uint8 edge mask per vertex as in the reference
// (DominoTiler.cpp:24-33).  Chains of a sampler are consecutive; all see one random stream.
// Site (i, m) for i in [1, N-2], m in [1, N/2-2] is a flip candidate; its TinyMT generator
// is number (i-1)*(N/2-2) + (m-1), the reference's work-item order (tinymt.clh:24).
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstring>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "domino_rules.h"
#include "domino_sweep.h"
#include "pdl.cuh"
#include "rng.cuh"
#include "rt_internal.h"

namespace rt {

// -----------------------------------------------------------------------------------------
// Kernels
// -----------------------------------------------------------------------------------------

__global__ void k_tmt_seed(uint4* st, const uint4* params, int64_t count, uint32_t seed) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  uint32_t m1 = kTmtMat1, m2 = kTmtMat2, tm = kTmtTmat;
  if (params) {
    uint4 p = params[k];
    m1 = p.x; m2 = p.y; tm = p.z;
  }
  st[k] = tmt_seed(seed + (uint32_t)k, m1, m2, tm);
}

// One half-sweep's rotation, TinyMT mode: every generator of the grid advances once (as
// the reference's NDRange does) and the draw decides the flip of site (i, m) of colour t
// in every chain.
template <bool kParams>
__global__ void k_rotate_tmt(DmView v, int t, DmRule rule) {
  pdl_begin();
  const int m = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int i = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (m > v.cols || i > v.rows) return;
  const int64_t k = (int64_t)(i - 1) * v.cols + (m - 1);
  uint32_t m1 = kTmtMat1, m2 = kTmtMat2, tm = kTmtTmat;
  if (kParams) {
    uint4 p = v.tmt_params[k];
    m1 = p.x; m2 = p.y; tm = p.z;
  }
  uint4 s = v.tmt[k];
  const uint32_t u = tmt_next_u23(s, m1, m2, tm);
  v.tmt[k] = s;
  const int c = (i & 1) | (t << 1);
  const uint32_t lo_up = rule.lo_up[c], w_up = rule.w_up[c], lo_dn = rule.lo_dn[c], w_dn = rule.w_dn[c];
  for (int ch = 0; ch < v.active; ++ch) {
    uint8_t* A = v.colour(ch, t);
    const size_t off = (size_t)i * v.P + m;
    const uint32_t e = A[off];
    const uint8_t n = dm_flip(e, u, lo_up, w_up, lo_dn, w_dn);
    if (n != e) A[off] = n;
  }
}

// Fast mode: one Philox call per column quad of a row gives the draws of its four sites.
__global__ void k_rotate_fast(DmView v, int t, DmRule rule, uint64_t seed, uint32_t stream, int64_t h) {
  pdl_begin();
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (4 * q > v.cols || i > v.rows) return;
  const uint4 r = fast_quad(seed, stream, h, (uint32_t)i, (uint32_t)q);
  const uint32_t u4[4] = {r.x, r.y, r.z, r.w};
  const int c = (i & 1) | (t << 1);
  const uint32_t lo_up = rule.lo_up[c], w_up = rule.w_up[c], lo_dn = rule.lo_dn[c], w_dn = rule.w_dn[c];
  for (int ch = 0; ch < v.active; ++ch) {
    uint32_t* word = reinterpret_cast<uint32_t*>(v.colour(ch, t) + (size_t)i * v.P) + q;  // columns 4q..4q+3
    const uint32_t e4 = *word;
    uint32_t n4 = e4;
#pragma unroll
    for (int r4 = 0; r4 < 4; ++r4) {
      const int m = 4 * q + r4;
      if (m < 1 || m > v.cols) continue;
      const uint32_t e = (e4 >> (8 * r4)) & 0xffu;
      n4 ^= (e ^ dm_flip(e, u4[r4], lo_up, w_up, lo_dn, w_dn)) << (8 * r4);
    }
    if (n4 != e4) *word = n4;
  }
}

// The passive colour rebuilt from the active one (dominokernel.cl:22-31): passive site
// (i, m) takes its up edge from the site above's down edge (bit 2 -> 1), its down edge from
// below's up edge (1 -> 2) and its two horizontal edges from the active sites left (8 -> 4)
// and right (4 -> 8) of it, at columns m, m+1 when i + t is odd and m-1, m otherwise.
// Four sites at a time: thread (w, i) rewrites 32-bit word w (columns 4w..4w+3) of passive
// row i from the active rows i-1, i, i+1; a neighbour one column over is a funnel shift of
// two adjacent words.  Columns outside [1, cols] keep their value, as the reference rebuilds
// only those sites.
__global__ void k_update_w(DmView v, int t) {
  pdl_begin();
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int words = v.P / 4;
  if (w >= words || i > v.rows) return;
  uint32_t keep = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int m = 4 * w + k;
    if (m < 1 || m > v.cols) keep |= 0xffu << (8 * k);
  }
  if (keep == 0xffffffffu) return;
  const bool odd = ((i + t) & 1) != 0;  // left / right neighbours at columns m, m+1 (else m-1, m)
  for (int ch = 0; ch < v.active; ++ch) {
    const uint32_t* A = reinterpret_cast<const uint32_t*>(v.colour(ch, t) + (size_t)i * v.P);
    uint32_t* Pw = reinterpret_cast<uint32_t*>(v.colour(ch, 1 - t) + (size_t)i * v.P) + w;
    const uint32_t cur = A[w], up = A[w - words], dn = A[w + words];
    uint32_t left, right;
    if (odd) {
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

// Scan of a host-layout tiling in device memory: flags bit 0 a value outside [0, 15], bit 1
// an edge whose two endpoints disagree (or leaves the array); each colour-array row's
// lowest/highest flip-candidate column (interior vertices: four covered squares around
// them, columns 1 .. N/2 - 2); with `interior`, the interior vertices of each colour.
__global__ void k_scan_tiling(const int32_t* t, int N, int* cand, unsigned long long* scan, int count_interior) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y, lane = threadIdx.x & 31;
  unsigned f = 0;
  int lo = INT_MAX, hi = -1;
  bool inter = false;
  if (j < N) {
    const int32_t v = t[(size_t)i * N + j];
    if ((uint32_t)v > 15u) f |= 1u;
    if (i + 1 < N && ((v >> 1) & 1) != (t[(size_t)(i + 1) * N + j] & 1)) f |= 2u;
    if (j + 1 < N && ((v >> 3) & 1) != ((t[(size_t)i * N + j + 1] >> 2) & 1)) f |= 2u;
    if ((i == 0 && (v & 1)) || (i == N - 1 && (v & 2)) || (j == 0 && (v & 4)) || (j == N - 1 && (v & 8))) f |= 2u;
    const int M = N - 1;
    if (i >= 1 && i <= M - 1 && j >= 1 && j <= M - 1) {
      auto sq = [&](int a, int b) {
        return ((t[(size_t)a * N + b] & 10) != 0) || ((t[(size_t)(a + 1) * N + b + 1] & 5) != 0);
      };
      inter = sq(i - 1, j - 1) && sq(i - 1, j) && sq(i, j - 1) && sq(i, j);
      const int m = j >> 1;
      if (inter && m >= 1 && m <= N / 2 - 2) {
        lo = hi = m;
        // A neighbour outside rows 1 .. N-2 or columns 1 .. N/2-2: a cell the reference never
        // rebuilds, which only the byte engines reproduce.
        if (i < 2 || i > N - 3 || ((j - 1) >> 1) < 1 || ((j + 1) >> 1) > N / 2 - 2) f |= 4u;
      }
    }
  }
  f = __reduce_or_sync(0xffffffffu, f);
  lo = __reduce_min_sync(0xffffffffu, lo);
  hi = __reduce_max_sync(0xffffffffu, hi);
  const unsigned black = __ballot_sync(0xffffffffu, inter && ((i + j) & 1) == 0);
  const unsigned white = __ballot_sync(0xffffffffu, inter && ((i + j) & 1) == 1);
  if (lane == 0) {
    if (f) atomicOr(reinterpret_cast<unsigned*>(&scan[0]), f);
    if (lo != INT_MAX) atomicMin(&cand[i], lo);
    if (hi >= 0) atomicMax(&cand[N + i], hi);
    if (count_interior) {
      if (white) atomicAdd(&scan[1], (unsigned long long)__popc(white));
      if (black) atomicAdd(&scan[2], (unsigned long long)__popc(black));
    }
  }
}

// Host-layout int32 tiling (N x N) <-> colour arrays of one chain.
__global__ void k_split(DmView v, int ch, const int32_t* tiling) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  if (j >= v.N) return;
  const int t = ((i + j) & 1) == 0 ? 1 : 0;
  v.colour(ch, t)[(size_t)i * v.P + (j >> 1)] = (uint8_t)tiling[(size_t)i * v.N + j];
}

__global__ void k_merge(DmView v, int ch, int32_t* tiling) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  if (j >= v.N) return;
  const int t = ((i + j) & 1) == 0 ? 1 : 0;
  tiling[(size_t)i * v.N + j] = v.colour(ch, t)[(size_t)i * v.P + (j >> 1)];
}

// Edge-placement counters of chain ch, layout [2][N][N]: [0][i][j] counts bit 2 of vertex
// (i, j) (the lattice edge to (i+1, j) lies inside a domino: a horizontal domino on faces
// (i, j-1) and (i, j)), [1][i][j] counts bit 8 (the edge to (i, j+1) inside a vertical domino
// on faces (i-1, j) and (i, j)).  One thread per vertex owns its two counters.
__global__ void k_acc_edges(DmView v, int ch, uint32_t* counts) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
  if (j >= v.N) return;
  const int t = ((i + j) & 1) == 0 ? 1 : 0;
  const uint8_t e = v.colour(ch, t)[(size_t)i * v.P + (j >> 1)];
  const size_t k = (size_t)i * v.N + j;
  if (e & 2) counts[k] += 1u;
  if (e & 8) counts[(size_t)v.N * v.N + k] += 1u;
}

// Sites where chains a and b differ: per 4-byte word, XOR then count the non-zero bytes
// (masks are < 16, so byte b is non-zero iff bit 4 of (b + 15) is set).
__global__ void k_diff(DmView v, int a, int b, unsigned long long* out) {
  const size_t words = (size_t)v.chain_stride / 4;
  const uint32_t* x = reinterpret_cast<const uint32_t*>(v.base + (size_t)a * v.chain_stride);
  const uint32_t* y = reinterpret_cast<const uint32_t*>(v.base + (size_t)b * v.chain_stride);
  unsigned long long local = 0;
  for (size_t w = (size_t)blockIdx.x * blockDim.x + threadIdx.x; w < words; w += (size_t)gridDim.x * blockDim.x) {
    uint32_t d = (x[w] ^ y[w]) & 0x0f0f0f0fu;
    local += __popc((d + 0x0f0f0f0fu) & 0x10101010u);
  }
  for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
  if ((threadIdx.x & 31) == 0 && local) atomicAdd(out, local);
}

// -----------------------------------------------------------------------------------------
// Sampler
// -----------------------------------------------------------------------------------------

#define RT_CUDA(expr)                                                                   \
  do {                                                                                  \
    cudaError_t _e = (expr);                                                            \
    if (_e != cudaSuccess)                                                              \
      return fail(RT_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e));     \
  } while (0)

DmSampler::~DmSampler() {
  bits.reset();  // the engines free their plan buffers on the stream before the stream goes
  runs.reset();
  persist.reset();
  for (void* p : {(void*)tmt, (void*)tmt_params, mtgp, (void*)base, (void*)scratch, (void*)counter, (void*)d_scan,
                  (void*)d_cand})
    dev_free(p, stream);
  for (void* p : {(void*)d_dom, (void*)d_cls, (void*)d_h, (void*)d_hflags})
    if (p) cudaFree(p);
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
  if (own_stream && stream) cudaStreamDestroy(stream);
}

DmView DmSampler::view() const {
  DmView v;
  v.base = base;
  v.N = N;
  v.P = P;
  v.rows = N - 2;
  v.cols = N / 2 - 2;
  v.active = active;
  v.chain_stride = chain_stride;
  v.colour_stride = colour_stride;
  v.tmt = tmt;
  v.tmt_params = tmt_params;
  return v;
}

rt_status DmSampler::create(int n_side, int n_chains, const rt_walk_opts& o, std::unique_ptr<DmSampler>* out) {
  if (n_side < 6 || n_side % 2) return fail(RT_ERR_INVALID_ARGUMENT, "tiling side must be even and >= 6");
  if (n_side > 32768) return fail(RT_ERR_INVALID_ARGUMENT, "tiling side must be <= 32768");
  if (n_chains < 1 || n_chains > 64) return fail(RT_ERR_INVALID_ARGUMENT, "n_chains must be in [1, 64]");
  if (o.engine < 0 || o.engine > 4) return fail(RT_ERR_INVALID_ARGUMENT, "engine must be 0, 1, 2, 3 or 4");
  if (o.rng_mode == RT_RNG_FAST && o.fast_stream >= 65536u)
    return fail(RT_ERR_INVALID_ARGUMENT, "fast_stream must be < 65536");
  DmRule rule{};
  const char* err = nullptr;
  if (!dm_rule_build(o.rule, o.rng_mode, o.weight_a, o.weight_b, &rule, &err)) return fail(RT_ERR_INVALID_ARGUMENT, err);
  if (o.tinymt_params && o.tinymt_params_count < 0) return fail(RT_ERR_INVALID_ARGUMENT, "negative parameter count");
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) {
    cudaGetLastError();
    return fail(RT_ERR_CUDA, "no CUDA device: the sweep has no CPU fallback");
  }
  auto s = std::make_unique<DmSampler>();
  s->N = n_side;
  s->P = ((n_side / 2) + 15) / 16 * 16;
  s->n_chains = n_chains;
  s->active = n_chains;
  s->opts = o;
  s->rule = rule;
  s->colour_stride = (size_t)s->N * s->P;
  s->chain_stride = 2 * s->colour_stride;
  if (o.cuda_stream) {
    s->stream = (cudaStream_t)o.cuda_stream;
  } else {
    RT_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    s->own_stream = true;
  }
  RT_CUDA(cudaEventCreate(&s->ev0));
  RT_CUDA(cudaEventCreate(&s->ev1));
  // Pool allocations, ordered on the sampler's stream (device_pool.cpp).
  if (rt_status st = dev_alloc(&s->base, s->chain_stride * n_chains, s->stream)) return st;
  RT_CUDA(cudaMemsetAsync(s->base, 0, s->chain_stride * n_chains, s->stream));
  if (rt_status st = dev_alloc(&s->scratch, (size_t)s->N * s->N * sizeof(int32_t), s->stream)) return st;
  if (rt_status st = dev_alloc(&s->counter, sizeof(unsigned long long), s->stream)) return st;
  if (rt_status st = dev_alloc(&s->d_scan, 3 * sizeof(unsigned long long), s->stream)) return st;
  if (rt_status st = dev_alloc(&s->d_cand, 2 * (size_t)s->N * sizeof(int), s->stream)) return st;
  {
    std::vector<int> init(2 * (size_t)s->N, -1);
    std::fill(init.begin(), init.begin() + s->N, INT_MAX);
    RT_CUDA(cudaMemcpyAsync(s->d_cand, init.data(), init.size() * sizeof(int), cudaMemcpyHostToDevice, s->stream));
    RT_CUDA(cudaStreamSynchronize(s->stream));
  }
  const int64_t cells = (int64_t)(s->N - 2) * (s->N / 2 - 2);
  if (o.rng_mode == RT_RNG_TINYMT) {
    if (rt_status st = dev_alloc(&s->tmt, cells * sizeof(uint4), s->stream)) return st;
    if (o.tinymt_params) {
      // Generators beyond the table keep the default set, as the oracle does.
      std::vector<uint4> p((size_t)cells);
      for (int64_t k = 0; k < cells; ++k) {
        if (k < o.tinymt_params_count)
          p[k] = make_uint4(o.tinymt_params[3 * k], o.tinymt_params[3 * k + 1], o.tinymt_params[3 * k + 2], 0);
        else
          p[k] = make_uint4(kTmtMat1, kTmtMat2, kTmtTmat, 0);
      }
      if (rt_status st = dev_alloc(&s->tmt_params, cells * sizeof(uint4), s->stream)) return st;
      RT_CUDA(cudaMemcpyAsync(s->tmt_params, p.data(), cells * sizeof(uint4), cudaMemcpyHostToDevice, s->stream));
      RT_CUDA(cudaStreamSynchronize(s->stream));
    }
  } else if (o.rng_mode == RT_RNG_MTGP) {
    if (o.engine >= 2) return fail(RT_ERR_INVALID_ARGUMENT, "MTGP mode runs on the per-half-sweep kernels only");
    if (rt_status st = dev_alloc(&s->mtgp, mtgp_state_bytes(mtgp_grid(s->N - 2, s->N / 2 - 2).count()), s->stream))
      return st;
  }
  *out = std::move(s);
  return RT_OK;
}

rt_status DmSampler::check_launch() {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(RT_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  return RT_OK;
}

rt_status DmSampler::load(int ch, const int32_t* tiling) {
  if (ch < 0 || ch >= n_chains || !tiling) return fail(RT_ERR_INVALID_ARGUMENT, "load: bad chain or NULL tiling");
  // The scan runs on the device copy: value range, consistency, flip candidates and (chain
  // 0) the interior vertices per colour, which count the flip attempts of a half-sweep.
  RT_CUDA(cudaMemcpyAsync(scratch, tiling, (size_t)N * N * sizeof(int32_t), cudaMemcpyHostToDevice, stream));
  RT_CUDA(cudaMemsetAsync(d_scan, 0, 3 * sizeof(unsigned long long), stream));
  k_scan_tiling<<<dim3((N + 255) / 256, N), 256, 0, stream>>>(scratch, N, d_cand, d_scan, ch == 0);
  launches++;
  unsigned long long h[3] = {0, 0, 0};
  RT_CUDA(cudaMemcpyAsync(h, d_scan, sizeof h, cudaMemcpyDeviceToHost, stream));
  RT_CUDA(cudaStreamSynchronize(stream));
  if (h[0] & 1u) return fail(RT_ERR_INVALID_ARGUMENT, "tiling values must be edge masks in [0, 15]");
  consistent = consistent && !(h[0] & 2u);
  border_candidates = border_candidates || (h[0] & 4u);
  if (ch == 0) {
    interior[0] = (int64_t)h[1];
    interior[1] = (int64_t)h[2];
  }
  plan_dirty = true;
  DmView v = view();
  k_split<<<dim3((N + 255) / 256, N), 256, 0, stream>>>(v, ch, scratch);
  launches++;
  return check_launch();
}

rt_status DmSampler::fetch_candidates() {
  std::vector<int> both(2 * (size_t)N);
  RT_CUDA(cudaMemcpyAsync(both.data(), d_cand, both.size() * sizeof(int), cudaMemcpyDeviceToHost, stream));
  RT_CUDA(cudaStreamSynchronize(stream));
  cand_lo.assign(N, -1);
  cand_hi.assign(N, -1);
  any_candidate = false;
  for (int i = 0; i < N; ++i)
    if (both[i] != INT_MAX) {
      cand_lo[i] = both[i];
      cand_hi[i] = both[N + i];
      any_candidate = true;
    }
  return RT_OK;
}

rt_status DmSampler::store(int ch, int32_t* tiling) {
  if (ch < 0 || ch >= n_chains || !tiling) return fail(RT_ERR_INVALID_ARGUMENT, "store: bad chain or NULL tiling");
  if (rt_status st = check_resident_error()) return st;
  DmView v = view();
  k_merge<<<dim3((N + 255) / 256, N), 256, 0, stream>>>(v, ch, scratch);
  launches++;
  if (rt_status s = check_launch()) return s;
  RT_CUDA(cudaMemcpyAsync(tiling, scratch, (size_t)N * N * sizeof(int32_t), cudaMemcpyDeviceToHost, stream));
  RT_CUDA(cudaStreamSynchronize(stream));
  return RT_OK;
}

rt_status DmSampler::copy_chain(int dst, int src) {
  if (dst < 0 || src < 0 || dst >= n_chains || src >= n_chains) return fail(RT_ERR_INVALID_ARGUMENT, "copy_chain: bad chain");
  if (dst == src) return RT_OK;
  RT_CUDA(cudaMemcpyAsync(base + (size_t)dst * chain_stride, base + (size_t)src * chain_stride, chain_stride,
                          cudaMemcpyDeviceToDevice, stream));
  return RT_OK;
}

rt_status DmSampler::seed(int64_t s) {
  if (opts.rng_mode == RT_RNG_MTGP) {
    if (rt_status st = mtgp_seed(mtgp, mtgp_grid(N - 2, N / 2 - 2).count(), s, stream)) return st;
    mtgp_seeded = true;
    return RT_OK;
  }
  if (opts.rng_mode != RT_RNG_TINYMT) return fail(RT_ERR_INVALID_ARGUMENT, "seed: sampler is not in TinyMT or MTGP mode");
  const int64_t cells = (int64_t)(N - 2) * (N / 2 - 2);
  k_tmt_seed<<<(unsigned)((cells + 255) / 256), 256, 0, stream>>>(tmt, tmt_params, cells, (uint32_t)s);
  launches++;
  return check_launch();
}

rt_status DmSampler::run(const uint8_t* colours, int64_t steps) {
  if (opts.rng_mode == RT_RNG_FAST) return fail(RT_ERR_INVALID_ARGUMENT, "run: sampler is in fast mode (run_fast)");
  if (steps < 0 || (steps > 0 && !colours)) return fail(RT_ERR_INVALID_ARGUMENT, "run: bad colours / steps");
  if (steps == 0) return RT_OK;
  if (opts.rng_mode == RT_RNG_MTGP) {
    // An MTGP state holds a pointer to its parameters: none exists before the first seed.
    if (!mtgp_seeded) return fail(RT_ERR_INVALID_ARGUMENT, "run: MTGP generators not seeded");
    last_engine = 1;
    DmView v = view();
    const dim3 blk_w(32, 8), grd_w((v.P / 4 + 31) / 32, (v.rows + 7) / 8);
    for (int64_t q = 0; q < steps; ++q) {
      const int t = colours[q] ? 1 : 0;
      if (rt_status st = mtgp_rotate(v, t, rule, mtgp, stream)) return st;
      pdl_launch(k_update_w, grd_w, blk_w, stream, v, t);
      launches += 2;
      half_sweeps[t]++;
    }
    return check_launch();
  }
  bool pers = false;
  if (rt_status st = use_persistent(&pers)) return st;
  if (pers) {
    last_engine = resident;
    for (int64_t q = 0; q < steps; ++q) half_sweeps[colours[q] ? 1 : 0]++;
    return launch_resident(colours, steps, 0, 0);
  }
  last_engine = 1;
  DmView v = view();
  const dim3 blk(128, 2), grd((v.cols + 127) / 128, (v.rows + 1) / 2);
  const dim3 blk_w(32, 8), grd_w((v.P / 4 + 31) / 32, (v.rows + 7) / 8);
  for (int64_t s = 0; s < steps; ++s) {
    const int t = colours[s] ? 1 : 0;
    if (tmt_params) pdl_launch(k_rotate_tmt<true>, grd, blk, stream, v, t, rule);
    else pdl_launch(k_rotate_tmt<false>, grd, blk, stream, v, t, rule);
    pdl_launch(k_update_w, grd_w, blk_w, stream, v, t);
    launches += 2;
    half_sweeps[t]++;
  }
  return check_launch();
}

rt_status DmSampler::run_fast(uint64_t seed_value, int64_t h0, int64_t steps) {
  if (opts.rng_mode != RT_RNG_FAST) return fail(RT_ERR_INVALID_ARGUMENT, "run_fast: sampler is not in fast mode");
  if (steps < 0) return fail(RT_ERR_INVALID_ARGUMENT, "run_fast: negative steps");
  const int64_t lim = (int64_t)1 << 47;
  if (h0 < -lim || h0 + steps > lim) return fail(RT_ERR_INVALID_ARGUMENT, "run_fast: half-sweep index out of range");
  if (steps == 0) return RT_OK;
  bool pers = false;
  if (rt_status st = use_persistent(&pers)) return st;
  if (pers) {
    last_engine = resident;
    for (int64_t q = 0; q < steps; ++q) half_sweeps[((h0 + q) & 1) ? 0 : 1]++;
    return launch_resident(nullptr, steps, seed_value, h0);
  }
  last_engine = 1;
  DmView v = view();
  const int quads = v.cols / 4 + 1;
  const dim3 blk(64, 4), grd_r((quads + 63) / 64, (v.rows + 3) / 4);
  const dim3 blk_u(32, 8), grd_u((v.P / 4 + 31) / 32, (v.rows + 7) / 8);
  for (int64_t s = 0; s < steps; ++s) {
    const int64_t h = h0 + s;
    const int t = (h & 1) ? 0 : 1;
    pdl_launch(k_rotate_fast, grd_r, blk, stream, v, t, rule, seed_value, opts.fast_stream, h);
    pdl_launch(k_update_w, grd_u, blk_u, stream, v, t);
    launches += 2;
    half_sweeps[t]++;
  }
  return check_launch();
}

rt_status DmSampler::diff(int a, int b, int64_t* ndiff) {
  if (a < 0 || b < 0 || a >= n_chains || b >= n_chains || !ndiff) return fail(RT_ERR_INVALID_ARGUMENT, "diff: bad arguments");
  RT_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), stream));
  DmView v = view();
  const size_t words = chain_stride / 4;
  const unsigned blocks = (unsigned)std::min<size_t>((words + 255) / 256, 1024);
  k_diff<<<blocks, 256, 0, stream>>>(v, a, b, counter);
  launches++;
  if (rt_status s = check_launch()) return s;
  if (rt_status st = check_resident_error()) return st;
  unsigned long long h = 0;
  RT_CUDA(cudaMemcpyAsync(&h, counter, sizeof h, cudaMemcpyDeviceToHost, stream));
  RT_CUDA(cudaStreamSynchronize(stream));
  *ndiff = (int64_t)h;
  return RT_OK;
}

rt_status DmSampler::accumulate_edges(int ch, uint32_t* counts) {
  if (ch < 0 || ch >= n_chains || !counts) return fail(RT_ERR_INVALID_ARGUMENT, "accumulate_edges: bad arguments");
  DmView v = view();
  k_acc_edges<<<dim3((N + 255) / 256, N), 256, 0, stream>>>(v, ch, counts);
  launches++;
  return check_launch();
}

rt_status DmSampler::set_domain(const int32_t* domain, int m_side) {
  if (!domain || m_side != N - 1) return fail(RT_ERR_INVALID_ARGUMENT, "set_domain: the domain must be (N-1) x (N-1)");
  const int M = m_side;
  for (int i = 0; i < M; ++i)
    for (int j = 0; j < M; ++j)
      if ((i < 1 || j < 1 || i >= M - 1 || j >= M - 1) && domain[(size_t)i * M + j])
        return fail(RT_ERR_INVALID_ARGUMENT, "domain must have an empty outer ring of squares");
  hf_start = dm_first_boundary_vertex(domain, M);
  if (hf_start < 0) return fail(RT_ERR_INVALID_ARGUMENT, "set_domain: empty domain");
  const size_t NN = (size_t)N * N;
  if (!d_dom) {
    RT_CUDA(cudaMalloc(&d_dom, (size_t)M * M * sizeof(int32_t)));
    RT_CUDA(cudaMalloc(&d_cls, NN * sizeof(int32_t)));
    RT_CUDA(cudaMalloc(&d_h, NN * sizeof(int32_t)));
    RT_CUDA(cudaMalloc(&d_hflags, 16 * sizeof(unsigned)));
  }
  RT_CUDA(cudaMemcpyAsync(d_dom, domain, (size_t)M * M * sizeof(int32_t), cudaMemcpyHostToDevice, stream));
  RT_CUDA(cudaMemsetAsync(d_hflags, 0, 16 * sizeof(unsigned), stream));
  if (rt_status st = dm_classes_device(d_dom, M, d_cls, d_hflags + 8, stream)) return st;
  RT_CUDA(cudaStreamSynchronize(stream));
  return RT_OK;
}

rt_status DmSampler::accumulate_heights(int ch, long long* sums, int32_t* heights) {
  if (ch < 0 || ch >= n_chains || (!sums && !heights)) return fail(RT_ERR_INVALID_ARGUMENT, "accumulate_heights: bad arguments");
  if (!d_dom) return fail(RT_ERR_INVALID_ARGUMENT, "accumulate_heights: set the domain first (rt_dm_sampler_set_domain)");
  DmView v = view();
  k_merge<<<dim3((N + 255) / 256, N), 256, 0, stream>>>(v, ch, scratch);
  launches++;
  if (rt_status st = check_launch()) return st;
  if (rt_status st = dm_heights_device(scratch, d_cls, d_dom, N, hf_start, d_h, d_hflags, stream)) return st;
  if (sums) {
    if (rt_status st = dm_heights_accumulate(d_h, N, sums, stream)) return st;
  }
  if (heights) RT_CUDA(cudaMemcpyAsync(heights, d_h, (size_t)N * N * sizeof(int32_t), cudaMemcpyDeviceToDevice, stream));
  return RT_OK;
}

rt_status DmSampler::sync() {
  RT_CUDA(cudaStreamSynchronize(stream));
  return check_resident_error();
}

rt_status DmSampler::use_persistent(bool* yes) {
  *yes = false;
  resident = 0;
  // The engine: opts.engine when set, else the sampler's explicit launch shape, else the
  // autotuner's entry for this side, chain count and mode, else automatic.
  int engine = opts.engine;
  const bool explicit_engine = engine != 0 || launch_engine != 0;
  eff_bands = launch_bands;
  eff_threads = launch_threads;
  tuned = false;
  if (engine == 0 && launch_engine != 0) {
    engine = launch_engine;
  } else if (engine == 0 && launch_bands == 0 && launch_threads == 0) {
    int e = 0, b = 0, t = 0;
    if (tune_lookup(RT_MODEL_DOMINO, N, active, opts.rng_mode, &e, &b, &t)) {
      engine = e;
      eff_bands = b;
      eff_threads = t;
      tuned = true;
    }
  }
  if (engine == 1 || opts.rng_mode == RT_RNG_MTGP) return RT_OK;
  if (plan_dirty) {
    if (rt_status st = fetch_candidates()) return st;
  }
  if (!consistent || !any_candidate) {
    if (engine >= 2 && explicit_engine)
      return fail(RT_ERR_INVALID_ARGUMENT, "persistent engine needs consistent loaded tilings");
    return RT_OK;
  }
  // Engine 0: the bit-plane kernel, else the run kernel, else k_persist; 4: the bit-plane
  // kernel alone; 2: the run kernel, else k_persist; 3: k_persist alone.
  if (plan_dirty ||
      (runs && (runs->nch != active || runs->bands_asked != eff_bands || runs->threads_asked != eff_threads)) ||
      (persist && persist->nch != active) || (bits && bits->nch != active)) {
    bits.reset();
    runs.reset();
    persist.reset();
  }
  plan_dirty = false;
  std::string why;
  if (engine == 0 || engine == 4) {
    if (!bits) {
      bits = std::make_unique<BitEngine>();
      if (rt_status st = bits->prepare(*this)) return st;
    }
    if (bits->ready) {
      resident = 4;
      *yes = true;
      return RT_OK;
    }
    if (engine == 4 && explicit_engine)
      return fail(RT_ERR_INVALID_ARGUMENT, "bit-plane engine unavailable: " + bits->plan.why);
    why = "bit-plane kernel: " + bits->plan.why + "; ";
  }
  if (engine != 3) {
    if (!runs) {
      runs = std::make_unique<RunEngine>();
      if (rt_status st = runs->prepare(*this)) return st;
    }
    if (runs->ready) {
      resident = 2;
      *yes = true;
      return RT_OK;
    }
    why += "run kernel: " + runs->plan.why + "; ";
  }
  if (!persist) {
    persist = std::make_unique<PersistEngine>();
    if (rt_status st = persist->prepare(*this)) return st;
  }
  if (persist->ready) {
    resident = 3;
    *yes = true;
    return RT_OK;
  }
  if (engine >= 2 && explicit_engine)
    return fail(RT_ERR_INVALID_ARGUMENT, "persistent engine unavailable: " + why + "k_persist: " + persist->plan.why);
  return RT_OK;
}

rt_status DmSampler::check_resident_error() {
  if (bits) {
    if (rt_status st = bits->check_error(*this)) return st;
  }
  if (runs) {
    if (rt_status st = runs->check_error(*this)) return st;
  }
  if (persist) {
    if (rt_status st = persist->check_error(*this)) return st;
  }
  return RT_OK;
}

rt_status DmSampler::launch_resident(const uint8_t* colours, int64_t steps, uint64_t fast_seed, int64_t h0) {
  if (resident == 4) return bits->launch(*this, colours, steps);
  if (resident == 2) return runs->launch(*this, colours, steps, fast_seed, h0);
  return persist->launch(*this, colours, steps, fast_seed, h0);
}

}  // namespace rt

// -----------------------------------------------------------------------------------------
// C ABI
// -----------------------------------------------------------------------------------------
using namespace rt;

struct rt_dm_sampler {
  std::unique_ptr<DmSampler> impl;
};

static rt_walk_opts opts_or_default(const rt_walk_opts* o) {
  rt_walk_opts d;
  rt_walk_opts_default(&d);
  return o ? *o : d;
}

extern "C" {

RT_API rt_status rt_dm_sampler_create(int32_t n_side, int32_t n_chains, const rt_walk_opts* opts, rt_dm_sampler** out) {
  clear_error();
  if (!out) return fail(RT_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  auto h = std::make_unique<rt_dm_sampler>();
  if (rt_status s = DmSampler::create(n_side, n_chains, opts_or_default(opts), &h->impl)) return s;
  *out = h.release();
  return RT_OK;
}

RT_API rt_status rt_dm_sampler_destroy(rt_dm_sampler* s) {
  clear_error();
  delete s;
  return RT_OK;
}

#define RT_SAMPLER(s) \
  clear_error();      \
  if (!(s) || !(s)->impl) return fail(RT_ERR_INVALID_ARGUMENT, "sampler is NULL")

RT_API rt_status rt_dm_sampler_load(rt_dm_sampler* s, int32_t chain, const int32_t* tiling) {
  RT_SAMPLER(s);
  return s->impl->load(chain, tiling);
}
RT_API rt_status rt_dm_sampler_store(rt_dm_sampler* s, int32_t chain, int32_t* tiling) {
  RT_SAMPLER(s);
  return s->impl->store(chain, tiling);
}
RT_API rt_status rt_dm_sampler_copy_chain(rt_dm_sampler* s, int32_t dst, int32_t src) {
  RT_SAMPLER(s);
  return s->impl->copy_chain(dst, src);
}
RT_API rt_status rt_dm_sampler_set_active(rt_dm_sampler* s, int32_t k) {
  RT_SAMPLER(s);
  if (k < 1 || k > s->impl->n_chains) return fail(RT_ERR_INVALID_ARGUMENT, "set_active: k must be in [1, n_chains]");
  s->impl->active = k;
  s->impl->plan_dirty = true;
  return RT_OK;
}
RT_API rt_status rt_dm_sampler_seed(rt_dm_sampler* s, uint32_t seed) {
  RT_SAMPLER(s);
  return s->impl->seed(seed);
}
RT_API rt_status rt_dm_sampler_run(rt_dm_sampler* s, const uint8_t* colours, int64_t steps) {
  RT_SAMPLER(s);
  return s->impl->run(colours, steps);
}
RT_API rt_status rt_dm_sampler_run_fast(rt_dm_sampler* s, uint64_t seed, int64_t h0, int64_t steps) {
  RT_SAMPLER(s);
  return s->impl->run_fast(seed, h0, steps);
}
RT_API rt_status rt_dm_sampler_diff(rt_dm_sampler* s, int32_t a, int32_t b, int64_t* ndiff) {
  RT_SAMPLER(s);
  return s->impl->diff(a, b, ndiff);
}
RT_API rt_status rt_dm_sampler_accumulate_edges(rt_dm_sampler* s, int32_t chain, uint32_t* counts_device) {
  RT_SAMPLER(s);
  return s->impl->accumulate_edges(chain, counts_device);
}
RT_API rt_status rt_dm_sampler_set_domain(rt_dm_sampler* s, const int32_t* domain, int32_t m_side) {
  RT_SAMPLER(s);
  return s->impl->set_domain(domain, m_side);
}
RT_API rt_status rt_dm_sampler_accumulate_heights(rt_dm_sampler* s, int32_t chain, long long* sums_device,
                                                  int32_t* heights_device) {
  RT_SAMPLER(s);
  return s->impl->accumulate_heights(chain, sums_device, heights_device);
}
RT_API rt_status rt_dm_sampler_sync(rt_dm_sampler* s) {
  RT_SAMPLER(s);
  return s->impl->sync();
}
RT_API void* rt_dm_sampler_stream(rt_dm_sampler* s) { return (s && s->impl) ? (void*)s->impl->stream : nullptr; }
RT_API int64_t rt_dm_sampler_interior_vertices(rt_dm_sampler* s) {
  return (s && s->impl) ? s->impl->interior[0] + s->impl->interior[1] : -1;
}
RT_API int64_t rt_dm_sampler_launches(rt_dm_sampler* s) { return (s && s->impl) ? s->impl->launches : -1; }
RT_API rt_status rt_dm_sampler_test_silent_band(rt_dm_sampler* s, int32_t band, int64_t max_spin) {
  RT_SAMPLER(s);
  if (max_spin < 0) return fail(RT_ERR_INVALID_ARGUMENT, "test_silent_band: max_spin must be >= 0");
  s->impl->test_silent_band = band < 0 ? -1 : band;
  s->impl->test_max_spin = (long)max_spin;
  return RT_OK;
}

RT_API rt_status rt_dm_sampler_engine_info(rt_dm_sampler* s, int64_t* out4) {
  RT_SAMPLER(s);
  if (!out4) return fail(RT_ERR_INVALID_ARGUMENT, "engine_info: out is NULL");
  DmSampler& d = *s->impl;
  bool pers = false;
  if (rt_status st = d.use_persistent(&pers)) return st;
  int64_t units = 0, bands = 0, k = 0;
  if (pers && d.resident == 4) {
    units = d.bits->plan.draw_cells;
    bands = (int64_t)d.bits->plan.bands.size();
    k = kBitSlots;
  } else if (pers && d.resident == 2) {
    units = d.runs->plan.draw_cells;
    bands = (int64_t)d.runs->plan.bands.size();
    k = d.runs->plan.K;
  } else if (pers) {
    for (const DmBand& b : d.persist->plan.bands) units += b.units;
    bands = (int64_t)d.persist->plan.bands.size();
    k = d.persist->plan.K;
  }
  out4[0] = pers ? d.resident : 1;
  out4[1] = units;
  out4[2] = bands;
  out4[3] = k;
  return RT_OK;
}

RT_API rt_status rt_dm_sampler_set_launch(rt_dm_sampler* s, int32_t engine, int32_t bands, int32_t threads) {
  RT_SAMPLER(s);
  if (engine < 0 || engine > 4 || bands < 0 || threads < 0 || threads > 1024 || threads % 32)
    return fail(RT_ERR_INVALID_ARGUMENT, "set_launch: engine 0..4, bands >= 0, threads a multiple of 32 up to 1024");
  DmSampler& d = *s->impl;
  d.launch_engine = engine;
  d.launch_bands = bands;
  d.launch_threads = threads;
  d.plan_dirty = true;
  return RT_OK;
}

RT_API rt_status rt_dm_sampler_launch_info(rt_dm_sampler* s, int64_t* out6) {
  RT_SAMPLER(s);
  if (!out6) return fail(RT_ERR_INVALID_ARGUMENT, "launch_info: out is NULL");
  int64_t e4[4];
  if (rt_status st = rt_dm_sampler_engine_info(s, e4)) return st;
  DmSampler& d = *s->impl;
  for (int k = 0; k < 4; ++k) out6[k] = e4[k];
  out6[4] = (e4[0] == 4)   ? (int64_t)d.bits->plan.warps * 32
            : (e4[0] == 2) ? d.runs->plan.threads
                           : (e4[0] == 3 ? (int64_t)kPersistThreads : 0);
  out6[5] = d.tuned ? 1 : 0;
  return RT_OK;
}

// ---- walks ---------------------------------------------------------------------------------

static std::vector<uint8_t> colour_draws(std::mt19937& mt, int64_t steps) {
  std::vector<uint8_t> c((size_t)steps);
  for (int64_t s = 0; s < steps; ++s) c[(size_t)s] = (uint8_t)(mt() % 2);
  return c;
}

RT_API rt_status rt_domino_walk(int32_t* tiling, int32_t n_side, int64_t steps, int64_t seed, const rt_walk_opts* opts) {
  clear_error();
  if (!tiling || steps < 0) return fail(RT_ERR_INVALID_ARGUMENT, "walk: NULL tiling or negative steps");
  rt_walk_opts o = opts_or_default(opts);
  std::unique_ptr<DmSampler> s;
  if (rt_status st = DmSampler::create(n_side, 1, o, &s)) return st;
  if (rt_status st = s->load(0, tiling)) return st;
  if (o.rng_mode == RT_RNG_TINYMT) {
    // DominoTiler.cpp:50-53 (OpenCL branch): generators seeded by the first draw, colours
    // from the following draws (:69-70).
    std::mt19937 mt((uint32_t)seed);
    if (rt_status st = s->seed((uint32_t)mt())) return st;
    std::vector<uint8_t> col = colour_draws(mt, steps);
    if (rt_status st = s->run(col.data(), steps)) return st;
  } else if (o.rng_mode == RT_RNG_MTGP) {
    // DominoTiler.cpp:51-66 (CUDA branch): block generator k seeded seed + k, colours from
    // mt19937(seed) starting with its first draw (:69).
    std::mt19937 mt((uint32_t)seed);
    if (rt_status st = s->seed(seed)) return st;
    std::vector<uint8_t> col = colour_draws(mt, steps);
    if (rt_status st = s->run(col.data(), steps)) return st;
  } else {
    if (rt_status st = s->run_fast((uint64_t)seed, 0, steps)) return st;
  }
  return s->store(0, tiling);
}

RT_API rt_status rt_domino_walk_epochs(int32_t* tiling, int32_t n_side, const int64_t* steps, const int64_t* seeds,
                                       int32_t n_epochs, const rt_walk_opts* opts) {
  clear_error();
  if (!tiling || n_epochs < 0 || (n_epochs > 0 && (!steps || !seeds)))
    return fail(RT_ERR_INVALID_ARGUMENT, "walk_epochs: bad arguments");
  for (int k = 0; k < n_epochs; ++k)
    if (steps[k] < 0) return fail(RT_ERR_INVALID_ARGUMENT, "walk_epochs: negative steps");
  rt_walk_opts o = opts_or_default(opts);
  std::unique_ptr<DmSampler> s;
  if (rt_status st = DmSampler::create(n_side, 1, o, &s)) return st;
  if (rt_status st = s->load(0, tiling)) return st;
  int64_t h = 0;
  for (int k = 0; k < n_epochs; ++k) {
    if (o.rng_mode != RT_RNG_FAST) {
      // DominoTiler.cpp:155-175: mt19937(seeds[k]) for the colours, generators from seeds[k]
      // (TinyMT: generator k seeded seeds[k] + k; MTGP: block generator k seeded seeds[k] + k).
      std::mt19937 mt((uint32_t)seeds[k]);
      if (rt_status st = s->seed(o.rng_mode == RT_RNG_MTGP ? seeds[k] : (int64_t)(uint32_t)seeds[k])) return st;
      std::vector<uint8_t> col = colour_draws(mt, steps[k]);
      if (rt_status st = s->run(col.data(), steps[k])) return st;
    } else {
      // Fast mode: epoch k is keyed by seeds[k] and restarts at half-sweep 0.
      if (rt_status st = s->run_fast((uint64_t)seeds[k], 0, steps[k])) return st;
      h += steps[k];
    }
  }
  return s->store(0, tiling);
}

RT_API rt_status rt_domino_cftp(const int32_t* tmax, const int32_t* tmin, int32_t n_side, int64_t driver_seed,
                                int64_t first_steps, int32_t schedule, int32_t max_attempts, const rt_walk_opts* opts,
                                int32_t* out, rt_cftp_stats* stats) {
  clear_error();
  if (!tmax || !tmin || !out) return fail(RT_ERR_INVALID_ARGUMENT, "cftp: NULL tiling");
  if (first_steps < 1 || max_attempts < 1 || max_attempts > 40 || (schedule != 0 && schedule != 1))
    return fail(RT_ERR_INVALID_ARGUMENT, "cftp: first_steps >= 1, 1 <= max_attempts <= 40, schedule 0 or 1");
  rt_walk_opts o = opts_or_default(opts);
  if (o.rule != RT_DOMINO_CFTP && o.rule != RT_DOMINO_CFTP_TWOPERIODIC)
    return fail(RT_ERR_INVALID_ARGUMENT, "cftp needs a monotone rule (RT_DOMINO_CFTP or RT_DOMINO_CFTP_TWOPERIODIC)");
  std::unique_ptr<DmSampler> s;
  // chains 0 (bottom) and 1 (top) are swept; 2 and 3 keep the min and max start states.
  if (rt_status st = DmSampler::create(n_side, 4, o, &s)) return st;
  if (rt_status st = s->load(0, tmin)) return st;  // also counts the interior vertices
  if (rt_status st = s->copy_chain(2, 0)) return st;
  if (rt_status st = s->load(3, tmax)) return st;
  s->active = 2;
  s->plan_dirty = true;
  const bool fast = o.rng_mode == RT_RNG_FAST;
  // The reference's epoch schedule (AztecDiamondCftpEx.cpp:54-77), drawn ahead for every
  // attempt: epoch k is created by attempt k with the driver's k-th draw as its seed, and
  // attempt a runs epochs a, a-1, ..., 0 in that order.  AztecDiamondCftpEx.cpp:76 gives the
  // new epoch 2 * steps.back() half-sweeps (schedule 0); schedule 1 doubles the oldest.
  std::mt19937 drv((uint32_t)driver_seed);
  std::vector<int64_t> ep_steps;
  std::vector<uint32_t> ep_seed;
  std::vector<std::vector<uint8_t>> ep_colours((size_t)max_attempts);
  if (!fast) {
    for (int k = 0; k < max_attempts; ++k) {
      ep_seed.push_back((uint32_t)drv());
      ep_steps.push_back(k == 0 ? first_steps : (schedule == 0 ? 2 * ep_steps[0] : 2 * ep_steps[k - 1]));
    }
  }
  auto colours_of = [&](int k) -> const std::vector<uint8_t>& {
    if (ep_colours[(size_t)k].empty() && ep_steps[(size_t)k] > 0) {
      std::mt19937 mt(ep_seed[(size_t)k]);
      ep_colours[(size_t)k] = colour_draws(mt, ep_steps[(size_t)k]);
    }
    return ep_colours[(size_t)k];
  };
  // Look-back of attempt a (half-sweeps) and its flip attempts over both chains.
  auto look_back = [&](int att) -> int64_t {
    if (fast) return 2 * (first_steps << att);
    int64_t t = 0;
    for (int k = 0; k <= att; ++k) t += ep_steps[(size_t)k];
    return t;
  };
  auto flips_of = [&](int att) -> int64_t {
    int64_t black = 0, total = look_back(att);
    if (fast) {
      black = total / 2;  // half-sweeps -2T .. -1 alternate, black at even h
    } else {
      for (int k = 0; k <= att; ++k)
        for (uint8_t c : colours_of(k)) black += c ? 1 : 0;
    }
    return 2 * (black * s->interior[1] + (total - black) * s->interior[0]);
  };
  rt_cftp_stats st_out{};
  float ms_total = 0.f;
  auto account = [&](int att) {
    st_out.attempts = att + 1;
    st_out.total_steps += look_back(att);
    st_out.final_steps = look_back(att);
    st_out.flip_attempts += flips_of(att);
  };
  // Attempts go to the run kernel in one launch per group whose look-backs sum to at most
  // kLaunchHalfSweeps (a launch of well under a second at order 1024); an attempt longer than
  // that, or a sampler the run kernel does not take, runs attempt by attempt from the host.
  const int64_t kLaunchHalfSweeps = (int64_t)1 << 21;
  bool pers = false;
  if (rt_status st = s->use_persistent(&pers)) return st;
  const bool one_launch = pers && (s->resident == 2 || s->resident == 4) && o.rng_mode != RT_RNG_MTGP;
  int att = 0;
  bool coalesced = false;
  while (att < max_attempts && !coalesced) {
    int n = 0;
    int64_t tot = 0;
    while (one_launch && att + n < max_attempts && tot + look_back(att + n) <= kLaunchHalfSweeps)
      tot += look_back(att + n++);
    if (n > 0) {
      std::vector<std::vector<RunEngine::Epoch>> epochs((size_t)n);
      for (int q = 0; !fast && q < n; ++q)
        for (int k = att + q; k >= 0; --k) epochs[(size_t)q].push_back({ep_seed[(size_t)k], &colours_of(k)});
      cudaEventRecord(s->ev0, s->stream);
      int ran = 0;
      if (s->resident == 4) {
        if (rt_status st = s->bits->cftp(*s, n, epochs, &ran, &coalesced)) return st;
      } else if (rt_status st = s->runs->cftp(*s, att, n, epochs, first_steps, (uint64_t)driver_seed, &ran, &coalesced)) {
        return st;
      }
      cudaEventRecord(s->ev1, s->stream);
      cudaEventSynchronize(s->ev1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, s->ev0, s->ev1);
      ms_total += ms;
      for (int q = 0; q < ran; ++q) account(att + q);
      att += ran;
      continue;
    }
    // One attempt from the host: reset, the attempt's half-sweeps, the coalescence count.
    if (rt_status st = s->copy_chain(0, 2)) return st;
    if (rt_status st = s->copy_chain(1, 3)) return st;
    cudaEventRecord(s->ev0, s->stream);
    if (!fast) {
      for (int k = att; k >= 0; --k) {
        if (rt_status st = s->seed(ep_seed[(size_t)k])) return st;
        if (rt_status st = s->run(colours_of(k).data(), ep_steps[(size_t)k])) return st;
      }
    } else {
      const int64_t T = first_steps << att;
      if (rt_status st = s->run_fast((uint64_t)driver_seed, -2 * T, 2 * T)) return st;
    }
    cudaEventRecord(s->ev1, s->stream);
    int64_t nd = -1;
    if (rt_status st = s->diff(0, 1, &nd)) return st;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    ms_total += ms;
    account(att);
    coalesced = nd == 0;
    ++att;
  }
  st_out.seconds = ms_total * 1e-3;
  if (stats) *stats = st_out;
  // out receives the top chain of the last attempt, so a caller can resume or inspect it.
  if (rt_status st = s->store(1, out)) return st;
  if (!coalesced) return fail(RT_ERR_NOT_COALESCED, "cftp: chains did not coalesce within max_attempts");
  return RT_OK;
}

}  // extern "C"
