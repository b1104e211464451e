// The lozenge three-colour sweep on the GPU (reference: src/Lozenge/LozengeTiler.cpp:27-159
// and src/Lozenge/lozengekernel.cl).
//
// Device layout of one chain: three colour arrays (colour c holds the vertices with
// (j - i) mod 3 == c, column j / 3 of row i), each N rows x P bytes, P = N/3 rounded up to
// 16.  One step rotates colour r: every vertex of that colour in state 25 becomes 38 with
// probability 0.4 and every 38 becomes 25 with probability 0.4 (one draw decides both, so
// coupled chains stay ordered), then rebuilds three bits of each of the two other colours.
// TinyMT generator k = i * (N/3) + j for every vertex slot of the N x N/3 grid, as the
// reference's NDRange numbers them.  MTGP mode: the reference's CUDA build instead (8 x 8
// blocks over the same grid, row from the x index, one cuRAND MTGP32 generator per block
// seeded seed + block; LozengeTiler.cpp:71-80, lozengekernel.cu:15-29).
#include <cuda_runtime.h>
#include <curand_kernel.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "lozenge_resident.h"
#include "pdl.cuh"
#include "rng.cuh"
#include "rt_internal.h"

namespace rt {
namespace {

#define LZ_CUDA(expr)                                                                   \
  do {                                                                                  \
    cudaError_t _e = (expr);                                                            \
    if (_e != cudaSuccess)                                                              \
      return fail(RT_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e));     \
  } while (0)

struct LzView {
  uint8_t* base;
  int N, M, P, active;
  size_t colour_stride, chain_stride;
  uint4* tmt;
  const uint4* tmt_params;  // per-generator {mat1, mat2, tmat} (LoadTinyMT), or NULL
  __host__ __device__ uint8_t* colour(int ch, int c) const {
    return base + (size_t)ch * chain_stride + (size_t)c * colour_stride;
  }
};

struct LzRule {
  uint32_t lo_up, w_up, lo_dn, w_dn;
};

__device__ __forceinline__ uint8_t lz_flip(uint32_t e, uint32_t u, const LzRule& r) {
  if (e == 25u) return (u - r.lo_up) < r.w_up ? 38 : 25;
  if (e == 38u) return (u - r.lo_dn) < r.w_dn ? 25 : 38;
  return (uint8_t)e;
}

// InitTinyMT (lozengekernel.cl:127-134): generator k, of the work item (i, j) = (k / M,
// k mod M), seeded seed + k with its own parameters when a table is loaded.
__global__ void k_lz_seed(uint4* st, const uint4* params, int64_t count, uint32_t seed) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const uint4 p = params ? params[k] : make_uint4(kTmtMat1, kTmtMat2, kTmtTmat, 0);
  st[k] = tmt_seed(seed + (uint32_t)k, p.x, p.y, p.z);
}

__global__ void k_lz_rotate_tmt(LzView v, int r, LzRule rule) {
  pdl_begin();
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
  if (j >= v.M) return;
  const int64_t k = (int64_t)i * v.M + j;
  uint4 s = v.tmt[k];
  const uint4 p = v.tmt_params ? v.tmt_params[k] : make_uint4(kTmtMat1, kTmtMat2, kTmtTmat, 0);
  const uint32_t u = tmt_next_u23(s, p.x, p.y, p.z);
  v.tmt[k] = s;
  for (int ch = 0; ch < v.active; ++ch) {
    uint8_t* p = v.colour(ch, r) + (size_t)i * v.P + j;
    const uint32_t e = *p;
    const uint8_t n = lz_flip(e, u, rule);
    if (n != e) *p = n;
  }
}

// MTGP mode (lozengekernel.cu:15-29): every thread of the 8 x 8 block draws from its block's
// generator before the bounds test; u is the float draw's bit pattern.
__global__ void __launch_bounds__(kMtgpBlock* kMtgpBlock) k_lz_rotate_mtgp(LzView v, int r, LzRule rule,
                                                                            curandStateMtgp32* states) {
  pdl_begin();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const float rd = curand_uniform(states + blockIdx.x * gridDim.y + blockIdx.y);
  if (i >= v.N || j >= v.M) return;
  const uint32_t u = __float_as_uint(rd);
  for (int ch = 0; ch < v.active; ++ch) {
    uint8_t* p = v.colour(ch, r) + (size_t)i * v.P + j;
    const uint32_t e = *p;
    const uint8_t n = lz_flip(e, u, rule);
    if (n != e) *p = n;
  }
}

// Thread (q, i): the column quad q (one 32-bit word, columns 4q..4q+3) of row i, with the
// quad's four draws; columns at or beyond M keep their value.
__global__ void k_lz_rotate_fast(LzView v, int r, LzRule rule, uint64_t seed, uint32_t stream, int64_t h) {
  pdl_begin();
  const int q = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
  if (4 * q >= v.M || i >= v.N) return;
  const uint4 d = fast_quad(seed, stream, h, (uint32_t)i, (uint32_t)q);
  const uint32_t u4[4] = {d.x, d.y, d.z, d.w};
  for (int ch = 0; ch < v.active; ++ch) {
    uint32_t* word = reinterpret_cast<uint32_t*>(v.colour(ch, r) + (size_t)i * v.P) + q;
    const uint32_t e4 = *word;
    uint32_t n4 = e4;
#pragma unroll
    for (int k4 = 0; k4 < 4; ++k4) {
      if (4 * q + k4 >= v.M) break;
      const uint32_t e = (e4 >> (8 * k4)) & 0xffu;
      n4 ^= (e ^ lz_flip(e, u4[k4], rule)) << (8 * k4);
    }
    if (n4 != e4) *word = n4;
  }
}

// lozengekernel.cl:107-125: colour (r+1) mod 3 gets bits 2, 4, 32 and colour (r+2) mod 3
// bits 1, 8, 16 from the rotated colour's neighbours; the column offsets depend on i mod 3:
// T2 = bit 16 of up[j + p2] -> 2, bit 8 of mid[j - p4] -> 4, bit 1 of dn[j] -> 32, and
// T3 = bit 32 of up[j] -> 1, bit 4 of mid[j + p8] -> 8, bit 2 of dn[j - p2] -> 16, with
// p2, p4, p8 = [i mod 3 == (2r+1), (2r+2), 2r mod 3] (exactly one is set).
// Four vertices at a time: thread (w, i) rewrites 32-bit word w (columns 4w..4w+3) of row i
// of both passive colours.  A neighbour one column to the right or left is a funnel shift of
// two adjacent words of the rotated colour, and every bit moves within its byte; bytes
// outside columns [1, M-2] (and rows 0 and N-1) keep their value, as the reference rebuilds
// only those vertices.
__global__ void k_lz_update_w(LzView v, int r) {
  pdl_begin();
  const int w = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int words = v.P / 4;
  if (w >= words || i > v.N - 2) return;
  const int im = i % 3;
  const bool p2 = im == (2 * r + 1) % 3, p4 = im == (2 * r + 2) % 3, p8 = im == (2 * r) % 3;
  uint32_t keep = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int j = 4 * w + k;
    if (j < 1 || j > v.M - 2) keep |= 0xffu << (8 * k);
  }
  if (keep == 0xffffffffu) return;
  for (int ch = 0; ch < v.active; ++ch) {
    const uint32_t* up = reinterpret_cast<const uint32_t*>(v.colour(ch, r) + (size_t)(i - 1) * v.P);
    const uint32_t* mid = up + words;
    const uint32_t* dn = mid + words;
    const uint32_t u0 = up[w], m0 = mid[w], d0 = dn[w];
    // x[j + 1] and x[j - 1] for the word's four columns
    const uint32_t u_r = __funnelshift_r(u0, w + 1 < words ? up[w + 1] : 0u, 8);
    const uint32_t m_r = __funnelshift_r(m0, w + 1 < words ? mid[w + 1] : 0u, 8);
    const uint32_t m_l = __funnelshift_l(w > 0 ? mid[w - 1] : 0u, m0, 8);
    const uint32_t d_l = __funnelshift_l(w > 0 ? dn[w - 1] : 0u, d0, 8);
    const uint32_t a2 = p2 ? u_r : u0, a4 = p4 ? m_l : m0, a8 = p8 ? m_r : m0, a16 = p2 ? d_l : d0;
    const uint32_t b2 = ((a2 & 0x10101010u) >> 3) | ((a4 & 0x08080808u) >> 1) | ((d0 & 0x01010101u) << 5);
    const uint32_t b3 = ((u0 & 0x20202020u) >> 5) | ((a8 & 0x04040404u) << 1) | ((a16 & 0x02020202u) << 3);
    uint32_t* T2 = reinterpret_cast<uint32_t*>(v.colour(ch, (r + 1) % 3) + (size_t)i * v.P) + w;
    uint32_t* T3 = reinterpret_cast<uint32_t*>(v.colour(ch, (r + 2) % 3) + (size_t)i * v.P) + w;
    const uint32_t t2 = *T2, t3 = *T3;
    const uint32_t n2 = (t2 & ~0x26262626u) | b2, n3 = (t3 & ~0x19191919u) | b3;
    *T2 = (n2 & ~keep) | (t2 & keep);
    *T3 = (n3 & ~keep) | (t3 & keep);
  }
}

__global__ void k_lz_split(LzView v, int ch, const int32_t* t) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
  if (j >= v.N) return;
  const int c = ((j - i) % 3 + 3) % 3;
  v.colour(ch, c)[(size_t)i * v.P + j / 3] = (uint8_t)t[(size_t)i * v.N + j];
}

__global__ void k_lz_merge(LzView v, int ch, int32_t* t) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
  if (j >= v.N) return;
  const int c = ((j - i) % 3 + 3) % 3;
  t[(size_t)i * v.N + j] = v.colour(ch, c)[(size_t)i * v.P + j / 3];
}

__global__ void k_lz_diff(const uint32_t* x, const uint32_t* y, size_t words, unsigned long long* out) {
  unsigned long long local = 0;
  for (size_t w = (size_t)blockIdx.x * blockDim.x + threadIdx.x; w < words; w += (size_t)gridDim.x * blockDim.x)
    local += __popc(__vcmpne4(x[w], y[w])) / 8;
  for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
  if ((threadIdx.x & 31) == 0 && local) atomicAdd(out, local);
}

// Acceptance intervals of the rotation.  Rule RT_LOZENGE_UNIFORM (lozengekernel.cl:92-96): up
// when rd < 0.4, down when 0.4 <= rd < 0.8.  Rule RT_LOZENGE_Q (qlozengekernel.cl:23-29, q a
// runtime argument): up (a cube added) when rd < 0.5 and q >= rd / 0.5, down when rd >= 0.5 and
// 1 / q >= (rd - 0.5) / 0.5; the reference multiplies by 0.5 in the last expression, which
// accepts every down move when rd >= 0.5 and breaks the q^volume law for q > 1 (identical
// decisions for q <= 1).  TinyMT draws u23 = rd * 2^23 exactly; fast draws resolve the same
// conditions on 32 bits (rd = u * 2^-32).
template <class F>
uint32_t count_below(uint32_t lo, uint32_t hi, F accept) {  // largest prefix [lo, x) with accept
  while (lo < hi) {
    const uint32_t mid = lo + (hi - lo) / 2;
    if (accept(mid)) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

LzRule lz_rule(int rng_mode, int rule, double q) {
  LzRule r;
  if (rule == RT_LOZENGE_Q) {
    if (rng_mode == RT_RNG_TINYMT) {
      const uint32_t half = 1u << 22;
      const uint32_t up = count_below(0, half, [&](uint32_t u) {
        float rd = (float)u * (1.0f / 8388608.0f);
        rd = (float)(rd / .5);
        return q >= rd;
      });
      const uint32_t dn = count_below(half, 1u << 23, [&](uint32_t u) {
        float rd = (float)u * (1.0f / 8388608.0f);
        rd = (float)((rd - .5) / .5);
        return 1 / q >= rd;
      });
      r = {0u, up, half, dn - half};
    } else {
      const double h = 2147483648.0;
      const uint32_t up = (uint32_t)std::min(h, std::floor(q * h) + 1.0);
      const uint32_t dn = (uint32_t)std::min(h, std::floor(h / q) + 1.0);
      r = {0u, up, 0x80000000u, dn};
    }
    return r;
  }
  if (rng_mode == RT_RNG_MTGP) {
    // u is the bit pattern of the float draw in (0, 1]; the kernel compares it with the
    // doubles .4 and .8 (lozengekernel.cu:24-27).
    auto below = [](double x) {  // float bit patterns b with float(b) < x
      return count_below(0, 0x3f800001u, [&](uint32_t b) {
        float f;
        std::memcpy(&f, &b, sizeof f);
        return (double)f < x;
      });
    };
    const uint32_t c4 = below(.4), c8 = below(.8);
    r = {0u, c4, c4, c8 - c4};
  } else if (rng_mode == RT_RNG_TINYMT) {
    auto below = [](double x) {  // number of u23 with u23 * 2^-23 < x
      return count_below(0, 1u << 23, [&](uint32_t u) { return (double)((float)u * (1.0f / 8388608.0f)) < x; });
    };
    const uint32_t c4 = below(.4), c8 = below(.8);
    r = {0u, c4, c4, c8 - c4};
  } else {
    const uint32_t c4 = (uint32_t)std::ceil(0.4 * 4294967296.0), c8 = (uint32_t)std::ceil(0.8 * 4294967296.0);
    r = {0u, c4, c4, c8 - c4};
  }
  return r;
}

struct LzSampler {
  int N = 0, M = 0, P = 0, n_chains = 0, active = 0;
  size_t colour_stride = 0, chain_stride = 0;
  rt_walk_opts opts{};
  LzRule rule{};
  uint8_t* base = nullptr;
  uint4* tmt = nullptr;
  uint4* tmt_params = nullptr;  // LoadTinyMT table, or NULL
  void* mtgp = nullptr;  // RT_RNG_MTGP: the block generators (curandStateMtgp32)
  bool mtgp_seeded = false;
  int32_t* scratch = nullptr;
  unsigned long long* counter = nullptr;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int64_t interior[3] = {0, 0, 0};
  int64_t steps_by_colour[3] = {0, 0, 0};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::unique_ptr<LzResidentState> res;  // the resident engine for `res_nch` swept chains
  int res_nch = 0;

  ~LzSampler() {
    res.reset();
    if (base) cudaFree(base);
    if (tmt) cudaFree(tmt);
    if (tmt_params) cudaFree(tmt_params);
    if (mtgp) cudaFree(mtgp);
    if (scratch) cudaFree(scratch);
    if (counter) cudaFree(counter);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (own_stream && stream) cudaStreamDestroy(stream);
  }
  LzView view() const {
    return LzView{base, N, M, P, active, colour_stride, chain_stride, tmt, tmt_params};
  }
  static rt_status create(int n_side, int chains, const rt_walk_opts& o, std::unique_ptr<LzSampler>* out) {
    if (n_side < 9 || n_side % 3 || n_side > 32766)
      return fail(RT_ERR_INVALID_ARGUMENT, "lozenge tiling side must be a multiple of 3 in [9, 32766]");
    if (o.rng_mode != RT_RNG_TINYMT && o.rng_mode != RT_RNG_FAST && o.rng_mode != RT_RNG_MTGP)
      return fail(RT_ERR_INVALID_ARGUMENT, "unknown rng mode");
    if (o.rng_mode == RT_RNG_MTGP && o.rule != RT_LOZENGE_UNIFORM)
      return fail(RT_ERR_INVALID_ARGUMENT, "lozenge sweep: the MTGP mode takes the uniform rule (lozengekernel.cu)");
    if (o.rng_mode == RT_RNG_FAST && o.fast_stream >= 65536u) return fail(RT_ERR_INVALID_ARGUMENT, "fast_stream must be < 65536");
    if (o.tinymt_params && o.rng_mode != RT_RNG_TINYMT)
      return fail(RT_ERR_INVALID_ARGUMENT, "lozenge sweep: a TinyMT parameter table needs the TinyMT mode");
    if (o.rule != RT_LOZENGE_UNIFORM && o.rule != RT_LOZENGE_Q) return fail(RT_ERR_INVALID_ARGUMENT, "lozenge sweep: unknown rule");
    if (o.engine < 0 || o.engine > 2)
      return fail(RT_ERR_INVALID_ARGUMENT, "lozenge sweep: engine 0 (automatic), 1 (per-step kernels) or 2 (resident)");
    if (o.engine == 2 && o.rng_mode == RT_RNG_MTGP)
      return fail(RT_ERR_INVALID_ARGUMENT, "lozenge sweep: the MTGP mode runs on the per-step kernels (engine 1)");
    if (o.rule == RT_LOZENGE_Q && (!(o.weight_a > 0.0) || !std::isfinite(o.weight_a)))
      return fail(RT_ERR_INVALID_ARGUMENT, "lozenge sweep: q (weight_a) must be finite and > 0");
    int devs = 0;
    if (cudaGetDeviceCount(&devs) != cudaSuccess || devs == 0) {
      cudaGetLastError();
      return fail(RT_ERR_CUDA, "no CUDA device: the sweep has no CPU fallback");
    }
    auto s = std::make_unique<LzSampler>();
    s->N = n_side;
    s->M = n_side / 3;
    s->P = (s->M + 15) / 16 * 16;
    s->n_chains = s->active = chains;
    s->opts = o;
    s->rule = lz_rule(o.rng_mode, o.rule, o.weight_a);
    s->colour_stride = (size_t)s->N * s->P;
    s->chain_stride = 3 * s->colour_stride;
    if (o.cuda_stream) {
      s->stream = (cudaStream_t)o.cuda_stream;
    } else {
      LZ_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
      s->own_stream = true;
    }
    LZ_CUDA(cudaEventCreate(&s->ev0));
    LZ_CUDA(cudaEventCreate(&s->ev1));
    LZ_CUDA(cudaMalloc(&s->base, s->chain_stride * chains));
    LZ_CUDA(cudaMemsetAsync(s->base, 0, s->chain_stride * chains, s->stream));
    LZ_CUDA(cudaMalloc(&s->scratch, (size_t)s->N * s->N * sizeof(int32_t)));
    LZ_CUDA(cudaMalloc(&s->counter, sizeof(unsigned long long)));
    if (o.rng_mode == RT_RNG_TINYMT) {
      LZ_CUDA(cudaMalloc(&s->tmt, (size_t)s->N * s->M * sizeof(uint4)));
      if (rt_status st = tmt_param_table(o, (int64_t)s->N * s->M, &s->tmt_params, s->stream)) return st;
    }
    if (o.rng_mode == RT_RNG_MTGP) LZ_CUDA(cudaMalloc(&s->mtgp, mtgp_state_bytes(mtgp_grid(s->N, s->M).count())));
    *out = std::move(s);
    return RT_OK;
  }
  LzResidentGeom geom() const { return LzResidentGeom{N, M, P, active, colour_stride, chain_stride}; }
  // The resident engine for the swept chains when the options allow it and a plan holds this
  // size (engine 0: where it holds, 2: required); NULL: the per-step kernels.
  rt_status resident(LzResidentState** out) {
    *out = nullptr;
    if (opts.engine == 1 || opts.rng_mode == RT_RNG_MTGP) return RT_OK;
    if (!res || res_nch != active) {
      res = std::make_unique<LzResidentState>();
      res->plan = lz_resident_plan(geom(), opts.rng_mode == RT_RNG_TINYMT);
      res_nch = active;
    }
    if (!res->plan.ok) {
      if (opts.engine == 2) return fail(RT_ERR_INVALID_ARGUMENT, "lozenge sweep: the resident engine does not hold this size");
      return RT_OK;
    }
    *out = res.get();
    return RT_OK;
  }
  rt_status resident_error() { return res ? lz_resident_error(*res, stream) : RT_OK; }
  rt_status check() {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(RT_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    return RT_OK;
  }
  rt_status load(int ch, const int32_t* t) {
    for (size_t p = 0; p < (size_t)N * N; ++p)
      if ((uint32_t)t[p] > 63u) return fail(RT_ERR_INVALID_ARGUMENT, "lozenge tiling values must be edge masks in [0, 63]");
    if (ch == 0) {
      // Interior vertices per colour (all six triangles covered): the flip attempts of one step.
      std::vector<int32_t> dom((size_t)2 * (N - 1) * (N - 1)), cls((size_t)N * N);
      if (rt_lozenge_tiling_to_domain(t, N, dom.data()) == RT_OK &&
          rt_lozenge_domain_to_vertices(dom.data(), N - 1, cls.data()) == RT_OK) {
        for (int c = 0; c < 3; ++c) interior[c] = 0;
        for (int i = 0; i < N; ++i)
          for (int j = 0; j < N; ++j)
            if (cls[(size_t)i * N + j] == 1) interior[((j - i) % 3 + 3) % 3]++;
      }
      clear_error();
    }
    LZ_CUDA(cudaMemcpyAsync(scratch, t, (size_t)N * N * sizeof(int32_t), cudaMemcpyHostToDevice, stream));
    k_lz_split<<<dim3((N + 255) / 256, N), 256, 0, stream>>>(view(), ch, scratch);
    return check();
  }
  rt_status store(int ch, int32_t* t) {
    if (rt_status st = resident_error()) return st;
    k_lz_merge<<<dim3((N + 255) / 256, N), 256, 0, stream>>>(view(), ch, scratch);
    if (rt_status s = check()) return s;
    LZ_CUDA(cudaMemcpyAsync(t, scratch, (size_t)N * N * sizeof(int32_t), cudaMemcpyDeviceToHost, stream));
    LZ_CUDA(cudaStreamSynchronize(stream));
    return RT_OK;
  }
  rt_status copy_chain(int dst, int src) {
    LZ_CUDA(cudaMemcpyAsync(base + dst * chain_stride, base + src * chain_stride, chain_stride, cudaMemcpyDeviceToDevice,
                            stream));
    return RT_OK;
  }
  // TinyMT: generator k seeded s + k on the device; MTGP: block generator k seeded s + k.
  rt_status seed(int64_t s) {
    if (opts.rng_mode == RT_RNG_MTGP) {
      if (rt_status st = mtgp_seed(mtgp, mtgp_grid(N, M).count(), s, stream)) return st;
      mtgp_seeded = true;
      return RT_OK;
    }
    const int64_t count = (int64_t)N * M;
    k_lz_seed<<<(unsigned)((count + 255) / 256), 256, 0, stream>>>(tmt, tmt_params, count, (uint32_t)s);
    return check();
  }
  rt_status run(const uint8_t* colours, int64_t steps) {
    const LzView v = view();
    if (opts.rng_mode == RT_RNG_MTGP) {
      // An MTGP state holds a pointer to its parameters: none exists before the first seed.
      if (!mtgp_seeded) return fail(RT_ERR_INVALID_ARGUMENT, "lozenge run: MTGP generators not seeded");
      const MtgpGrid g = mtgp_grid(N, M);
      const dim3 gu((P / 4 + 31) / 32, (N - 2 + 7) / 8);
      for (int64_t s = 0; s < steps; ++s) {
        const int r = colours[s];
        pdl_launch(k_lz_rotate_mtgp, dim3(g.gx, g.gy), dim3(kMtgpBlock, kMtgpBlock), stream, v, r, rule,
                   static_cast<curandStateMtgp32*>(mtgp));
        pdl_launch(k_lz_update_w, gu, dim3(32, 8), stream, v, r);
        steps_by_colour[r]++;
      }
      return check();
    }
    LzResidentState* rs = nullptr;
    if (rt_status st = resident(&rs)) return st;
    if (rs) {
      const LzResidentRule rr{rule.lo_up, rule.w_up, rule.lo_dn, rule.w_dn};
      if (rt_status st = lz_resident_run(*rs, geom(), base, rr, true, tmt, tmt_params, colours, steps, 0, 0, 0, stream))
        return st;
      for (int64_t s = 0; s < steps; ++s) steps_by_colour[colours[s]]++;
      return RT_OK;
    }
    const dim3 gr((M + 127) / 128, N), gu((P / 4 + 31) / 32, (N - 2 + 7) / 8);
    for (int64_t s = 0; s < steps; ++s) {
      const int r = colours[s];
      pdl_launch(k_lz_rotate_tmt, gr, dim3(128), stream, v, r, rule);
      pdl_launch(k_lz_update_w, gu, dim3(32, 8), stream, v, r);
      steps_by_colour[r]++;
    }
    return check();
  }
  rt_status run_fast(uint64_t seed_value, int64_t h0, int64_t steps) {
    LzResidentState* rs = nullptr;
    if (rt_status st = resident(&rs)) return st;
    if (rs) {
      const LzResidentRule rr{rule.lo_up, rule.w_up, rule.lo_dn, rule.w_dn};
      if (rt_status st = lz_resident_run(*rs, geom(), base, rr, false, nullptr, nullptr, nullptr, steps, seed_value,
                                         opts.fast_stream, h0, stream))
        return st;
      for (int64_t s = 0; s < steps; ++s) steps_by_colour[(((h0 + s) % 3) + 3) % 3]++;
      return RT_OK;
    }
    const LzView v = view();
    const int quads = (M + 3) / 4;
    const dim3 gr((quads + 31) / 32, (N + 7) / 8), gu((P / 4 + 31) / 32, (N - 2 + 7) / 8);
    for (int64_t s = 0; s < steps; ++s) {
      const int64_t h = h0 + s;
      const int r = (int)(((h % 3) + 3) % 3);
      pdl_launch(k_lz_rotate_fast, gr, dim3(32, 8), stream, v, r, rule, seed_value, opts.fast_stream, h);
      pdl_launch(k_lz_update_w, gu, dim3(32, 8), stream, v, r);
      steps_by_colour[r]++;
    }
    return check();
  }
  rt_status diff(int a, int b, int64_t* nd) {
    if (rt_status st = resident_error()) return st;
    LZ_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), stream));
    const size_t words = chain_stride / 4;
    k_lz_diff<<<(unsigned)std::min<size_t>((words + 255) / 256, 1024), 256, 0, stream>>>(
        reinterpret_cast<const uint32_t*>(base + a * chain_stride), reinterpret_cast<const uint32_t*>(base + b * chain_stride),
        words, counter);
    if (rt_status s = check()) return s;
    unsigned long long h = 0;
    LZ_CUDA(cudaMemcpyAsync(&h, counter, sizeof h, cudaMemcpyDeviceToHost, stream));
    LZ_CUDA(cudaStreamSynchronize(stream));
    *nd = (int64_t)h;
    return RT_OK;
  }
};

// LozengeTiler.cpp:84-90: colours from std::default_random_engine seeded with the walk seed
// through uniform_int_distribution(0, 2).
std::vector<uint8_t> lz_colours(int64_t seed, int64_t steps) {
  std::default_random_engine gen;
  std::uniform_int_distribution<int> dist(0, 2);
  gen.seed(seed);
  std::vector<uint8_t> c((size_t)steps);
  for (int64_t s = 0; s < steps; ++s) c[(size_t)s] = (uint8_t)dist(gen);
  return c;
}

rt_walk_opts opts_or_default(const rt_walk_opts* o) {
  rt_walk_opts d;
  rt_walk_opts_default(&d);
  return o ? *o : d;
}

}  // namespace
}  // namespace rt

using namespace rt;

extern "C" {

RT_API rt_status rt_lozenge_walk(int32_t* tiling, int32_t n_side, int64_t steps, int64_t seed, const rt_walk_opts* opts) {
  clear_error();
  if (!tiling || steps < 0) return fail(RT_ERR_INVALID_ARGUMENT, "lozenge walk: NULL tiling or negative steps");
  rt_walk_opts o = opts_or_default(opts);
  std::unique_ptr<LzSampler> s;
  if (rt_status st = LzSampler::create(n_side, 1, o, &s)) return st;
  if (rt_status st = s->load(0, tiling)) return st;
  if (o.rng_mode != RT_RNG_FAST) {
    // LozengeTiler.cpp:71-88: TinyMT generators (OpenCL branch) or MTGP block generators
    // (CUDA branch) seeded from the walk seed itself, colours from default_random_engine(seed).
    if (rt_status st = s->seed(o.rng_mode == RT_RNG_MTGP ? seed : (int64_t)(uint32_t)seed)) return st;
    std::vector<uint8_t> col = lz_colours(seed, steps);
    if (rt_status st = s->run(col.data(), steps)) return st;
  } else {
    if (rt_status st = s->run_fast((uint64_t)seed, 0, steps)) return st;
  }
  return s->store(0, tiling);
}

RT_API rt_status rt_lozenge_mtgp_draws(int32_t n_side, int64_t seed, int64_t launches, float* out) {
  clear_error();
  if (n_side < 9 || n_side % 3 || n_side > 32766 || launches < 0 || (launches > 0 && !out))
    return fail(RT_ERR_INVALID_ARGUMENT, "lozenge mtgp_draws: n_side a multiple of 3 in [9, 32766], launches >= 0");
  return mtgp_draws_grid(n_side, n_side / 3, seed, launches, out);
}

RT_API rt_status rt_lozenge_cftp(const int32_t* tmax, const int32_t* tmin, int32_t n_side, int64_t driver_seed,
                                 int64_t first_steps, int32_t schedule, int32_t max_attempts, const rt_walk_opts* opts,
                                 int32_t* out, rt_cftp_stats* stats) {
  clear_error();
  if (!tmax || !tmin || !out) return fail(RT_ERR_INVALID_ARGUMENT, "lozenge cftp: NULL tiling");
  if (first_steps < 1 || max_attempts < 1 || max_attempts > 40 || (schedule != 0 && schedule != 1))
    return fail(RT_ERR_INVALID_ARGUMENT, "lozenge cftp: first_steps >= 1, 1 <= max_attempts <= 40, schedule 0 or 1");
  rt_walk_opts o = opts_or_default(opts);
  std::unique_ptr<LzSampler> s;
  if (rt_status st = LzSampler::create(n_side, 4, o, &s)) return st;
  if (rt_status st = s->load(0, tmin)) return st;  // also counts the interior vertices
  if (rt_status st = s->copy_chain(2, 0)) return st;
  if (rt_status st = s->load(3, tmax)) return st;
  s->active = 2;
  std::mt19937 drv((uint32_t)driver_seed);
  std::vector<int64_t> steps{first_steps};
  std::vector<uint32_t> seeds{(uint32_t)drv()};
  rt_cftp_stats st_out{};
  float ms_total = 0.f;
  for (int attempt = 1; attempt <= max_attempts; ++attempt) {
    if (rt_status st = s->copy_chain(0, 2)) return st;
    if (rt_status st = s->copy_chain(1, 3)) return st;
    int64_t before[3] = {s->steps_by_colour[0], s->steps_by_colour[1], s->steps_by_colour[2]};
    cudaEventRecord(s->ev0, s->stream);
    int64_t look_back = 0;
    if (o.rng_mode != RT_RNG_FAST) {
      // Each epoch is one reference Walk(t, steps_k, seed_k) on both chains.
      for (size_t k = 0; k < steps.size(); ++k) {
        if (rt_status st = s->seed(seeds[k])) return st;
        std::vector<uint8_t> col = lz_colours(seeds[k], steps[k]);
        if (rt_status st = s->run(col.data(), steps[k])) return st;
        look_back += steps[k];
      }
    } else {
      const int64_t T = first_steps << (attempt - 1);
      if (rt_status st = s->run_fast((uint64_t)driver_seed, -3 * T, 3 * T)) return st;
      look_back = 3 * T;
    }
    cudaEventRecord(s->ev1, s->stream);
    int64_t nd = -1;
    if (rt_status st = s->diff(0, 1, &nd)) return st;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    ms_total += ms;
    st_out.attempts = attempt;
    st_out.total_steps += look_back;
    st_out.final_steps = look_back;
    for (int c = 0; c < 3; ++c) st_out.flip_attempts += 2 * (s->steps_by_colour[c] - before[c]) * s->interior[c];
    st_out.seconds = ms_total * 1e-3;
    if (nd == 0) {
      if (stats) *stats = st_out;
      return s->store(1, out);
    }
    if (o.rng_mode != RT_RNG_FAST) {
      const int64_t next = schedule == 0 ? steps.back() * 2 : steps.front() * 2;
      steps.insert(steps.begin(), next);
      seeds.insert(seeds.begin(), (uint32_t)drv());
    }
  }
  if (stats) *stats = st_out;
  if (rt_status st = s->store(1, out)) return st;
  return fail(RT_ERR_NOT_COALESCED, "lozenge cftp: chains did not coalesce within max_attempts");
}

}  // extern "C"
