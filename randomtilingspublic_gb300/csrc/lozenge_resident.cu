// Resident engine of the lozenge sweep: one cooperative launch runs many steps of the
// three-colour chain (lozengekernel.cl RotateTiles + UpdateTiles per step,
// LozengeTiler.cpp:92-108) with every chain held in shared memory.
//
// The N rows are split into bands, one CTA each.  A band keeps its rows of every chain and
// colour plus one halo row above and below (3 x chains x (R + 2) x P bytes).  One step of
// colour r is:
//   1. the rotation of colour r on the band's rows: each thread owns column quads (four
//      vertices, one 32-bit word per chain) with their draws - TinyMT generators of the
//      reference's numbering (one per vertex slot, k = i * M + j, all stepping every step) in
//      registers, or the fast mode's Philox draw keyed by (seed, stream, step, row, quad) -
//      and flips 25 <-> 38 for the four bytes at once;
//   2. the words of the band's first and last rows go to global memory as 64-bit tagged words
//      (data | step tag << 32, one single-copy-atomic store each), in a slot chosen by the
//      step's parity; the band reads its neighbours' words of the same step into its halo
//      rows, polling each until its tag matches (a bounded wait: after max_spin polls the
//      band records an error and leaves, and so do the bands waiting on it);
//   3. a CTA barrier, the rebuild of the two other colours on the band's rows from colour r
//      (lozengekernel.cl:36-54 semantics, four vertices per word), a CTA barrier.
// A band can run at most one step ahead of a neighbour (it needs the neighbour's words of each
// step), so a parity slot is rewritten only after its reader has consumed it.  Every draw and
// every byte operation is the per-step kernels', so a walk or CFTP gives the same tiling with
// either engine.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "lozenge_resident.h"
#include "rng.cuh"

namespace rt {
namespace {

constexpr int kLzThreads = 1024;
constexpr long kLzMaxSpin = 1L << 22;
constexpr int64_t kLzChunk = 1 << 16;  // steps per launch

struct LzResArgs {
  uint8_t* base;
  size_t colour_stride, chain_stride;
  int N, M, P, nbands, plane_rows;
  uint32_t lo_up, w_up, lo_dn, w_dn;
  uint4* tmt;
  const uint4* params;
  const uint8_t* colours;  // TinyMT: colour of each step; NULL in fast mode
  int64_t steps, h0;
  uint64_t seed;
  uint32_t stream;
  uint64_t* xbuf;  // [2 parities][bands][first, last row][chains][quads]
  uint32_t tag0;
  int* error;
  long max_spin;
};

__device__ __forceinline__ uint32_t lz_bytes_equal(uint32_t x, uint32_t bbbb) {
  return ~((x ^ bbbb) + 0x7f7f7f7fu) & 0x80808080u;  // bytes below 0x80: no carries
}
__device__ __forceinline__ uint32_t lz_byte_bit(bool p, int k) { return p ? 0x80u << (8 * k) : 0u; }

__device__ __forceinline__ void st_tagged(uint64_t* p, uint64_t v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint64_t ld_tagged(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// kTmt: TinyMT draws from K quads' generators in registers (units t + k * threads); fast
// mode: Philox draws, any number of quads per thread.
template <bool kTmt, int K, int NCH>
__global__ void __launch_bounds__(kLzThreads, 1) k_lz_resident(LzResArgs a) {
  extern __shared__ __align__(16) uint8_t sm[];
  const int b = blockIdx.x, T = blockDim.x, t = threadIdx.x;
  const int N = a.N, M = a.M, P = a.P;
  const int r0 = (int)((int64_t)b * N / a.nbands), r1 = (int)((int64_t)(b + 1) * N / a.nbands);
  const int s0 = max(0, r0 - 1), s1 = min(N, r1 + 1);
  const size_t plane = (size_t)a.plane_rows * P;
  const int QD = (M + 3) / 4, words = P / 4;
  const int units = (r1 - r0) * QD;
  const bool has_up = b > 0, has_dn = b + 1 < a.nbands;
  auto row = [&](int c, int k, int i) { return sm + (size_t)(c * 3 + k) * plane + (size_t)(i - s0) * P; };
  auto slot = [&](int par, int band, int dir, int c) {
    return a.xbuf + ((((size_t)par * a.nbands + band) * 2 + dir) * NCH + c) * QD;
  };

  // load the stored rows of every chain and colour
  {
    const int vec = P / 16, nrow = s1 - s0;
    for (int k = t; k < NCH * 3 * nrow * vec; k += T) {
      const int x = k % vec, rk = k / vec;
      const int i = s0 + rk % nrow, ck = rk / nrow;  // ck = c * 3 + colour
      const uint8_t* g = a.base + (size_t)(ck / 3) * a.chain_stride + (size_t)(ck % 3) * a.colour_stride + (size_t)i * P;
      reinterpret_cast<uint4*>(row(ck / 3, ck % 3, i))[x] = reinterpret_cast<const uint4*>(g)[x];
    }
  }
  uint4 gen[kTmt ? K : 1][4];
  if constexpr (kTmt) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int u = t + k * T;
      if (u < units) {
        const int i = r0 + u / QD, q = u % QD;
#pragma unroll
        for (int k4 = 0; k4 < 4; ++k4)
          if (4 * q + k4 < M) gen[k][k4] = a.tmt[(size_t)i * M + 4 * q + k4];
      }
    }
  }
  __syncthreads();

  bool failed = false;
  for (int64_t s = 0; s < a.steps; ++s) {
    const uint32_t tag = a.tag0 + (uint32_t)s + 1u;
    const int par = (int)(tag & 1u);
    const int64_t h = a.h0 + s;
    const int r = kTmt ? (int)a.colours[s] : (int)(((h % 3) + 3) % 3);
    // 1. rotation of colour r, boundary rows published
    auto rotate = [&](int u, uint32_t d0, uint32_t d1, uint32_t d2, uint32_t d3) {
      const int i = r0 + u / QD, q = u % QD;
      uint32_t valid = 0x80808080u;  // vertices j = 4q + k below M
      const int over = 4 * q + 4 - M;
      if (over > 0) valid = 0x80808080u >> (8 * over);
      const uint32_t acc_up = (lz_byte_bit(d0 - a.lo_up < a.w_up, 0) | lz_byte_bit(d1 - a.lo_up < a.w_up, 1) |
                               lz_byte_bit(d2 - a.lo_up < a.w_up, 2) | lz_byte_bit(d3 - a.lo_up < a.w_up, 3)) & valid;
      const uint32_t acc_dn = (lz_byte_bit(d0 - a.lo_dn < a.w_dn, 0) | lz_byte_bit(d1 - a.lo_dn < a.w_dn, 1) |
                               lz_byte_bit(d2 - a.lo_dn < a.w_dn, 2) | lz_byte_bit(d3 - a.lo_dn < a.w_dn, 3)) & valid;
#pragma unroll
      for (int c = 0; c < NCH; ++c) {
        uint32_t* word = reinterpret_cast<uint32_t*>(row(c, r, i)) + q;
        const uint32_t e4 = *word;
        const uint32_t f = (lz_bytes_equal(e4, 0x19191919u) & acc_up) | (lz_bytes_equal(e4, 0x26262626u) & acc_dn);
        const uint32_t n4 = e4 ^ ((f >> 7) * 63u);
        if (n4 != e4) *word = n4;
        const uint64_t tagged = ((uint64_t)tag << 32) | n4;
        if (i == r0 && has_up) st_tagged(slot(par, b, 0, c) + q, tagged);
        if (i == r1 - 1 && has_dn) st_tagged(slot(par, b, 1, c) + q, tagged);
      }
    };
    if constexpr (kTmt) {
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const int u = t + k * T;
        if (u < units) {
          const int i = r0 + u / QD, q = u % QD;
          uint32_t d[4] = {0, 0, 0, 0};
#pragma unroll
          for (int k4 = 0; k4 < 4; ++k4) {
            if (4 * q + k4 < M) {
              const size_t gk = (size_t)i * M + 4 * q + k4;
              const uint4 p = a.params ? __ldg(a.params + gk) : make_uint4(kTmtMat1, kTmtMat2, kTmtTmat, 0);
              d[k4] = tmt_next_u23(gen[k][k4], p.x, p.y, p.z);
            }
          }
          rotate(u, d[0], d[1], d[2], d[3]);
        }
      }
    } else {
      for (int u = t; u < units; u += T) {
        const int i = r0 + u / QD, q = u % QD;
        const uint4 d = fast_quad(a.seed, a.stream, h, (uint32_t)i, (uint32_t)q);
        rotate(u, d.x, d.y, d.z, d.w);
      }
    }
    // 2. the neighbours' boundary words of this step into the halo rows
    const int halo_units = 2 * NCH * QD;
    for (int k = t; k < halo_units; k += T) {
      const int dir = k / (NCH * QD), rest = k - dir * (NCH * QD);
      const int c = rest / QD, q = rest - c * QD;
      if (dir == 0 ? !has_up : !has_dn) continue;
      const uint64_t* src = dir == 0 ? slot(par, b - 1, 1, c) + q : slot(par, b + 1, 0, c) + q;
      uint64_t v = ld_tagged(src);
      long spins = 0;
      while ((uint32_t)(v >> 32) != tag) {
        if (++spins > a.max_spin) {
          failed = true;
          break;
        }
        v = ld_tagged(src);
      }
      reinterpret_cast<uint32_t*>(row(c, r, dir == 0 ? r0 - 1 : r1))[q] = (uint32_t)v;
    }
    if (__syncthreads_or(failed)) {
      failed = true;
      break;
    }
    // 3. rebuild of colours r + 1 and r + 2 on rows [max(r0, 1), min(r1, N - 1))
    const int b0 = max(r0, 1), b1 = min(r1, N - 1);
    for (int k = t; k < (b1 - b0) * words; k += T) {
      const int i = b0 + k / words, w = k % words;
      uint32_t keep = 0;  // vertices outside columns [1, M - 2]
      if (w == 0) keep = 0xffu;
      const int over = 4 * w + 3 - (M - 2);
      if (over >= 4) continue;
      if (over > 0) keep |= 0xffffffffu << (8 * (4 - over));
      const int im = i % 3;
      const bool p2 = im == (2 * r + 1) % 3, p4 = im == (2 * r + 2) % 3, p8 = im == (2 * r) % 3;
#pragma unroll
      for (int c = 0; c < NCH; ++c) {
        const uint32_t* up = reinterpret_cast<const uint32_t*>(row(c, r, i - 1));
        const uint32_t* mid = up + words;
        const uint32_t* dn = mid + words;
        uint32_t* T2 = reinterpret_cast<uint32_t*>(row(c, (r + 1) % 3, i)) + w;
        uint32_t* T3 = reinterpret_cast<uint32_t*>(row(c, (r + 2) % 3, i)) + w;
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
    __syncthreads();
  }
  if (failed && t == 0) atomicExch(a.error, 1);

  // write back the band's rows and the generators
  {
    const int vec = P / 16, nrow = r1 - r0;
    for (int k = t; k < NCH * 3 * nrow * vec; k += T) {
      const int x = k % vec, rk = k / vec;
      const int i = r0 + rk % nrow, ck = rk / nrow;
      uint8_t* g = a.base + (size_t)(ck / 3) * a.chain_stride + (size_t)(ck % 3) * a.colour_stride + (size_t)i * P;
      reinterpret_cast<uint4*>(g)[x] = reinterpret_cast<const uint4*>(row(ck / 3, ck % 3, i))[x];
    }
  }
  if constexpr (kTmt) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int u = t + k * T;
      if (u < units) {
        const int i = r0 + u / QD, q = u % QD;
#pragma unroll
        for (int k4 = 0; k4 < 4; ++k4)
          if (4 * q + k4 < M) a.tmt[(size_t)i * M + 4 * q + k4] = gen[k][k4];
      }
    }
  }
}

void* kernel_for(bool tinymt, int K, int nch) {
  if (tinymt) {
    if (K == 1) return nch == 1 ? (void*)k_lz_resident<true, 1, 1> : (void*)k_lz_resident<true, 1, 2>;
    return nch == 1 ? (void*)k_lz_resident<true, 2, 1> : (void*)k_lz_resident<true, 2, 2>;
  }
  return nch == 1 ? (void*)k_lz_resident<false, 0, 1> : (void*)k_lz_resident<false, 0, 2>;
}

}  // namespace

rt_status lz_resident_error(LzResidentState& st, cudaStream_t s) {
  if (!st.error) return RT_OK;
  int err = 0;
  if (cudaMemcpyAsync(&err, st.error, sizeof err, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    const cudaError_t e = cudaGetLastError();
    return fail(RT_ERR_CUDA, std::string("lozenge resident engine: ") + cudaGetErrorString(e));
  }
  if (err) {
    cudaMemsetAsync(st.error, 0, sizeof(int), s);
    return fail(RT_ERR_TIMEOUT, "lozenge resident engine: a band gave up waiting for a neighbour's boundary row");
  }
  return RT_OK;
}

LzResidentState::~LzResidentState() {
  if (xbuf) cudaFree(xbuf);
  if (error) cudaFree(error);
  if (colours) cudaFree(colours);
}

LzResidentPlan lz_resident_plan(const LzResidentGeom& g, bool tinymt) {
  LzResidentPlan p;
  if (g.nch < 1 || g.nch > 2) return p;
  int dev = 0, sms = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
    cudaGetLastError();
    return p;
  }
  // at least 4 rows a band, at most one band per SM
  const int bands = std::max(1, std::min(sms, g.N / 4));
  const int rows_max = (g.N + bands - 1) / bands;
  const int QD = (g.M + 3) / 4;
  const int K = (rows_max * QD + kLzThreads - 1) / kLzThreads;
  if (tinymt && K > 2) return p;
  const size_t smem = (size_t)g.nch * 3 * (rows_max + 2) * g.P;
  if (smem > (size_t)optin - 1024) return p;
  void* kern = kernel_for(tinymt, std::max(1, K), g.nch);
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
    cudaGetLastError();
    return p;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kLzThreads, smem) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    return p;
  }
  p.ok = true;
  p.bands = bands;
  p.threads = kLzThreads;
  p.K = std::max(1, K);
  p.smem = smem;
  p.rows_max = rows_max;
  return p;
}

rt_status lz_resident_run(LzResidentState& st, const LzResidentGeom& g, uint8_t* base, const LzResidentRule& rule,
                          bool tinymt, uint4* tmt, const uint4* params, const uint8_t* colours_host, int64_t steps,
                          uint64_t fast_seed, uint32_t fast_stream, int64_t h0, cudaStream_t s) {
  const LzResidentPlan& p = st.plan;
  if (!p.ok) return fail(RT_ERR_INVALID_ARGUMENT, "lozenge resident engine: no plan for this size");
  const int QD = (g.M + 3) / 4;
  if (!st.xbuf) {
    const size_t bytes = (size_t)2 * p.bands * 2 * g.nch * QD * sizeof(uint64_t);
    if (cudaMalloc(&st.xbuf, bytes) != cudaSuccess || cudaMalloc(&st.error, sizeof(int)) != cudaSuccess) {
      cudaGetLastError();
      return fail(RT_ERR_OUT_OF_MEMORY, "lozenge resident engine: device allocation failed");
    }
    cudaMemsetAsync(st.xbuf, 0, bytes, s);
    cudaMemsetAsync(st.error, 0, sizeof(int), s);
  }
  if (tinymt && steps > st.colours_cap) {
    if (st.colours) cudaFree(st.colours);
    st.colours = nullptr;
    st.colours_cap = 0;
    if (cudaMalloc(&st.colours, (size_t)steps) != cudaSuccess) {
      cudaGetLastError();
      return fail(RT_ERR_OUT_OF_MEMORY, "lozenge resident engine: device allocation failed");
    }
    st.colours_cap = steps;
  }
  if (tinymt && steps > 0 && cudaMemcpyAsync(st.colours, colours_host, (size_t)steps, cudaMemcpyHostToDevice, s) != cudaSuccess) {
    cudaGetLastError();
    return fail(RT_ERR_CUDA, "lozenge resident engine: colour copy failed");
  }
  void* kern = kernel_for(tinymt, p.K, g.nch);
  for (int64_t done = 0; done < steps; done += kLzChunk) {
    LzResArgs a;
    a.base = base;
    a.colour_stride = g.colour_stride;
    a.chain_stride = g.chain_stride;
    a.N = g.N;
    a.M = g.M;
    a.P = g.P;
    a.nbands = p.bands;
    a.plane_rows = p.rows_max + 2;
    a.lo_up = rule.lo_up;
    a.w_up = rule.w_up;
    a.lo_dn = rule.lo_dn;
    a.w_dn = rule.w_dn;
    a.tmt = tmt;
    a.params = params;
    a.colours = tinymt ? st.colours + done : nullptr;
    a.steps = std::min(kLzChunk, steps - done);
    a.h0 = h0 + done;
    a.seed = fast_seed;
    a.stream = fast_stream;
    a.xbuf = st.xbuf;
    a.tag0 = st.tag;
    a.error = st.error;
    a.max_spin = kLzMaxSpin;
    void* args[] = {&a};
    const cudaError_t e = cudaLaunchCooperativeKernel(kern, dim3(p.bands), dim3(p.threads), args, p.smem, s);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(RT_ERR_CUDA, std::string("lozenge resident engine launch: ") + cudaGetErrorString(e));
    }
    st.tag += (uint32_t)a.steps;
  }
  return RT_OK;
}

}  // namespace rt
