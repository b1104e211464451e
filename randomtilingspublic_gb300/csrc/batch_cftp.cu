// Batched coupling from the past: many independent domino and lozenge instances in one
// persistent launch.
//
// A CTA takes the next instance from a device work queue (an atomic counter), keeps that
// instance's coupled max and min chains in shared memory and runs its whole CFTP there:
// attempt j resets the chains to the extremal tilings and runs the half-sweeps [-S T, 0)
// (S = 2 colours for dominoes, 3 for lozenges, T = first * 2^j sweeps) with fast-mode draws
// keyed by (instance seed, instance stream, half-sweep, row, column quad), then tests
// coalescence with a block reduction.  No CTA ever waits on another, so uneven instance
// sizes only change how many instances each CTA ends up taking.  The draws, rules and
// schedule are those of the single-instance fast mode, so every sample equals what
// rt_domino_cftp / rt_lozenge_cftp return for the same (seed, stream): the batch changes
// the throughput, not the samples.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "domino_rules.h"
#include "rng.cuh"
#include "rt_internal.h"

namespace rt {
namespace {

constexpr int kBatchThreads = 256;

#define BT_CUDA(expr)                                                                   \
  do {                                                                                  \
    cudaError_t _e = (expr);                                                            \
    if (_e != cudaSuccess)                                                              \
      return fail(RT_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e));     \
  } while (0)

// One instance as the kernel sees it.  Colour arrays are N rows x P bytes (P a multiple of
// 16), ncol of them per chain (2 dominoes, 3 lozenges); tmax / tmin / out point at ncol
// consecutive arrays in global memory.
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

struct BatchArgs {
  DevInstance* inst;
  int count;
  uint8_t* tilings;
  unsigned* queue;
};

__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = threadIdx.x < kBatchThreads / 32 ? red[threadIdx.x] : 0;
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

// One domino half-sweep of colour t on both chains held in shared memory (chain c, colour
// k at sm + (c * 2 + k) * N * P): flips with the fast draws of half-sweep h, then the full
// rebuild of the passive colour (dominokernel.cl:22-31 semantics).
__device__ void domino_half_sweep(uint8_t* sm, const DevInstance& in, int t, int64_t h) {
  const int N = in.N, P = in.P, cols = in.cols - 1;  // sites m in [1, cols]
  const size_t plane = (size_t)N * P;
  const int quads = cols / 4 + 1, units = (N - 2) * quads;
  for (int k = threadIdx.x; k < units; k += kBatchThreads) {
    const int i = 1 + k / quads, q = k - (i - 1) * quads;
    const uint4 r = fast_quad(in.seed, in.stream, h, (uint32_t)i, (uint32_t)q);
    const uint32_t rr[4] = {r.x, r.y, r.z, r.w};
    const int c = (i & 1) | (t << 1);
    for (int ch = 0; ch < 2; ++ch) {
      uint8_t* row = sm + (size_t)(ch * 2 + t) * plane + (size_t)i * P;
#pragma unroll
      for (int k4 = 0; k4 < 4; ++k4) {
        const int m = 4 * q + k4;
        if (m < 1 || m > cols) continue;
        const uint32_t e = row[m];
        const uint8_t n = dm_flip_b(e, rr[k4], in.lo_up[c], in.w_up[c], in.lo_dn[c], in.w_dn[c]);
        if (n != e) row[m] = n;
      }
    }
  }
  __syncthreads();
  const int sites = (N - 2) * cols;
  for (int k = threadIdx.x; k < 2 * sites; k += kBatchThreads) {
    const int ch = k >= sites ? 1 : 0, kk = k - ch * sites;
    const int i = 1 + kk / cols, m = 1 + kk % cols;
    const uint8_t* A = sm + (size_t)(ch * 2 + t) * plane;
    uint8_t* Pp = sm + (size_t)(ch * 2 + 1 - t) * plane;
    const int left = m - ((i + t + 1) & 1), right = m + ((i + t) & 1);
    Pp[(size_t)i * P + m] = (uint8_t)(((A[(size_t)(i - 1) * P + m] & 2) >> 1) | ((A[(size_t)(i + 1) * P + m] & 1) << 1) |
                                      ((A[(size_t)i * P + left] & 8) >> 1) | ((A[(size_t)i * P + right] & 4) << 1));
  }
  __syncthreads();
}

// One lozenge step of colour r on both chains (chain c, colour k at sm + (c * 3 + k) * N * P):
// rotation 25 <-> 38 with the fast draws of step h, then the rebuild of the two other colours
// (lozengekernel.cl:107-125 semantics).
__device__ void lozenge_step(uint8_t* sm, const DevInstance& in, int r, int64_t h, uint32_t c4, uint32_t c8) {
  const int N = in.N, P = in.P, M = in.cols;
  const size_t plane = (size_t)N * P;
  const int quads = (M + 3) / 4, units = N * quads;
  for (int k = threadIdx.x; k < units; k += kBatchThreads) {
    const int i = k / quads, q = k - i * quads;
    const uint4 d = fast_quad(in.seed, in.stream, h, (uint32_t)i, (uint32_t)q);
    const uint32_t uu[4] = {d.x, d.y, d.z, d.w};
    for (int ch = 0; ch < 2; ++ch) {
      uint8_t* row = sm + (size_t)(ch * 3 + r) * plane + (size_t)i * P;
#pragma unroll
      for (int k4 = 0; k4 < 4; ++k4) {
        const int j = 4 * q + k4;
        if (j >= M) break;
        const uint32_t e = row[j];
        uint8_t n = (uint8_t)e;
        if (e == 25u && uu[k4] < c4) n = 38;
        else if (e == 38u && uu[k4] >= c4 && uu[k4] < c8) n = 25;
        if (n != e) row[j] = n;
      }
    }
  }
  __syncthreads();
  const int sites = (N - 2) * (M - 2);
  for (int k = threadIdx.x; k < 2 * sites; k += kBatchThreads) {
    const int ch = k >= sites ? 1 : 0, kk = k - ch * sites;
    const int i = 1 + kk / (M - 2), j = 1 + kk % (M - 2);
    const int im = i % 3;
    const int p2 = im == (2 * r + 1) % 3, p4 = im == (2 * r + 2) % 3, p8 = im == (2 * r) % 3, p16 = p2;
    const uint8_t* A = sm + (size_t)(ch * 3 + r) * plane;
    uint8_t* T2 = sm + (size_t)(ch * 3 + (r + 1) % 3) * plane + (size_t)i * P + j;
    uint8_t* T3 = sm + (size_t)(ch * 3 + (r + 2) % 3) * plane + (size_t)i * P + j;
    const uint8_t* up = A + (size_t)(i - 1) * P;
    const uint8_t* mid = A + (size_t)i * P;
    const uint8_t* dn = A + (size_t)(i + 1) * P;
    *T2 = (uint8_t)((*T2 & ~(2 | 4 | 32)) | ((up[j + p2] & 16) >> 3) | ((mid[j - p4] & 8) >> 1) | ((dn[j] & 1) << 5));
    *T3 = (uint8_t)((*T3 & ~(1 | 8 | 16)) | ((up[j] & 32) >> 5) | ((mid[j + p8] & 4) << 1) | ((dn[j - p16] & 2) << 3));
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kBatchThreads) k_batch_cftp(BatchArgs a, uint32_t lz_c4, uint32_t lz_c8) {
  extern __shared__ __align__(16) uint8_t sm[];
  __shared__ int s_idx;
  __shared__ uint32_t red[kBatchThreads / 32];
  for (;;) {
    if (threadIdx.x == 0) s_idx = (int)atomicAdd(a.queue, 1u);
    __syncthreads();
    const int idx = s_idx;
    __syncthreads();
    if (idx >= a.count) break;
    DevInstance& g = a.inst[idx];
    const DevInstance in = g;
    const int ncol = in.model == 0 ? 2 : 3;
    const size_t plane = (size_t)in.N * in.P, chain = ncol * plane;
    const uint32_t* gmax = reinterpret_cast<const uint32_t*>(a.tilings + in.off_max);
    const uint32_t* gmin = reinterpret_cast<const uint32_t*>(a.tilings + in.off_min);
    uint32_t* s32 = reinterpret_cast<uint32_t*>(sm);
    const int words = (int)(chain / 4);
    int attempts = 0;
    int64_t look = 0;
    bool done = false;
    for (int att = 0; att < in.max_attempts && !done; ++att) {
      // chain 0 starts at the min tiling, chain 1 at the max tiling
      for (int w = threadIdx.x; w < words; w += kBatchThreads) {
        s32[w] = gmin[w];
        s32[words + w] = gmax[w];
      }
      __syncthreads();
      const int64_t T = in.first_sweeps << att;
      look = ncol * T;
      for (int64_t h = -look; h < 0; ++h) {
        if (in.model == 0) domino_half_sweep(sm, in, (h & 1) ? 0 : 1, h);
        else lozenge_step(sm, in, (int)(((h % 3) + 3) % 3), h, lz_c4, lz_c8);
      }
      uint32_t differ = 0;
      for (int w = threadIdx.x; w < words; w += kBatchThreads) differ += s32[w] != s32[words + w];
      differ = block_sum(differ, red);
      attempts = att + 1;
      done = differ == 0;
    }
    uint32_t* gout = reinterpret_cast<uint32_t*>(a.tilings + in.off_out);
    for (int w = threadIdx.x; w < words; w += kBatchThreads) gout[w] = s32[words + w];
    if (threadIdx.x == 0) {
      g.attempts = done ? attempts : -attempts;
      g.final_half_sweeps = look;
    }
    __syncthreads();
  }
}

}  // namespace
}  // namespace rt

using namespace rt;

extern "C" {

RT_API rt_status rt_cftp_batch(rt_cftp_instance* inst, int32_t count, void* cuda_stream, rt_batch_stats* stats) {
  clear_error();
  if (!inst || count < 1) return fail(RT_ERR_INVALID_ARGUMENT, "cftp_batch: need at least one instance");
  int dev = 0, sms = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return fail(RT_ERR_CUDA, "no CUDA device: the sweep has no CPU fallback");
  }
  BT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  BT_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  // Host side: validate, colour-split the extremal tilings, lay them out in one buffer.
  std::vector<DevInstance> dv((size_t)count);
  size_t bytes = 0, smem_max = 0;
  std::vector<std::pair<size_t, size_t>> spans;
  for (int k = 0; k < count; ++k) {
    const rt_cftp_instance& x = inst[k];
    if (!x.tmax || !x.tmin || !x.out) return fail(RT_ERR_INVALID_ARGUMENT, "cftp_batch: NULL tiling in instance");
    if (x.first_steps < 1 || x.max_attempts < 1 || x.max_attempts > 40)
      return fail(RT_ERR_INVALID_ARGUMENT, "cftp_batch: first_steps >= 1 and 1 <= max_attempts <= 40");
    if (x.stream >= 65536u) return fail(RT_ERR_INVALID_ARGUMENT, "cftp_batch: stream must be < 65536");
    DevInstance& d = dv[k];
    std::memset(&d, 0, sizeof d);
    d.model = x.model;
    d.N = x.n_side;
    if (x.model == RT_MODEL_DOMINO) {
      if (x.n_side < 6 || x.n_side % 2) return fail(RT_ERR_INVALID_ARGUMENT, "cftp_batch: domino side must be even >= 6");
      if (x.rule != RT_DOMINO_CFTP && x.rule != RT_DOMINO_CFTP_TWOPERIODIC)
        return fail(RT_ERR_INVALID_ARGUMENT, "cftp_batch: domino instances need a monotone rule");
      DmRule r;
      const char* err = nullptr;
      if (!dm_rule_build(x.rule, RT_RNG_FAST, x.weight_a, x.weight_b, &r, &err)) return fail(RT_ERR_INVALID_ARGUMENT, err);
      std::memcpy(d.lo_up, r.lo_up, sizeof r.lo_up);
      std::memcpy(d.w_up, r.w_up, sizeof r.w_up);
      std::memcpy(d.lo_dn, r.lo_dn, sizeof r.lo_dn);
      std::memcpy(d.w_dn, r.w_dn, sizeof r.w_dn);
      d.cols = x.n_side / 2 - 1;
      d.P = ((x.n_side / 2) + 15) / 16 * 16;
    } else if (x.model == RT_MODEL_LOZENGE) {
      if (x.n_side < 9 || x.n_side % 3) return fail(RT_ERR_INVALID_ARGUMENT, "cftp_batch: lozenge side must be a multiple of 3 >= 9");
      d.cols = x.n_side / 3;
      d.P = ((x.n_side / 3) + 15) / 16 * 16;
    } else {
      return fail(RT_ERR_INVALID_ARGUMENT, "cftp_batch: model must be RT_MODEL_DOMINO or RT_MODEL_LOZENGE");
    }
    d.seed = x.seed;
    d.stream = x.stream;
    d.max_attempts = x.max_attempts;
    d.first_sweeps = x.first_steps;
    const int ncol = x.model == RT_MODEL_DOMINO ? 2 : 3;
    const size_t chain = (size_t)ncol * d.N * d.P;
    smem_max = std::max(smem_max, 2 * chain);
    d.off_max = (int64_t)bytes;
    d.off_min = (int64_t)(bytes + chain);
    d.off_out = (int64_t)(bytes + 2 * chain);
    bytes += 3 * chain;
  }
  if (smem_max > (size_t)optin - 1024)
    return fail(RT_ERR_INVALID_ARGUMENT, "cftp_batch: an instance's two chains exceed one CTA's shared memory");
  std::vector<uint8_t> host(bytes, 0);
  for (int k = 0; k < count; ++k) {
    const rt_cftp_instance& x = inst[k];
    const DevInstance& d = dv[k];
    const int N = d.N, ncol = d.model == RT_MODEL_DOMINO ? 2 : 3;
    const size_t plane = (size_t)N * d.P;
    for (int which = 0; which < 2; ++which) {
      const int32_t* t = which == 0 ? x.tmax : x.tmin;
      uint8_t* dst = host.data() + (which == 0 ? d.off_max : d.off_min);
      for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) {
          const int32_t v = t[(size_t)i * N + j];
          if ((uint32_t)v > 63u) return fail(RT_ERR_INVALID_ARGUMENT, "cftp_batch: tiling values out of range");
          int c, col;
          if (ncol == 2) {
            c = ((i + j) & 1) == 0 ? 1 : 0;  // black (t = 1) at even i + j
            col = j / 2;
          } else {
            c = ((j - i) % 3 + 3) % 3;
            col = j / 3;
          }
          dst[(size_t)c * plane + (size_t)i * d.P + col] = (uint8_t)v;
        }
    }
  }
  cudaStream_t stream = (cudaStream_t)cuda_stream;
  uint8_t* d_tilings = nullptr;
  DevInstance* d_inst = nullptr;
  unsigned* d_queue = nullptr;
  auto cleanup = [&]() {
    if (d_tilings) cudaFree(d_tilings);
    if (d_inst) cudaFree(d_inst);
    if (d_queue) cudaFree(d_queue);
  };
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  rt_status status = RT_OK;
  do {
    if (cudaMalloc(&d_tilings, bytes) != cudaSuccess || cudaMalloc(&d_inst, dv.size() * sizeof(DevInstance)) != cudaSuccess ||
        cudaMalloc(&d_queue, sizeof(unsigned)) != cudaSuccess) {
      cudaGetLastError();
      status = fail(RT_ERR_OUT_OF_MEMORY, "cftp_batch: device allocation failed");
      break;
    }
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaMemcpyAsync(d_tilings, host.data(), bytes, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d_inst, dv.data(), dv.size() * sizeof(DevInstance), cudaMemcpyHostToDevice, stream);
    cudaMemsetAsync(d_queue, 0, sizeof(unsigned), stream);
    cudaFuncSetAttribute(k_batch_cftp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_cftp, kBatchThreads, smem_max);
    const int grid = std::max(1, std::min(count, std::max(1, per_sm) * sms));
    const uint32_t c4 = (uint32_t)std::ceil(0.4 * 4294967296.0), c8 = (uint32_t)std::ceil(0.8 * 4294967296.0);
    BatchArgs ba{d_inst, count, d_tilings, d_queue};
    cudaEventRecord(e0, stream);
    k_batch_cftp<<<grid, kBatchThreads, smem_max, stream>>>(ba, c4, c8);
    cudaEventRecord(e1, stream);
    cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) {
      status = fail(RT_ERR_CUDA, std::string("cftp_batch launch: ") + cudaGetErrorString(le));
      break;
    }
    cudaMemcpyAsync(host.data(), d_tilings, bytes, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(dv.data(), d_inst, dv.size() * sizeof(DevInstance), cudaMemcpyDeviceToHost, stream);
    cudaError_t se = cudaStreamSynchronize(stream);
    if (se != cudaSuccess) {
      status = fail(RT_ERR_CUDA, std::string("cftp_batch: ") + cudaGetErrorString(se));
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    int coalesced = 0;
    for (int k = 0; k < count; ++k) {
      rt_cftp_instance& x = inst[k];
      const DevInstance& d = dv[k];
      const int N = d.N, ncol = d.model == RT_MODEL_DOMINO ? 2 : 3;
      const size_t plane = (size_t)N * d.P;
      const uint8_t* src = host.data() + d.off_out;
      for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) {
          const int c = ncol == 2 ? (((i + j) & 1) == 0 ? 1 : 0) : ((j - i) % 3 + 3) % 3;
          x.out[(size_t)i * N + j] = src[(size_t)c * plane + (size_t)i * d.P + (ncol == 2 ? j / 2 : j / 3)];
        }
      x.attempts = d.attempts;
      x.final_steps = d.final_half_sweeps;
      coalesced += d.attempts > 0;
    }
    if (stats) {
      stats->instances = count;
      stats->coalesced = coalesced;
      stats->seconds = ms * 1e-3;
      stats->ctas = grid;
    }
    if (coalesced != count) status = fail(RT_ERR_NOT_COALESCED, "cftp_batch: some instances did not coalesce");
  } while (false);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cleanup();
  return status;
}

}  // extern "C"
