// rt_dm_sweep_noalloc: the resident sweep kernel run on chains the caller already holds on
// the GPU, for callers that cannot allocate device memory themselves or through this
// library - for instance a host application that hands the library a fixed device arena
// carved out up front, or code running where a device allocation could stall or fail at an
// awkward moment (a latency-critical loop, a process sharing a GPU under a hard memory cap).
//
// The kernel's own scratch - the neighbour exchange rows, the band flags and error word,
// the band plan and the colour sequence - lives in one file-scope static device array of a
// fixed size instead of memory allocated per call.  Limits: tiling side N <= 1024, at most
// 2 chains, at most 65536 half-sweeps per call, at most 256 CTAs.
//
// The array (kScratchBytes, about 2.2 MiB) belongs to the library's device code module, so a
// GPU holds it from the moment that module is loaded on it until the process exits.  With
// CUDA's lazy module loading (the default) that happens at the first call on the device, which
// also loads the sweep kernels: a caller that must not see that happen later (inside a timed
// loop, under a memory cap) makes one call with steps = 0 first, which does all of the set-up
// and sweeps nothing, or sets CUDA_MODULE_LOADING=EAGER.  All calls share the array and it
// keeps the last call's contents: each call clears the exchange rows, flags and error word it
// relies on, and calls that overlap on the GPU (for example on two streams at once) race on
// it, so callers must order them.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "domino_persist.h"
#include "domino_rules.h"
#include "rt_internal.h"

namespace rt {
namespace {

constexpr int kMaxSide = 1024;
constexpr int kMaxPitch = kMaxSide / 2;  // P of a 1024 side: 512, a multiple of 16
constexpr int kMaxChains = 2;
constexpr int kMaxBands = 256;
constexpr int64_t kMaxSteps = 65536;

// Scratch layout (byte offsets, each 256-aligned).
constexpr size_t kXbufBytes = (size_t)2 * kMaxBands * 2 * kMaxChains * kMaxPitch * 2;  // 2 MiB
constexpr size_t kOffFlags = kXbufBytes;
constexpr size_t kFlagsBytes = 2048;  // kMaxBands + 1 words, padded
constexpr size_t kOffBands = kOffFlags + kFlagsBytes;
constexpr size_t kBandsBytes = (size_t)kMaxBands * sizeof(DmBand);
constexpr size_t kOffRows = kOffBands + kBandsBytes;
constexpr size_t kRowsBytes = ((size_t)2 * (kMaxSide + 1) * sizeof(int) + 255) / 256 * 256;
constexpr size_t kOffColours = kOffRows + kRowsBytes;
constexpr size_t kScratchBytes = kOffColours + (size_t)kMaxSteps;

static __device__ __align__(256) unsigned char g_sweep_scratch[kScratchBytes];

// Device address of g_sweep_scratch on the current device.  Taken on every call, with the
// device current: it costs nothing once the module is loaded, allocates nothing, and stays
// right after a cudaDeviceReset, which reloads the module at another address.
rt_status scratch_address(unsigned char** out) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_sweep_scratch);
  if (e != cudaSuccess || !p)
    return fail(RT_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
  *out = static_cast<unsigned char*>(p);
  return RT_OK;
}

#define NOALLOC_CUDA(expr)                                                              \
  do {                                                                                  \
    cudaError_t _e = (expr);                                                            \
    if (_e != cudaSuccess)                                                              \
      return fail(RT_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e));     \
  } while (0)

}  // namespace
}  // namespace rt

using namespace rt;

extern "C" RT_API rt_status rt_dm_sweep_noalloc(uint8_t* dev_chains, void* dev_generators, int32_t n_side,
                                                int32_t n_chains, const uint8_t* colours, int64_t steps,
                                                uint64_t fast_seed, int64_t h0, const rt_walk_opts* opts) {
  clear_error();
  rt_walk_opts o;
  rt_walk_opts_default(&o);
  if (opts) o = *opts;
  if (n_side < 6 || n_side % 2 || n_side > kMaxSide)
    return fail(RT_ERR_INVALID_ARGUMENT, "sweep_noalloc: tiling side must be even, >= 6 and <= 1024");
  if (n_chains < 1 || n_chains > kMaxChains) return fail(RT_ERR_INVALID_ARGUMENT, "sweep_noalloc: 1 or 2 chains");
  if (steps < 0 || steps > kMaxSteps)
    return fail(RT_ERR_INVALID_ARGUMENT, "sweep_noalloc: steps must be in [0, 65536] per call");
  if (!dev_chains || ((uintptr_t)dev_chains & 15))
    return fail(RT_ERR_INVALID_ARGUMENT, "sweep_noalloc: chains must be a 16-byte aligned device pointer");
  if (o.rng_mode != RT_RNG_TINYMT && o.rng_mode != RT_RNG_FAST)
    return fail(RT_ERR_INVALID_ARGUMENT, "sweep_noalloc: TinyMT or fast mode only");
  if (o.rng_mode == RT_RNG_TINYMT && (!dev_generators || ((uintptr_t)dev_generators & 15) || (steps > 0 && !colours)))
    return fail(RT_ERR_INVALID_ARGUMENT, "sweep_noalloc: TinyMT mode needs generators (16-byte aligned) and colours");
  if (o.rng_mode == RT_RNG_FAST && (o.fast_stream >= 65536u || h0 < -((int64_t)1 << 47) || h0 + steps > ((int64_t)1 << 47)))
    return fail(RT_ERR_INVALID_ARGUMENT, "sweep_noalloc: fast stream or half-sweep index out of range");
  if (o.tinymt_params) return fail(RT_ERR_INVALID_ARGUMENT, "sweep_noalloc: per-generator parameter tables are not supported");
  DmRule rule{};
  const char* err = nullptr;
  if (!dm_rule_build(o.rule, o.rng_mode, o.weight_a, o.weight_b, &rule, &err))
    return fail(RT_ERR_INVALID_ARGUMENT, std::string("sweep_noalloc: ") + err);

  // Set-up, also for steps = 0 (the warm-up call): the device, the scratch address (which
  // loads the module holding the array and the kernels), the plan and the kernel attributes.
  int dev = 0, sms = 0, coop = 0, optin = 0;
  NOALLOC_CUDA(cudaGetDevice(&dev));
  NOALLOC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  NOALLOC_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  NOALLOC_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  if (!coop) return fail(RT_ERR_CUDA, "sweep_noalloc: device lacks cooperative launch");
  unsigned char* scratch = nullptr;
  if (rt_status st = scratch_address(&scratch)) return st;

  // Plan: every site of rows 1..N-2, columns 1..N/2-2 is a unit, so windows span whole rows
  // and the sweep equals the reference's for any input.
  const int N = n_side, H = N / 2, P = (H + 15) / 16 * 16;
  std::vector<uint8_t> cand((size_t)N * H, 0);
  for (int i = 1; i <= N - 2; ++i)
    for (int m = 1; m <= H - 2; ++m) cand[(size_t)i * H + m] = 1;
  PersistPlan plan;
  if (rt_status st = plan.build(cand, N, P, o.rng_mode, n_chains, std::min(sms, kMaxBands), (size_t)optin - 1024))
    return st;
  if (!plan.ok) return fail(RT_ERR_INVALID_ARGUMENT, "sweep_noalloc: " + plan.why);
  void* kernel = dm_persist_kernel_ptr(o.rng_mode, plan.K, false, n_chains, false);
  NOALLOC_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)plan.smem_bytes));
  int per_sm = 0;
  NOALLOC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kPersistThreads, plan.smem_bytes));
  const int nbands = (int)plan.bands.size();
  if ((int64_t)per_sm * sms < nbands) return fail(RT_ERR_CUDA, "sweep_noalloc: bands cannot all be resident");
  if (steps == 0) return RT_OK;

  cudaStream_t stream = (cudaStream_t)o.cuda_stream;
  std::vector<int> rows((size_t)2 * (kMaxSide + 1), 0);
  std::copy(plan.row_lo.begin(), plan.row_lo.end(), rows.begin());
  std::copy(plan.row_prefix.begin(), plan.row_prefix.end(), rows.begin() + (kMaxSide + 1));
  NOALLOC_CUDA(cudaMemcpyAsync(scratch + kOffBands, plan.bands.data(), nbands * sizeof(DmBand), cudaMemcpyHostToDevice,
                               stream));
  NOALLOC_CUDA(cudaMemcpyAsync(scratch + kOffRows, rows.data(), rows.size() * sizeof(int), cudaMemcpyHostToDevice, stream));
  if (o.rng_mode == RT_RNG_TINYMT)
    NOALLOC_CUDA(cudaMemcpyAsync(scratch + kOffColours, colours, (size_t)steps, cudaMemcpyHostToDevice, stream));
  NOALLOC_CUDA(cudaMemsetAsync(scratch + kOffFlags, 0, kFlagsBytes, stream));
  NOALLOC_CUDA(cudaMemsetAsync(scratch, 0, dm_xbuf_bytes(nbands, n_chains, P), stream));  // no stale tags

  PersistArgs a{};
  a.base = dev_chains;
  a.P = P;
  a.cols = H - 2;
  a.colour_stride = (size_t)N * P;
  a.chain_stride = 2 * a.colour_stride;
  a.nch = n_chains;
  a.tmt = static_cast<uint4*>(dev_generators);
  a.tmt_params = nullptr;
  a.bands = reinterpret_cast<const DmBand*>(scratch + kOffBands);
  a.nbands = nbands;
  a.row_lo = reinterpret_cast<const int*>(scratch + kOffRows);
  a.row_prefix = reinterpret_cast<const int*>(scratch + kOffRows) + (kMaxSide + 1);
  a.rule = rule;
  a.xbuf = scratch;
  a.flags = reinterpret_cast<unsigned*>(scratch + kOffFlags);
  a.error = reinterpret_cast<int*>(scratch + kOffFlags) + nbands;
  a.max_spin = 1L << 22;
  a.steps = steps;
  a.h0 = h0;
  a.fast_seed = fast_seed;
  a.fast_stream = o.fast_stream;
  a.colours = scratch + kOffColours;
  void* args[] = {&a};
  NOALLOC_CUDA(cudaLaunchCooperativeKernel(kernel, dim3((unsigned)nbands), dim3(kPersistThreads), args, plan.smem_bytes,
                                           stream));
  int err_word = 0;
  NOALLOC_CUDA(cudaMemcpyAsync(&err_word, a.error, sizeof(int), cudaMemcpyDeviceToHost, stream));
  NOALLOC_CUDA(cudaStreamSynchronize(stream));
  if (err_word) return fail(RT_ERR_TIMEOUT, "sweep_noalloc: a band wait gave up (neighbour never published)");
  return RT_OK;
}
