// cuRAND MTGP32 mode of the domino sweep: the random stream of the reference's CUDA build.
//
// The reference's CUDA Walk (src/Domino/DominoTiler.cpp:51-66) launches its rotate kernel
// on 8 x 8 blocks over the (N-2) x (N/2-2) flip candidates (row i from the x index, column
// j from the y index, dominokernel.cu:10-11), gives block (bx, by) the MTGP32 generator
// number bx * gridDim.y + by (dominokernel.cu:14), seeds generator k with seed + k through
// curandMakeMTGP32KernelState with the mtgp32dc_params_fast_11213 parameter set
// (DominoTiler.cpp:62-65, LoadMTGP :239-242), and has every thread of a block draw one
// curand_uniform from that generator per launch, out-of-range threads included, before the
// bounds test.  This file keeps exactly that geometry so the draws are the reference's; the
// generator itself is cuRAND's, called through its public device and host API.  The flip
// decision uses the rule's acceptance intervals over the float draw's bit pattern
// (dm_rule_build, RT_RNG_MTGP), and the passive colour is rebuilt by the sampler's word
// kernel, as in the other modes.
#include <curand_kernel.h>
#include <curand_mtgp32_host.h>
#include <curand_mtgp32dc_p_11213.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "domino_sweep.h"
#include "pdl.cuh"
#include "rt_internal.h"

#define RT_CUDA(expr)                                                                   \
  do {                                                                                  \
    cudaError_t _e = (expr);                                                            \
    if (_e != cudaSuccess)                                                              \
      return fail(RT_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e));     \
  } while (0)

namespace rt {

namespace {

// One half-sweep's rotation of colour t: every thread of every block draws once from its
// block's generator, then the in-range ones decide their site in every active chain.
__global__ void __launch_bounds__(kMtgpBlock* kMtgpBlock) k_rotate_mtgp(DmView v, int t, DmRule rule,
                                                                         curandStateMtgp32* states) {
  pdl_begin();
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int m = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const float rd = curand_uniform(states + blockIdx.x * gridDim.y + blockIdx.y);
  if (i > v.rows || m > v.cols) return;
  const uint32_t u = __float_as_uint(rd);
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

// The draws of one launch on a rows x cols grid, row-major (row x from the x index, column
// y from the y index): what the rotate kernels of both tilers decide with.
__global__ void __launch_bounds__(kMtgpBlock* kMtgpBlock) k_mtgp_draws(curandStateMtgp32* states, int rows, int cols,
                                                                        float* out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const float rd = curand_uniform(states + blockIdx.x * gridDim.y + blockIdx.y);
  if (x >= rows || y >= cols) return;
  out[(size_t)x * cols + y] = rd;
}

// The kernel parameters of the parameter set (curandMakeMTGP32Constants), made once per
// device and kept for the process, as the reference's LoadMTGP keeps its copy.
rt_status kernel_params(mtgp32_kernel_params** out) {
  static std::mutex mu;
  static std::vector<mtgp32_kernel_params*> per_device;
  int dev = 0;
  RT_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  if ((int)per_device.size() <= dev) per_device.resize(dev + 1, nullptr);
  if (!per_device[dev]) {
    mtgp32_kernel_params* kp = nullptr;
    RT_CUDA(cudaMalloc(&kp, sizeof(mtgp32_kernel_params)));
    if (curandMakeMTGP32Constants(mtgp32dc_params_fast_11213, kp) != CURAND_STATUS_SUCCESS) {
      cudaFree(kp);
      return fail(RT_ERR_CUDA, "curandMakeMTGP32Constants failed");
    }
    per_device[dev] = kp;
  }
  *out = per_device[dev];
  return RT_OK;
}

}  // namespace

size_t mtgp_state_bytes(int count) { return (size_t)count * sizeof(curandStateMtgp32); }

rt_status mtgp_seed(void* states, int count, int64_t seed, cudaStream_t stream) {
  mtgp32_kernel_params* kp = nullptr;
  if (rt_status st = kernel_params(&kp)) return st;
  // curandMakeMTGP32KernelState copies each state with a blocking cudaMemcpy, which does not
  // wait for kernels still queued on a non-blocking stream: drain the stream first.
  RT_CUDA(cudaStreamSynchronize(stream));
  curandStateMtgp32* s = static_cast<curandStateMtgp32*>(states);
  int dev = 0;
  RT_CUDA(cudaGetDevice(&dev));
  // Generator k is seeded seed + k, one state per call (DominoTiler.cpp:63-65,
  // LozengeTiler.cpp:78-80); large grids split the calls over host threads.
  const int nthreads = count < 512 ? 1 : (int)std::min(16u, std::max(1u, std::thread::hardware_concurrency()));
  std::vector<int> bad(nthreads, 0);
  auto work = [&](int tid) {
    if (cudaSetDevice(dev) != cudaSuccess) {
      bad[tid] = 1;
      return;
    }
    for (int k = tid; k < count; k += nthreads)
      if (curandMakeMTGP32KernelState(s + k, mtgp32dc_params_fast_11213, kp, 1,
                                      (unsigned long long)(seed + (int64_t)k)) != CURAND_STATUS_SUCCESS) {
        bad[tid] = 1;
        return;
      }
  };
  if (nthreads == 1) {
    work(0);
  } else {
    std::vector<std::thread> th;
    for (int k = 0; k < nthreads; ++k) th.emplace_back(work, k);
    for (auto& x : th) x.join();
  }
  if (std::any_of(bad.begin(), bad.end(), [](int b) { return b != 0; }))
    return fail(RT_ERR_CUDA, "curandMakeMTGP32KernelState failed");
  return RT_OK;
}

rt_status mtgp_rotate(const DmView& v, int t, const DmRule& rule, void* states, cudaStream_t stream) {
  const MtgpGrid g = mtgp_grid(v.rows, v.cols);
  const cudaError_t e = pdl_launch(k_rotate_mtgp, dim3(g.gx, g.gy), dim3(kMtgpBlock, kMtgpBlock), stream, v, t, rule,
                                   static_cast<curandStateMtgp32*>(states));
  if (e != cudaSuccess) return fail(RT_ERR_CUDA, std::string("k_rotate_mtgp: ") + cudaGetErrorString(e));
  return RT_OK;
}

rt_status mtgp_draws_grid(int rows, int cols, int64_t seed, int64_t launches, float* out) {
  const size_t per = (size_t)rows * cols;
  const MtgpGrid g = mtgp_grid(rows, cols);
  cudaStream_t stream = nullptr;
  RT_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  void* states = nullptr;
  float* d_out = nullptr;
  rt_status st = RT_OK;
  if (cudaMalloc(&states, mtgp_state_bytes(g.count())) != cudaSuccess ||
      cudaMalloc(&d_out, per * sizeof(float)) != cudaSuccess)
    st = fail(RT_ERR_OUT_OF_MEMORY, "mtgp_draws: device allocation failed");
  if (!st) st = mtgp_seed(states, g.count(), seed, stream);
  for (int64_t k = 0; !st && k < launches; ++k) {
    k_mtgp_draws<<<dim3(g.gx, g.gy), dim3(kMtgpBlock, kMtgpBlock), 0, stream>>>(
        static_cast<curandStateMtgp32*>(states), rows, cols, d_out);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(out + k * per, d_out, per * sizeof(float), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) st = fail(RT_ERR_CUDA, std::string("mtgp_draws: ") + cudaGetErrorString(e));
  }
  if (d_out) cudaFree(d_out);
  if (states) cudaFree(states);
  cudaStreamDestroy(stream);
  return st;
}

}  // namespace rt

using namespace rt;

extern "C" {

RT_API rt_status rt_domino_mtgp_draws(int32_t n_side, int64_t seed, int64_t launches, float* out) {
  clear_error();
  if (n_side < 6 || n_side % 2 || n_side > 32768 || launches < 0 || (launches > 0 && !out))
    return fail(RT_ERR_INVALID_ARGUMENT, "mtgp_draws: even n_side in [6, 32768], launches >= 0, out not NULL");
  return mtgp_draws_grid(n_side - 2, n_side / 2 - 2, seed, launches, out);
}

}  // extern "C"
