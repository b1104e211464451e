// Stream-ordered device memory for the library's per-call buffers (samplers and the resident
// engine's plan).  One memory pool per device keeps freed blocks up to a release threshold,
// so a call that frees and then allocates the sizes of the previous call (the CFTP entry
// points do this every call) makes no driver allocation and, unlike cudaFree, no device-wide
// synchronisation.  Blocks are allocated and freed in the order of the stream that uses them.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "rt_internal.h"

namespace rt {
namespace {

constexpr int kMaxDevices = 128;
// Bytes a pool keeps reserved while idle: enough for the samplers of an order-2048 domain.
constexpr uint64_t kPoolKeepBytes = 2ull << 30;

std::mutex g_pool_mu;
cudaMemPool_t g_pool[kMaxDevices] = {};

rt_status pool_of(cudaMemPool_t* out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return fail(RT_ERR_CUDA, "no CUDA device: the sweep has no CPU fallback");
  }
  std::lock_guard<std::mutex> lock(g_pool_mu);
  if (!g_pool[dev]) {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t p = nullptr;
    cudaError_t e = cudaMemPoolCreate(&p, &props);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(RT_ERR_CUDA, std::string("cudaMemPoolCreate: ") + cudaGetErrorString(e));
    }
    uint64_t keep = kPoolKeepBytes;
    cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
    g_pool[dev] = p;
  }
  *out = g_pool[dev];
  return RT_OK;
}

}  // namespace

rt_status dev_alloc(void** p, size_t bytes, cudaStream_t s) {
  *p = nullptr;
  cudaMemPool_t pool = nullptr;
  if (rt_status st = pool_of(&pool)) return st;
  cudaError_t e = cudaMallocFromPoolAsync(p, bytes, pool, s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return fail(e == cudaErrorMemoryAllocation ? RT_ERR_OUT_OF_MEMORY : RT_ERR_CUDA,
                std::string("device allocation: ") + cudaGetErrorString(e));
  }
  return RT_OK;
}

void dev_free(void* p, cudaStream_t s) {
  if (p) cudaFreeAsync(p, s);
}

}  // namespace rt
