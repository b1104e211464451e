// Device tables of per-generator TinyMT parameters (rt_internal.h: tmt_param_table).
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "rng.cuh"
#include "rt_internal.h"

namespace rt {

rt_status tmt_param_table(const rt_walk_opts& o, int64_t count, uint4** out, cudaStream_t s) {
  *out = nullptr;
  if (!o.tinymt_params) return RT_OK;
  if (o.tinymt_params_count < 0) return fail(RT_ERR_INVALID_ARGUMENT, "negative TinyMT parameter count");
  std::vector<uint4> p((size_t)count);
  for (int64_t k = 0; k < count; ++k)
    p[(size_t)k] = k < o.tinymt_params_count ? make_uint4(o.tinymt_params[3 * k], o.tinymt_params[3 * k + 1],
                                                          o.tinymt_params[3 * k + 2], 0)
                                             : make_uint4(kTmtMat1, kTmtMat2, kTmtTmat, 0);
  uint4* d = nullptr;
  cudaError_t e = cudaMalloc(&d, (size_t)count * sizeof(uint4));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(RT_ERR_OUT_OF_MEMORY, std::string("TinyMT parameter table: ") + cudaGetErrorString(e));
  }
  e = cudaMemcpyAsync(d, p.data(), (size_t)count * sizeof(uint4), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    cudaFree(d);
    return fail(RT_ERR_CUDA, std::string("TinyMT parameter table: ") + cudaGetErrorString(e));
  }
  *out = d;
  return RT_OK;
}

}  // namespace rt
