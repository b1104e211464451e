// Programmatic dependent launch for chains of short dependent kernels (one kernel per
// step): the next kernel is launched while the current one runs, and each kernel waits for
// its predecessor's completion (and memory) at griddepcontrol.wait before touching device
// state.  Every kernel launched through pdl_launch must call pdl_begin() before its first
// access to data the previous kernel wrote.
#pragma once
#include <cuda_runtime.h>

namespace rt {

// Waits for the preceding grid in the stream to complete, then lets the next grid launch.
__device__ __forceinline__ void pdl_begin() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" :::);
}

template <class... KArgs, class... Args>
inline cudaError_t pdl_launch(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t stream, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

}  // namespace rt
