// Programmatic dependent launch for the kernels of a contraction chain.
//
// A kernel launched with launch_pdl may start while the previous grid on its
// stream is still running: each CTA first lets the next grid launch
// (pdl_trigger: griddepcontrol.launch_dependents), may read data that no
// kernel writes (its work list, the operand view tables of its plan), and
// then waits (pdl_wait: griddepcontrol.wait) until the previous grid has
// completed and its writes are visible, before it reads an operand or writes
// anything.  The next launch's set-up, CTA rasterisation and work-list
// latency thus overlap this one's tail, while every access to data a kernel
// writes stays ordered as on a plain stream.  Without the launch attribute
// (or after a non-PDL kernel) the wait returns at once; a second wait in the
// same thread returns at once too.
#pragma once
#include <cuda_runtime.h>

#include "../engine/engine.h"

namespace tn {

__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                       Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  TN_CUDA(cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...));
}

}  // namespace tn
