// pdl.cuh -- programmatic dependent launch for the image encoders.
//
// An encoder launched with programmatic stream serialization may have its
// CTAs scheduled while the previous kernel in the stream is still draining
// (once every CTA of that kernel has signalled), runs its prologue (barriers,
// tables in shared memory) there, and waits in griddepcontrol.wait until the
// previous kernel has completed and its memory is visible before it touches
// global memory.  After a kernel that never signals -- any kernel that is not
// one of these encoders -- it starts at that kernel's completion, as an
// ordinary launch does.  Each encoder signals at its start, so back-to-back
// encodes overlap one grid's tail with the next grid's launch.
#pragma once
#include <cuda_runtime.h>

namespace goofy_gpu {

// Allows the next kernel in the stream to be scheduled once every CTA of this
// grid has executed it (or exited).
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Waits until the kernels this grid depends on have completed and their memory
// operations are visible; returns at once for a grid without the dependency.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                       Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

}  // namespace goofy_gpu
