// pdl.cuh -- programmatic dependent launch for the solver's kernel chain.
//
// Every pass is a grid-wide dependency of the one before, so the kernels of an
// iteration are a strict chain.  Launched with programmatic stream
// serialisation, a kernel's CTAs may be scheduled while its predecessor's last
// CTAs are still running; the kernel then waits in griddepcontrol.wait until
// the predecessor has completed and its writes are visible, before it touches
// memory.  This hides the launch gap between passes (17 launches per
// iteration); the arithmetic and its order are unchanged.
#pragma once

#include <cuda_runtime.h>

namespace e2d {

// First statement of every kernel launched through launch_chained.  A no-op
// when the kernel was launched without the attribute.
__device__ __forceinline__ void wait_prior_grid() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline void launch_chained_smem(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                                Args... args) {
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
    cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

template <typename... KArgs, typename... Args>
inline void launch_chained(void (*kern)(KArgs...), dim3 grid, dim3 block, cudaStream_t s, Args... args) {
    launch_chained_smem(kern, grid, block, 0, s, args...);
}

}  // namespace e2d
