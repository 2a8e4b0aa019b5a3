// Programmatic dependent launch for the kernels of one sweep (draw ->
// warm start -> primary Newton -> fallback -> moments): each is launched
// with programmatic stream serialisation, so its blocks are placed while its
// predecessor drains.  Every such kernel starts with pdl_wait()
// (griddepcontrol.wait: returns once the predecessor grid has completed and
// its memory is visible) before it touches global memory, then calls
// pdl_trigger() (griddepcontrol.launch_dependents) so that its own
// successor may be placed.  Launched without the attribute, both are no-ops.
#pragma once
#include <cuda_runtime.h>

#include <utility>

namespace sp {

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

struct ChainedLaunch {
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg;
    ChainedLaunch(dim3 grid, dim3 block, size_t smem, cudaStream_t st) : cfg{} {
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.gridDim = grid;
        cfg.blockDim = block;
        cfg.dynamicSmemBytes = smem;
        cfg.stream = st;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
    }
};

// Launch `kernel` (which must begin with pdl_wait()) chained to the previous
// work of stream st.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_chained(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                                  Args&&... args) {
    ChainedLaunch L(grid, block, smem, st);
    return cudaLaunchKernelEx(&L.cfg, kernel, std::forward<Args>(args)...);
}

}  // namespace sp
