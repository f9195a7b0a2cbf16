// Programmatic dependent launch for chains of short dependent kernels (the
// PCG iterations and the V-cycle levels): a kernel launched with
// launch_pdl may be scheduled while its predecessor in the stream still
// runs its last wave. Every such kernel calls pdl_sync() before it reads
// anything the predecessor wrote: griddepcontrol.wait returns once the
// predecessor grid has completed and its memory is visible, so the chain
// keeps stream order. griddepcontrol.launch_dependents, issued first, lets
// the successor be scheduled as soon as every block of this grid has
// started. Both are no-ops for a kernel launched without the attribute.
#ifndef SPG_PDL_CUH
#define SPG_PDL_CUH

#include <utility>

#include <cuda_runtime.h>

namespace spg {

__device__ __forceinline__ void pdl_sync() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

template <class... KArgs, class... Args>
inline void launch_pdl(void (*kernel)(KArgs...), unsigned grid, unsigned block, cudaStream_t s, Args &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

}  // namespace spg

#endif
