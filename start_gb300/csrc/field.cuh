// Stamp check of the lazily computed per-tet field (FieldArgs), shared by the
// FP64 and the mixed-form kernels. The stamp is read from L2, so a stamp that
// another SM swapped in this kernel is seen; the lane whose compare-and-swap
// succeeds computes the tet, every other lane skips it.
#ifndef SPG_FIELD_CUH
#define SPG_FIELD_CUH

#include <cstdint>

namespace spg {

template <class F>
__device__ __forceinline__ void refresh_tet(uint32_t *stamp, uint32_t epoch, int t, F compute) {
    const uint32_t old = __ldcg(stamp + t);
    if (old == epoch) return;
    if (atomicCAS(stamp + t, old, epoch) == old) compute(t);
}

}  // namespace spg

#endif
