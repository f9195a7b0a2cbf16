// SELL-32 sparse row times vector, shared by the PCG and AMG kernels.
#ifndef SPG_SELL_CUH
#define SPG_SELL_CUH

#include <cstdint>

namespace spg {

// Row i of A x in SELL-32 storage: rows are grouped in slices of 32 (one
// warp), each slice padded to its longest row and stored column-major, so
// lane l of a warp reads entry j of its row at slice_ptr[s] + 32 j + l and a
// warp's 32 loads of one j are contiguous. Padding entries have value 0.
// The slice width is the same for the 32 lanes of a warp, so the loop below
// branches uniformly: eight entries per trip with all their column and value
// loads issued before the gathers, then the remaining (< 8) entries the same
// way, so a row costs two dependent load stages per eight entries and no
// FMA is spent on padding beyond the slice width.
// xf(c) supplies x[c]: a plain gather, or a value formed from several
// vectors at the gathered column (a fused vector update).
template <class T, class X>
__device__ __forceinline__ T spmv_row_sell_f(const int64_t *__restrict__ slice_ptr, const int32_t *__restrict__ scol,
                                             const T *__restrict__ sval, X xf, int64_t i) {
    const int64_t s = i >> 5;
    const int64_t base = __ldg(slice_ptr + s) + (i & 31);
    const int w = int((__ldg(slice_ptr + s + 1) - __ldg(slice_ptr + s)) >> 5);
    T a0 = T(0), a1 = T(0);
    int j = 0;
    for (; j + 8 <= w; j += 8) {
        int32_t c[8];
        T v[8], xv[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            c[u] = __ldg(scol + base + 32 * (j + u));
            v[u] = __ldg(sval + base + 32 * (j + u));
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) xv[u] = xf(c[u]);
#pragma unroll
        for (int u = 0; u < 8; u += 2) {
            a0 = fma(v[u], xv[u], a0);
            a1 = fma(v[u + 1], xv[u + 1], a1);
        }
    }
    const int rem = w - j;  // 0..7, warp-uniform
    if (rem > 0) {
        int32_t c[7];
        T v[7], xv[7];
#pragma unroll
        for (int u = 0; u < 7; ++u)
            if (u < rem) {
                c[u] = __ldg(scol + base + 32 * (j + u));
                v[u] = __ldg(sval + base + 32 * (j + u));
            }
#pragma unroll
        for (int u = 0; u < 7; ++u)
            if (u < rem) xv[u] = xf(c[u]);
#pragma unroll
        for (int u = 0; u < 7; ++u)
            if (u < rem) {
                if (u & 1)
                    a1 = fma(v[u], xv[u], a1);
                else
                    a0 = fma(v[u], xv[u], a0);
            }
    }
    return a0 + a1;
}

template <class T>
__device__ __forceinline__ T spmv_row_sell(const int64_t *__restrict__ slice_ptr, const int32_t *__restrict__ scol,
                                           const T *__restrict__ sval, const T *__restrict__ x, int64_t i) {
    return spmv_row_sell_f<T>(slice_ptr, scol, sval, [x](int32_t c) { return __ldg(x + c); }, i);
}

}  // namespace spg

#endif
