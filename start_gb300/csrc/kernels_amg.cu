// V-cycle of the smoothed-aggregation AMG preconditioner (hierarchy from
// amg_setup.cpp). Per level: Jacobi-Chebyshev pre-smoothing from a zero
// guess, residual, restriction R = P^T, the coarser level, prolongation, and
// post-smoothing with the same polynomial (degree 1, damped Jacobi, or
// degree 2, per level); the coarsest level multiplies by its dense inverse.
// Pre- and post-smoother are the same polynomial in D^-1 A, so the V-cycle
// is a symmetric positive definite operator and CG stays CG.
// Operators with short rows are stored SELL-32 with one thread per row (level
// 0 shares the solver's matrix); long rows (coarse operators, restriction)
// CSR with 4-32 lanes per row. No atomics, so z = M^-1 r is deterministic.
#include "pdl.cuh"
#include "sell.cuh"
#include "spg_internal.h"

namespace spg {

namespace {

constexpr int kT = 256;

// converged: 1 or 2 (plain PCG), or 3 (inner cap of the mixed form)
// (Every V-cycle kernel starts here: pdl_sync orders it after its predecessor.)
__device__ __forceinline__ bool done(const PcgScalars *sc) {
    pdl_sync();
    return sc && *(volatile const int *)&sc->converged;
}

// Row `row` of M x, xf(c) = x[c]. G = 0: SELL-32, the calling thread owns
// the row. G > 0: CSR, the G lanes of a group (lane = lane index within the
// group) stride over the row's entries and a butterfly over the group leaves
// the sum in every lane of the group.
template <class T, int G, class X>
__device__ __forceinline__ T mat_row_f(const DevSellT<T> &M, X xf, int64_t row, int lane) {
    if constexpr (G == 0) {
        return spmv_row_sell_f<T>(M.slice_ptr, M.scol, M.sval, xf, row);
    } else {
        const int64_t k0 = __ldg(M.slice_ptr + row), k1 = __ldg(M.slice_ptr + row + 1);
        T a0 = T(0), a1 = T(0);
        int64_t k = k0 + lane;
        for (; k + 3 * G < k1; k += 4 * G) {  // four entries per lane in flight
            const int32_t c0 = __ldg(M.scol + k), c1 = __ldg(M.scol + k + G);
            const int32_t c2 = __ldg(M.scol + k + 2 * G), c3 = __ldg(M.scol + k + 3 * G);
            const T v0 = __ldg(M.sval + k), v1 = __ldg(M.sval + k + G);
            const T v2 = __ldg(M.sval + k + 2 * G), v3 = __ldg(M.sval + k + 3 * G);
            const T x0 = xf(c0), x1 = xf(c1), x2 = xf(c2), x3 = xf(c3);
            a0 = fma(v0, x0, a0);
            a1 = fma(v1, x1, a1);
            a0 = fma(v2, x2, a0);
            a1 = fma(v3, x3, a1);
        }
        // the last (at most three) entries of this lane: their column and value
        // loads issued together, then the gathers, then the sums
        int32_t cr[3];
        T vr[3], xr[3];
#pragma unroll
        for (int u = 0; u < 3; ++u) {
            const int64_t kk = k + int64_t(u) * G;
            cr[u] = kk < k1 ? __ldg(M.scol + kk) : -1;
            vr[u] = kk < k1 ? __ldg(M.sval + kk) : T(0);
        }
#pragma unroll
        for (int u = 0; u < 3; ++u) xr[u] = cr[u] >= 0 ? xf(cr[u]) : T(0);
#pragma unroll
        for (int u = 0; u < 3; ++u)
            if (cr[u] >= 0) a0 = fma(vr[u], xr[u], a0);
        T s = a0 + a1;
#pragma unroll
        for (int off = G / 2; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off, G);
        return s;
    }
}

// Thread -> (row, lane within the row's group); `own`: this thread writes the row.
template <int G>
__device__ __forceinline__ void row_of(int64_t n, int64_t &row, int &lane, bool &own) {
    const int64_t t = int64_t(blockIdx.x) * kT + threadIdx.x;
    if constexpr (G == 0) {
        row = t;
        lane = 0;
    } else {
        row = t / G;
        lane = int(t % G);
    }
    own = row < n && lane == 0;
}

// Every lane of a warp joins the group shuffles; rows past n read nothing.
template <class T, int G, class X>
__device__ __forceinline__ T mat_row_safe_f(const DevSellT<T> &M, X xf, int64_t row, int lane, int64_t n) {
    if constexpr (G == 0) {
        return row < n ? mat_row_f<T, 0>(M, xf, row, 0) : T(0);
    } else {
        if (row >= n) {
            T s = T(0);
#pragma unroll
            for (int off = G / 2; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off, G);
            return s;
        }
        return mat_row_f<T, G>(M, xf, row, lane);
    }
}

template <class T, int G>
__device__ __forceinline__ T mat_row_safe(const DevSellT<T> &M, const T *__restrict__ x, int64_t row, int lane,
                                          int64_t n) {
    return mat_row_safe_f<T, G>(M, [x](int32_t c) { return __ldg(x + c); }, row, lane, n);
}

// The first smoothing step from x = 0, x0 = D^-1 b / theta. The FP32
// V-cycle forms it where it is read (k_resid_j, k_prolong_j) instead of
// storing it; the FP64 V-cycle stores it (k_jacobi0), because forming it at
// every gathered column would triple the FP64 work of the residual.
template <class T>
__device__ __forceinline__ T jacobi0(const AmgLevelDevT<T> &L, const T *__restrict__ b, int64_t i) {
    return T(L.inv_theta) * (__ldg(L.dinv + i) * __ldg(b + i));
}

// x = D^-1 b / theta (degree 1, FP64 V-cycle)
template <class T>
__global__ void __launch_bounds__(kT) k_jacobi0(const AmgLevelDevT<T> L, const T *__restrict__ b, T *__restrict__ x,
                                                const PcgScalars *sc) {
    if (done(sc)) return;
    const int64_t i = int64_t(blockIdx.x) * kT + threadIdx.x;
    if (i < L.n) x[i] = jacobi0(L, b, i);
}

// x = d = D^-1 b / theta (first Chebyshev step from x = 0)
template <class T>
__global__ void __launch_bounds__(kT) k_cheb0(const AmgLevelDevT<T> L, const T *__restrict__ b, T *__restrict__ x,
                                              const PcgScalars *sc) {
    if (done(sc)) return;
    const int64_t i = int64_t(blockIdx.x) * kT + threadIdx.x;
    if (i >= L.n) return;
    const T v = T(L.inv_theta) * (L.dinv[i] * b[i]);
    x[i] = v;
    L.d[i] = v;
}

// r = b - A x_in; d = ca d + cb D^-1 r; x_out = x_in + d
template <class T, int G>
__global__ void __launch_bounds__(kT) k_cheb_step(const AmgLevelDevT<T> L, const T *__restrict__ b,
                                                  const T *__restrict__ xin, T *__restrict__ xout, double ca,
                                                  double cb, const PcgScalars *sc) {
    if (done(sc)) return;
    int64_t i;
    int lane;
    bool own;
    row_of<G>(L.n, i, lane, own);
    const T ax = mat_row_safe<T, G>(L.A, xin, i, lane, L.n);
    if (!own) return;
    const T r = b[i] - ax;
    const T d = T(ca) * L.d[i] + T(cb) * (L.dinv[i] * r);
    L.d[i] = d;
    xout[i] = xin[i] + d;
}

template <class T, int G>
__global__ void __launch_bounds__(kT) k_resid(const AmgLevelDevT<T> L, const T *__restrict__ b,
                                              const T *__restrict__ xin, const PcgScalars *sc) {
    if (done(sc)) return;
    int64_t i;
    int lane;
    bool own;
    row_of<G>(L.n, i, lane, own);
    const T ax = mat_row_safe<T, G>(L.A, xin, i, lane, L.n);
    if (own) L.r[i] = b[i] - ax;
}

// Degree 1: r = b - A x0 with x0 = D^-1 b / theta formed at each column.
template <class T, int G>
__global__ void __launch_bounds__(kT) k_resid_j(const AmgLevelDevT<T> L, const T *__restrict__ b,
                                                const PcgScalars *sc) {
    if (done(sc)) return;
    int64_t i;
    int lane;
    bool own;
    row_of<G>(L.n, i, lane, own);
    const T *dinv = L.dinv;
    const T it = T(L.inv_theta);
    const T ax = mat_row_safe_f<T, G>(
        L.A, [dinv, b, it](int32_t c) { return it * (__ldg(dinv + c) * __ldg(b + c)); }, i, lane, L.n);
    if (own) L.r[i] = b[i] - ax;
}

// Degree 1: x_out = x0 + P x_coarse (x0 as in k_resid_j)
template <class T, int G>
__global__ void __launch_bounds__(kT) k_prolong_j(const AmgLevelDevT<T> L, const T *__restrict__ b,
                                                  const T *__restrict__ xc, T *__restrict__ xout,
                                                  const PcgScalars *sc) {
    if (done(sc)) return;
    int64_t i;
    int lane;
    bool own;
    row_of<G>(L.P.n, i, lane, own);
    const T v = mat_row_safe<T, G>(L.P, xc, i, lane, L.P.n);
    if (own) xout[i] = jacobi0(L, b, i) + v;
}

// Degree 1 post-smoothing: x_out = x_in + D^-1 (b - A x_in) / theta
template <class T, int G>
__global__ void __launch_bounds__(kT) k_jacobi_step(const AmgLevelDevT<T> L, const T *__restrict__ b,
                                                    const T *__restrict__ xin, T *__restrict__ xout,
                                                    const PcgScalars *sc) {
    if (done(sc)) return;
    int64_t i;
    int lane;
    bool own;
    row_of<G>(L.n, i, lane, own);
    const T ax = mat_row_safe<T, G>(L.A, xin, i, lane, L.n);
    if (!own) return;
    const T r = b[i] - ax;
    xout[i] = xin[i] + T(L.inv_theta) * (L.dinv[i] * r);
}

// b_next = R r
template <class T, int G>
__global__ void __launch_bounds__(kT) k_restrict(const DevSellT<T> R, const T *__restrict__ r, T *__restrict__ bnext,
                                                 const PcgScalars *sc) {
    if (done(sc)) return;
    int64_t i;
    int lane;
    bool own;
    row_of<G>(R.n, i, lane, own);
    const T v = mat_row_safe<T, G>(R, r, i, lane, R.n);
    if (own) bnext[i] = v;
}

// x_out = x_in + P x_coarse
template <class T, int G>
__global__ void __launch_bounds__(kT) k_prolong(const DevSellT<T> P, const T *__restrict__ xin,
                                                const T *__restrict__ xc, T *__restrict__ xout, const PcgScalars *sc) {
    if (done(sc)) return;
    int64_t i;
    int lane;
    bool own;
    row_of<G>(P.n, i, lane, own);
    const T v = mat_row_safe<T, G>(P, xc, i, lane, P.n);
    if (own) xout[i] = xin[i] + v;
}

// x = A_c^-1 b: one warp per row of the dense inverse, fixed-order lane sums.
template <class T>
__global__ void __launch_bounds__(kT) k_coarse(const T *__restrict__ inv, int64_t nc, const T *__restrict__ b,
                                               T *__restrict__ x, const PcgScalars *sc) {
    if (done(sc)) return;
    const int64_t row = (int64_t(blockIdx.x) * kT + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= nc) return;
    T s = T(0);
    for (int64_t k = lane; k < nc; k += 32) s += inv[row * nc + k] * b[k];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if (lane == 0) x[row] = s;
}

inline unsigned blocks_for(int64_t n, int g = 0) {
    const int64_t threads = n * (g > 0 ? g : 1);
    return unsigned((threads + kT - 1) / kT);
}

#define SPG_AMG_DISPATCH(g, KERNEL, GRIDN, ...)                                             \
    switch (g) {                                                                            \
    case 4: launch_pdl(KERNEL<T, 4>, blocks_for(GRIDN, 4), kT, s, __VA_ARGS__); break;     \
    case 8: launch_pdl(KERNEL<T, 8>, blocks_for(GRIDN, 8), kT, s, __VA_ARGS__); break;     \
    case 16: launch_pdl(KERNEL<T, 16>, blocks_for(GRIDN, 16), kT, s, __VA_ARGS__); break;  \
    case 32: launch_pdl(KERNEL<T, 32>, blocks_for(GRIDN, 32), kT, s, __VA_ARGS__); break;  \
    default: launch_pdl(KERNEL<T, 0>, blocks_for(GRIDN, 0), kT, s, __VA_ARGS__); break;    \
    }

// skip_last: level 0's last Jacobi step (x1 = L.x[1] -> z) is left to the
// caller, which fuses it with the PCG's r.z (FP32 degree-1 level 0 only).
template <class T>
void vcycle_level(const AmgDevT<T> &a, int l, const T *b, T *xa, const PcgScalars *sc, cudaStream_t s,
                  bool skip_last = false) {
    const AmgLevelDevT<T> &L = a.lev[l];
    if (l == a.levels - 1) {
        launch_pdl(k_coarse<T>, unsigned((a.nc * 32 + kT - 1) / kT), kT, s, a.coarse_inv, a.nc, b, xa, sc);
        return;
    }
    T *xb = L.x[1];
    const int ga = L.A.g;
    const AmgLevelDevT<T> &N = a.lev[l + 1];
    if (L.degree == 1 && sizeof(T) == 4) {  // x0 = D^-1 b / theta; residual; coarse correction; damped Jacobi
        SPG_AMG_DISPATCH(ga, k_resid_j, L.n, L, b, sc)
        SPG_AMG_DISPATCH(L.R.g, k_restrict, L.R.n, L.R, L.r, N.b, sc)
        vcycle_level<T>(a, l + 1, N.b, N.x[0], sc, s);
        SPG_AMG_DISPATCH(L.P.g, k_prolong_j, L.P.n, L, b, N.x[0], xb, sc)
        if (skip_last) return;
        SPG_AMG_DISPATCH(ga, k_jacobi_step, L.n, L, b, xb, xa, sc)
        return;
    }
    if (L.degree == 1) {
        launch_pdl(k_jacobi0<T>, blocks_for(L.n), kT, s, L, b, xa, sc);
        SPG_AMG_DISPATCH(ga, k_resid, L.n, L, b, xa, sc)
        SPG_AMG_DISPATCH(L.R.g, k_restrict, L.R.n, L.R, L.r, N.b, sc)
        vcycle_level<T>(a, l + 1, N.b, N.x[0], sc, s);
        SPG_AMG_DISPATCH(L.P.g, k_prolong, L.P.n, L.P, xa, N.x[0], xb, sc)
        SPG_AMG_DISPATCH(ga, k_jacobi_step, L.n, L, b, xb, xa, sc)
        return;
    }
    launch_pdl(k_cheb0<T>, blocks_for(L.n), kT, s, L, b, xa, sc);
    SPG_AMG_DISPATCH(ga, k_cheb_step, L.n, L, b, xa, xb, L.cheb_a, L.cheb_b, sc)
    SPG_AMG_DISPATCH(ga, k_resid, L.n, L, b, xb, sc)
    SPG_AMG_DISPATCH(L.R.g, k_restrict, L.R.n, L.R, L.r, N.b, sc)
    vcycle_level<T>(a, l + 1, N.b, N.x[0], sc, s);
    SPG_AMG_DISPATCH(L.P.g, k_prolong, L.P.n, L.P, xb, N.x[0], xa, sc)
    SPG_AMG_DISPATCH(ga, k_cheb_step, L.n, L, b, xa, xb, 0.0, L.inv_theta, sc)
    SPG_AMG_DISPATCH(ga, k_cheb_step, L.n, L, b, xb, xa, L.cheb_a, L.cheb_b, sc)
}

}  // namespace

void launch_amg_vcycle(const AmgDev &a, const double *r, double *z, const PcgScalars *sc, cudaStream_t s) {
    vcycle_level<double>(a, 0, r, z, sc, s);
}

void launch_amg_vcycle(const AmgDev32 &a, const float *r, float *z, const PcgScalars *sc, cudaStream_t s) {
    vcycle_level<float>(a, 0, r, z, sc, s);
}

bool amg_last_step_fusable(const AmgDev32 &a) { return a.levels > 1 && a.lev[0].degree == 1 && a.lev[0].A.g == 0; }

void launch_amg_vcycle_but_last(const AmgDev32 &a, const float *r, float *z, const PcgScalars *sc, cudaStream_t s) {
    vcycle_level<float>(a, 0, r, z, sc, s, true);
}

}  // namespace spg
