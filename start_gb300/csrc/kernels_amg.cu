// V-cycle of the smoothed-aggregation AMG preconditioner (hierarchy from
// amg_setup.cpp). Per level: Chebyshev pre-smoothing of degree 2 from a zero
// guess, residual, restriction R = P^T, the coarser level, prolongation, and
// Chebyshev post-smoothing of degree 2; the coarsest level multiplies by its
// dense inverse. Pre- and post-smoother are the same polynomial in D^-1 A, so
// the V-cycle is a symmetric positive definite operator and CG stays CG.
// Every operator is stored SELL-32 (level 0 shares the solver's matrix); one
// row per thread; no atomics, so z = M^-1 r is deterministic.
#include "sell.cuh"
#include "spg_internal.h"

namespace spg {

namespace {

constexpr int kT = 256;

__device__ __forceinline__ bool done(const PcgScalars *sc) { return sc && *(volatile const int *)&sc->converged; }

__device__ __forceinline__ double row_mul(const DevSell &M, const double *__restrict__ x, int64_t i) {
    return spmv_row_sell<double>(M.slice_ptr, M.scol, M.sval, x, i);
}

// x = d = D^-1 b / theta (first Chebyshev step from x = 0)
__global__ void __launch_bounds__(kT) k_cheb0(const AmgLevelDev L, const double *__restrict__ b,
                                              double *__restrict__ x, const PcgScalars *sc) {
    if (done(sc)) return;
    const int64_t i = int64_t(blockIdx.x) * kT + threadIdx.x;
    if (i >= L.n) return;
    const double v = L.inv_theta * (L.dinv[i] * b[i]);
    x[i] = v;
    L.d[i] = v;
}

// r = b - A x_in; d = ca d + cb D^-1 r; x_out = x_in + d
__global__ void __launch_bounds__(kT) k_cheb_step(const AmgLevelDev L, const double *__restrict__ b,
                                                  const double *__restrict__ xin, double *__restrict__ xout,
                                                  double ca, double cb, const PcgScalars *sc) {
    if (done(sc)) return;
    const int64_t i = int64_t(blockIdx.x) * kT + threadIdx.x;
    if (i >= L.n) return;
    const double r = b[i] - row_mul(L.A, xin, i);
    const double d = ca * L.d[i] + cb * (L.dinv[i] * r);
    L.d[i] = d;
    xout[i] = xin[i] + d;
}

__global__ void __launch_bounds__(kT) k_resid(const AmgLevelDev L, const double *__restrict__ b,
                                              const double *__restrict__ xin, const PcgScalars *sc) {
    if (done(sc)) return;
    const int64_t i = int64_t(blockIdx.x) * kT + threadIdx.x;
    if (i >= L.n) return;
    L.r[i] = b[i] - row_mul(L.A, xin, i);
}

// b_next = R r
__global__ void __launch_bounds__(kT) k_restrict(const DevSell R, const double *__restrict__ r,
                                                 double *__restrict__ bnext, const PcgScalars *sc) {
    if (done(sc)) return;
    const int64_t i = int64_t(blockIdx.x) * kT + threadIdx.x;
    if (i >= R.n) return;
    bnext[i] = row_mul(R, r, i);
}

// x_out = x_in + P x_coarse
__global__ void __launch_bounds__(kT) k_prolong(const DevSell P, const double *__restrict__ xin,
                                                const double *__restrict__ xc, double *__restrict__ xout,
                                                const PcgScalars *sc) {
    if (done(sc)) return;
    const int64_t i = int64_t(blockIdx.x) * kT + threadIdx.x;
    if (i >= P.n) return;
    xout[i] = xin[i] + row_mul(P, xc, i);
}

// x = A_c^-1 b: one warp per row of the dense inverse, fixed-order lane sums.
__global__ void __launch_bounds__(kT) k_coarse(const double *__restrict__ inv, int64_t nc,
                                               const double *__restrict__ b, double *__restrict__ x,
                                               const PcgScalars *sc) {
    if (done(sc)) return;
    const int64_t row = (int64_t(blockIdx.x) * kT + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= nc) return;
    double s = 0.0;
    for (int64_t k = lane; k < nc; k += 32) s += inv[row * nc + k] * b[k];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if (lane == 0) x[row] = s;
}

inline unsigned blocks_for(int64_t n) { return unsigned((n + kT - 1) / kT); }

void vcycle_level(const AmgDev &a, int l, const double *b, double *xa, const PcgScalars *sc, cudaStream_t s) {
    const AmgLevelDev &L = a.lev[l];
    if (l == a.levels - 1) {
        k_coarse<<<unsigned((a.nc * 32 + kT - 1) / kT), kT, 0, s>>>(a.coarse_inv, a.nc, b, xa, sc);
        return;
    }
    double *xb = L.x[1];
    const unsigned g = blocks_for(L.n);
    k_cheb0<<<g, kT, 0, s>>>(L, b, xa, sc);
    k_cheb_step<<<g, kT, 0, s>>>(L, b, xa, xb, L.cheb_a, L.cheb_b, sc);
    k_resid<<<g, kT, 0, s>>>(L, b, xb, sc);
    const AmgLevelDev &N = a.lev[l + 1];
    k_restrict<<<blocks_for(N.n), kT, 0, s>>>(L.R, L.r, N.b, sc);
    vcycle_level(a, l + 1, N.b, N.x[0], sc, s);
    k_prolong<<<g, kT, 0, s>>>(L.P, xb, N.x[0], xa, sc);
    k_cheb_step<<<g, kT, 0, s>>>(L, b, xa, xb, 0.0, L.inv_theta, sc);
    k_cheb_step<<<g, kT, 0, s>>>(L, b, xb, xa, L.cheb_a, L.cheb_b, sc);
}

}  // namespace

void launch_amg_vcycle(const AmgDev &a, const double *r, double *z, const PcgScalars *sc, cudaStream_t s) {
    vcycle_level(a, 0, r, z, sc, s);
}

}  // namespace spg
