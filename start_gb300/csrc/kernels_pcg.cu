// FEM Poisson solve: CSR SpMV + Jacobi-preconditioned conjugate gradients,
// FP64. Replaces MatrixEquationSolver::solve (Belos + MueLu,
// src/FiniteElementMethod/Solvers/MatrixEquationSolver.cpp:359-427).
//
// All CG scalars live in device memory. Each dot product is reduced in two
// stages: per-block partial sums, then the last block to finish (ticket
// counter) sums the partials in block order and updates the scalars, so an
// iteration needs no host synchronisation and the sums are deterministic for
// a given grid. A converged (or capped) solve turns the remaining launched
// iterations into no-ops.
#include <algorithm>
#include <vector>

#include "pdl.cuh"
#include "sell.cuh"
#include "spg_internal.h"

namespace spg {

namespace {

constexpr int kThreads = 256;
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(kFull, v, off);
    return v;
}

// Block sum of two values into partials[2*blockIdx.x + {0,1}]; returns true in
// thread 0 of the last block to finish, whose totals are then in tot[0..1].
// FP64 adds issue per warp at the FP64 rate, so the block sum runs in warp 0
// only: the 256 per-thread values go through shared memory, lane l adds the
// eight values l, l+32, ..., l+224 in that order and a five-level shuffle
// tree finishes (a fixed order, so the sums are deterministic for a grid).
__device__ __forceinline__ void block_sum2(double &a, double &b) {
    __shared__ double sa[kThreads], sb[kThreads];
    sa[threadIdx.x] = a;
    sb[threadIdx.x] = b;
    __syncthreads();
    if (threadIdx.x < 32) {
        double ta = sa[threadIdx.x], tb = sb[threadIdx.x];
#pragma unroll
        for (int w = 1; w < kThreads / 32; ++w) {
            ta += sa[threadIdx.x + 32 * w];
            tb += sb[threadIdx.x + 32 * w];
        }
        a = warp_sum(ta);
        b = warp_sum(tb);
    }
}

__device__ bool block_reduce2(double a, double b, double *partials, PcgScalars *sc, double tot[2]) {
    __shared__ bool last;
    block_sum2(a, b);
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = a;
        partials[2 * blockIdx.x + 1] = b;
        __threadfence();
        const unsigned ticket = atomicInc(&sc->ticket, gridDim.x - 1);
        last = ticket == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return false;
    // last block: fixed-order sum of the partials
    __threadfence();
    double ta = 0.0, tb = 0.0;
    for (int k = threadIdx.x; k < int(gridDim.x); k += kThreads) {
        ta += __ldcg(partials + 2 * k);
        tb += __ldcg(partials + 2 * k + 1);
    }
    __syncthreads();  // the shared buffers of block_sum2 are reused
    block_sum2(ta, tb);
    if (threadIdx.x != 0) return false;
    tot[0] = ta;
    tot[1] = tb;
    return true;
}

__device__ __forceinline__ double spmv_row(const PcgDev &d, const double *__restrict__ x, int64_t i) {
    return spmv_row_sell<double>(d.slice_ptr, d.scol, d.sval, x, i);
}

__global__ void k_rhs(const double *__restrict__ node_q, double inv_eps0, const double *__restrict__ lift,
                      const uint8_t *__restrict__ is_dir, const double *__restrict__ g, double *__restrict__ b,
                      int64_t n) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    b[i] = is_dir[i] ? g[i] : node_q[i] * inv_eps0 - lift[i];
}

__global__ void k_node_rho(const double *__restrict__ node_q, const double *__restrict__ dual_vol,
                           double *__restrict__ rho, int64_t n) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    rho[i] = node_q[i] / dual_vol[i];
}

// Charge of each node from a given nodal density: q = rho V_dual.
__global__ void k_node_q_from_rho(const double *__restrict__ rho, const double *__restrict__ dual_vol,
                                  double *__restrict__ node_q, int64_t n) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    node_q[i] = rho[i] * dual_vol[i];
}

// r = b - A x, z = D^-1 r, p = z; rz = r.z, bb = b.b, rr = r.r
__global__ void __launch_bounds__(kThreads) k_setup(PcgDev d, const double *__restrict__ b) {
    pdl_sync();
    double rz = 0.0, bb = 0.0;
    __shared__ double s_rr[kThreads / 32];
    double rr = 0.0;
    for (int64_t i = int64_t(blockIdx.x) * kThreads + threadIdx.x; i < d.n; i += int64_t(gridDim.x) * kThreads) {
        const double bi = b[i];
        const double ri = bi - spmv_row(d, d.x, i);
        const double zi = ri * d.inv_diag[i];
        d.r[i] = ri;
        d.z[i] = zi;
        d.p[i] = zi;
        rz += ri * zi;
        bb += bi * bi;
        rr += ri * ri;
    }
    // rr rides on a second pass through partials: fold it into the block's
    // shared total first, then reduce (rz, bb) and (rr) separately.
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    rr = warp_sum(rr);
    if (lane == 0) s_rr[wid] = rr;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) t += s_rr[w];
        d.partials[2 * gridDim.x + blockIdx.x] = t;
    }
    double tot[2];
    if (block_reduce2(rz, bb, d.partials, d.sc, tot)) {
        double rrt = 0.0;
        for (unsigned k = 0; k < gridDim.x; ++k) rrt += __ldcg(d.partials + 2 * gridDim.x + k);
        PcgScalars *sc = d.sc;
        sc->rz = tot[0];
        sc->bb = tot[1];
        sc->rr = rrt;
        sc->tol2 = sc->tol2 * tot[1];  // rtol^2 -> rtol^2 ||b||^2
        sc->iters = 0;
        sc->converged = (rrt <= sc->tol2 || tot[1] == 0.0) ? 1 : 0;
        sc->alpha = 0.0;
        sc->beta = 0.0;
    }
}

// q = A p; pq = p.q; alpha = rz / pq
__global__ void __launch_bounds__(kThreads) k_spmv_dot(PcgDev d) {
    pdl_sync();
    if (d.sc->converged) return;
    double pq = 0.0;
    for (int64_t i = int64_t(blockIdx.x) * kThreads + threadIdx.x; i < d.n; i += int64_t(gridDim.x) * kThreads) {
        const double qi = spmv_row(d, d.p, i);
        d.q[i] = qi;
        pq += d.p[i] * qi;
    }
    double tot[2];
    if (block_reduce2(pq, 0.0, d.partials, d.sc, tot)) {
        PcgScalars *sc = d.sc;
        sc->pq = tot[0];
        if (tot[0] > 0.0) {
            sc->alpha = sc->rz / tot[0];
        } else {
            sc->alpha = 0.0;
            sc->converged = 2;  // breakdown: A not SPD on this subspace
        }
    }
}

// x += alpha p; r -= alpha q; z = D^-1 r; rz' = r.z, rr = r.r; beta = rz'/rz
__global__ void __launch_bounds__(kThreads) k_update(PcgDev d) {
    pdl_sync();
    if (d.sc->converged) return;
    const double alpha = d.sc->alpha;
    double rz = 0.0, rr = 0.0;
    for (int64_t i = int64_t(blockIdx.x) * kThreads + threadIdx.x; i < d.n; i += int64_t(gridDim.x) * kThreads) {
        d.x[i] += alpha * d.p[i];
        const double ri = d.r[i] - alpha * d.q[i];
        const double zi = ri * d.inv_diag[i];
        d.r[i] = ri;
        d.z[i] = zi;
        rz += ri * zi;
        rr += ri * ri;
    }
    double tot[2];
    if (block_reduce2(rz, rr, d.partials, d.sc, tot)) {
        PcgScalars *sc = d.sc;
        sc->iters += 1;
        sc->rr = tot[1];
        if (tot[1] <= sc->tol2) {
            sc->converged = 1;
        } else if (sc->iters >= sc->max_iter) {
            sc->converged = 2;
        } else {
            sc->beta = tot[0] / sc->rz;
            sc->rz = tot[0];
        }
    }
}

// p = z + beta p
__global__ void __launch_bounds__(kThreads) k_pupdate(PcgDev d) {
    pdl_sync();
    if (d.sc->converged) return;
    const double beta = d.sc->beta;
    for (int64_t i = int64_t(blockIdx.x) * kThreads + threadIdx.x; i < d.n; i += int64_t(gridDim.x) * kThreads)
        d.p[i] = d.z[i] + beta * d.p[i];
}

// ------------------------------------------------- PCG with the AMG V-cycle
// M = false: the FP64 V-cycle reads r and writes z. M = true (mixed form):
// the FP32 V-cycle reads r32 = float(r) and writes z32; x, r, p, q and all
// sums stay FP64, so the solve still stops on the FP64 residual.

// r = b - A x; bb = b.b, rr = r.r (z = M^-1 r follows as a V-cycle)
template <bool M>
__global__ void __launch_bounds__(kThreads) k_setup_amg(PcgDev d, const double *__restrict__ b, float *__restrict__ r32) {
    pdl_sync();
    double bb = 0.0, rr = 0.0;
    for (int64_t i = int64_t(blockIdx.x) * kThreads + threadIdx.x; i < d.n; i += int64_t(gridDim.x) * kThreads) {
        const double bi = b[i];
        const double ri = bi - spmv_row(d, d.x, i);
        d.r[i] = ri;
        if constexpr (M) r32[i] = float(ri);
        bb += bi * bi;
        rr += ri * ri;
    }
    double tot[2];
    if (block_reduce2(rr, bb, d.partials, d.sc, tot)) {
        PcgScalars *sc = d.sc;
        sc->rr = tot[0];
        sc->bb = tot[1];
        sc->tol2 = sc->tol2 * tot[1];  // rtol^2 -> rtol^2 ||b||^2
        sc->iters = 0;
        sc->converged = (tot[0] <= sc->tol2 || tot[1] == 0.0) ? 1 : 0;
        sc->alpha = 0.0;
        sc->beta = 0.0;
        sc->rz = 0.0;
    }
}

// x += alpha p; r -= alpha q; rr = r.r and the stop test
template <bool M>
__global__ void __launch_bounds__(kThreads) k_update_amg(PcgDev d, float *__restrict__ r32) {
    pdl_sync();
    if (d.sc->converged) return;
    const double alpha = d.sc->alpha;
    double rr = 0.0;
    for (int64_t i = int64_t(blockIdx.x) * kThreads + threadIdx.x; i < d.n; i += int64_t(gridDim.x) * kThreads) {
        d.x[i] += alpha * d.p[i];
        const double ri = d.r[i] - alpha * d.q[i];
        d.r[i] = ri;
        if constexpr (M) r32[i] = float(ri);
        rr += ri * ri;
    }
    double tot[2];
    if (block_reduce2(rr, 0.0, d.partials, d.sc, tot)) {
        PcgScalars *sc = d.sc;
        sc->iters += 1;
        sc->rr = tot[0];
        if (tot[0] <= sc->tol2)
            sc->converged = 1;
        else if (sc->iters >= sc->max_iter)
            sc->converged = 2;
    }
}

// rz' = r.z (z from the V-cycle); first: p = z; else beta = rz'/rz
template <bool M>
__global__ void __launch_bounds__(kThreads) k_rz_amg(PcgDev d, const float *__restrict__ z32, int first) {
    pdl_sync();
    if (d.sc->converged) return;
    double rz = 0.0;
    for (int64_t i = int64_t(blockIdx.x) * kThreads + threadIdx.x; i < d.n; i += int64_t(gridDim.x) * kThreads) {
        double zi;
        if constexpr (M)
            zi = double(z32[i]);
        else
            zi = d.z[i];
        rz += d.r[i] * zi;
        if (first) d.p[i] = zi;
    }
    double tot[2];
    if (block_reduce2(rz, 0.0, d.partials, d.sc, tot)) {
        PcgScalars *sc = d.sc;
        if (!first) sc->beta = tot[0] / sc->rz;
        sc->rz = tot[0];
    }
}

// The V-cycle's last level-0 Jacobi step z32 = x1 + D^-1 (r32 - A x1) / theta
// (k_jacobi_step's arithmetic) fused with k_rz_amg: rz' = r.z (FP64 r, z
// promoted), first: p = z (and beta = 0); else beta = rz'/rz. First = 2: the
// first iteration is the one with no update yet (sc->iters == 0).
template <int FirstArg>
__global__ void __launch_bounds__(kThreads) k_jacobi_rz(PcgDev d, const AmgLevelDevT<float> L,
                                                        const float *__restrict__ r32, float *__restrict__ z32) {
    pdl_sync();
    if (d.sc->converged) return;
    const bool First = FirstArg == 2 ? d.sc->iters == 0 : FirstArg == 1;
    const float *xin = L.x[1];
    double rz = 0.0;
    for (int64_t i = int64_t(blockIdx.x) * kThreads + threadIdx.x; i < d.n; i += int64_t(gridDim.x) * kThreads) {
        const float ax = spmv_row_sell<float>(L.A.slice_ptr, L.A.scol, L.A.sval, xin, i);
        const float rr = r32[i] - ax;
        const float zi = xin[i] + float(L.inv_theta) * (L.dinv[i] * rr);
        z32[i] = zi;
        const double zd = double(zi);
        rz += d.r[i] * zd;
        if (First) d.p[i] = zd;
    }
    double tot[2];
    if (block_reduce2(rz, 0.0, d.partials, d.sc, tot)) {
        PcgScalars *sc = d.sc;
        sc->beta = First ? 0.0 : tot[0] / sc->rz;
        sc->rz = tot[0];
    }
}

// The loop condition of the PCG while-graph: go on until the scalars say
// converged (1), capped (2) or failed.
__global__ void k_pcg_continue(cudaGraphConditionalHandle cond, const PcgScalars *sc) {
    cudaGraphSetConditional(cond, *(volatile const int *)&sc->converged ? 0u : 1u);
}

// p = z32 + beta p (mixed form)
__global__ void __launch_bounds__(kThreads) k_pupdate_m(PcgDev d, const float *__restrict__ z32) {
    pdl_sync();
    if (d.sc->converged) return;
    const double beta = d.sc->beta;
    for (int64_t i = int64_t(blockIdx.x) * kThreads + threadIdx.x; i < d.n; i += int64_t(gridDim.x) * kThreads)
        d.p[i] = fma(beta, d.p[i], double(z32[i]));
}

// ------------------------------------------------- mixed precision (SPG_MIXED)
// FP32 SpMV PCG for the correction e in A e = r, inside FP64 iterative
// refinement x <- x + e on r = b - A x (FP64 SpMV). Dot products are FP64:
// each warp sums its FP32 products in FP32, the warp sum is promoted and all
// further accumulation is FP64.

__device__ __forceinline__ float spmv_row32(const PcgDev32 &d, const float *__restrict__ x, int64_t i) {
    return spmv_row_sell<float>(d.slice_ptr, d.scol, d.sval, x, i);
}

__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(kFull, v, off);
    return v;
}

// FP64 block reduction of FP32 per-thread partials: each warp sums in FP32
// (the total lands in lane 0), only lane 0 passes it on, and everything from
// there on is FP64.
__device__ bool block_reduce2_w(float a, float b, double *partials, PcgScalars *sc, double tot[2]) {
    a = warp_sumf(a);
    b = warp_sumf(b);
    const bool lead = (threadIdx.x & 31) == 0;
    return block_reduce2(lead ? double(a) : 0.0, lead ? double(b) : 0.0, partials, sc, tot);
}

// Outer step: r = b - A x in FP64, rr = r.r, bb = b.b; start the inner solve:
// e = 0, r32 = r, z = D^-1 r32, p = z, rz = r32.z.
__global__ void __launch_bounds__(kThreads) k_refine_setup(PcgDev d, PcgDev32 f, const double *__restrict__ b) {
    pdl_sync();
    double rr = 0.0, bb = 0.0;
    float rz = 0.0f;
    __shared__ double s_rz[kThreads / 32];
    for (int64_t i = int64_t(blockIdx.x) * kThreads + threadIdx.x; i < d.n; i += int64_t(gridDim.x) * kThreads) {
        const double bi = b[i];
        const double ri = bi - spmv_row(d, d.x, i);
        const float r32 = float(ri);
        const float z32 = r32 * f.inv_diag[i];
        f.r[i] = r32;
        f.z[i] = z32;
        f.p[i] = z32;
        f.e[i] = 0.0f;
        rr += ri * ri;
        bb += bi * bi;
        rz = fmaf(r32, z32, rz);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const float rzw = warp_sumf(rz);
    if (lane == 0) s_rz[wid] = double(rzw);
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) t += s_rz[w];
        d.partials[2 * gridDim.x + blockIdx.x] = t;
    }
    double tot[2];
    if (block_reduce2(rr, bb, d.partials, d.sc, tot)) {
        double rzt = 0.0;
        for (unsigned k = 0; k < gridDim.x; ++k) rzt += __ldcg(d.partials + 2 * gridDim.x + k);
        PcgScalars *sc = d.sc;  // outer scalars
        sc->rr = tot[0];
        sc->bb = tot[1];
        sc->converged = (tot[0] <= sc->tol2 * tot[1] || tot[1] == 0.0) ? 1 : 0;
        PcgScalars *si = f.sc;  // inner scalars
        si->rz = rzt;
        si->rr = tot[0];
        si->bb = tot[0];  // inner tolerance relative to the outer residual
        si->iters = 0;
        si->converged = sc->converged;
        si->alpha = 0.0;
        si->beta = 0.0;
    }
}

__global__ void __launch_bounds__(kThreads) k_spmv_dot32(PcgDev32 f) {
    pdl_sync();
    if (f.sc->converged) return;
    float pq = 0.0f;
    for (int64_t i = int64_t(blockIdx.x) * kThreads + threadIdx.x; i < f.n; i += int64_t(gridDim.x) * kThreads) {
        const float qi = spmv_row32(f, f.p, i);
        f.q[i] = qi;
        pq = fmaf(f.p[i], qi, pq);
    }
    double tot[2];
    if (block_reduce2_w(pq, 0.0f, f.partials, f.sc, tot)) {
        PcgScalars *sc = f.sc;
        sc->pq = tot[0];
        if (tot[0] > 0.0) {
            sc->alpha = sc->rz / tot[0];
        } else {
            sc->alpha = 0.0;
            sc->converged = 2;
        }
    }
}

__global__ void __launch_bounds__(kThreads) k_update32(PcgDev32 f) {
    pdl_sync();
    if (f.sc->converged) return;
    const float alpha = float(f.sc->alpha);
    float rz = 0.0f, rr = 0.0f;
    for (int64_t i = int64_t(blockIdx.x) * kThreads + threadIdx.x; i < f.n; i += int64_t(gridDim.x) * kThreads) {
        f.e[i] = fmaf(alpha, f.p[i], f.e[i]);
        const float ri = fmaf(-alpha, f.q[i], f.r[i]);
        const float zi = ri * f.inv_diag[i];
        f.r[i] = ri;
        f.z[i] = zi;
        rz = fmaf(ri, zi, rz);
        rr = fmaf(ri, ri, rr);
    }
    double tot[2];
    if (block_reduce2_w(rz, rr, f.partials, f.sc, tot)) {
        PcgScalars *sc = f.sc;
        sc->iters += 1;
        sc->rr = tot[1];
        if (tot[1] <= sc->tol2 * sc->bb) {
            sc->converged = 1;
        } else if (sc->iters >= sc->max_iter) {
            sc->converged = 3;  // inner cap: the outer loop refines again
        } else {
            sc->beta = tot[0] / sc->rz;
            sc->rz = tot[0];
        }
    }
}

__global__ void __launch_bounds__(kThreads) k_pupdate32(PcgDev32 f) {
    pdl_sync();
    if (f.sc->converged) return;
    const float beta = float(f.sc->beta);
    for (int64_t i = int64_t(blockIdx.x) * kThreads + threadIdx.x; i < f.n; i += int64_t(gridDim.x) * kThreads)
        f.p[i] = fmaf(beta, f.p[i], f.z[i]);
}

__global__ void k_refine_apply(double *__restrict__ x, const float *__restrict__ e, int64_t n) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    x[i] += double(e[i]);
}

}  // namespace

// Each kernel runs SMs x (its resident 256-thread blocks per SM) blocks, one
// wave; each thread then handles several rows of a large system, so the FP64
// shuffle reductions of the dot products (which issue per warp at the FP64
// rate) are amortised over several rows.
static int sm_count_attr() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

int pcg_blocks(int64_t n) {
    const int64_t want = (n + kThreads - 1) / kThreads;
    const int64_t cap = int64_t(sm_count_attr()) * (2048 / kThreads);
    return int(want < cap ? (want < 1 ? 1 : want) : cap);
}

namespace {
template <class K>
int wave(K kernel, int64_t n) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, 0);
    const int64_t cap = int64_t(sm_count_attr()) * (per_sm > 0 ? per_sm : 1);
    const int64_t want = (n + kThreads - 1) / kThreads;
    const int g = int(want < cap ? (want < 1 ? 1 : want) : cap);
    return g < pcg_blocks(n) ? g : pcg_blocks(n);  // the partials hold pcg_blocks(n) blocks
}
}  // namespace

PcgGrid pcg_grid64(int64_t n) {
    PcgGrid g;
    g.setup = wave(k_setup, n);
    g.spmv = wave(k_spmv_dot, n);
    g.update = wave(k_update, n);
    g.pupdate = wave(k_pupdate, n);
    return g;
}

void launch_pcg_rhs(const double *node_q, double inv_eps0, const double *lift, const uint8_t *is_dir,
                    const double *dir_value, double *b, int64_t n, cudaStream_t s) {
    k_rhs<<<unsigned((n + 255) / 256), 256, 0, s>>>(node_q, inv_eps0, lift, is_dir, dir_value, b, n);
}

void launch_node_rho(const double *node_q, const double *dual_vol, double *rho, int64_t n, cudaStream_t s) {
    k_node_rho<<<unsigned((n + 255) / 256), 256, 0, s>>>(node_q, dual_vol, rho, n);
}

void launch_node_q_from_rho(const double *rho, const double *dual_vol, double *node_q, int64_t n, cudaStream_t s) {
    if (n > 0) k_node_q_from_rho<<<unsigned((n + 255) / 256), 256, 0, s>>>(rho, dual_vol, node_q, n);
}

void launch_pcg_setup(const PcgDev &d, const double *b, cudaStream_t s) {
    launch_pdl(k_setup, d.grid.setup, kThreads, s, d, b);
}

void launch_pcg_setup_amg(const PcgDev &d, const AmgDev &a, const double *b, cudaStream_t s) {
    launch_pdl(k_setup_amg<false>, d.grid.setup, kThreads, s, d, b, nullptr);
    launch_amg_vcycle(a, d.r, d.z, d.sc, s);
    launch_pdl(k_rz_amg<false>, d.grid.update, kThreads, s, d, nullptr, 1);
}

void launch_pcg_iteration_amg(PcgDev &d, const AmgDev &a, cudaStream_t s) {
    launch_pdl(k_spmv_dot, d.grid.spmv, kThreads, s, d);
    launch_pdl(k_update_amg<false>, d.grid.update, kThreads, s, d, nullptr);
    launch_amg_vcycle(a, d.r, d.z, d.sc, s);
    launch_pdl(k_rz_amg<false>, d.grid.update, kThreads, s, d, nullptr, 0);
    launch_pdl(k_pupdate, d.grid.pupdate, kThreads, s, d);
}

// z32 = M^-1 r32 and r.z: the V-cycle's last step fused with the sum where
// level 0 allows it, else the whole V-cycle and k_rz_amg.
static void vcycle_rz(PcgDev d, const AmgDev32 &a, float *r32, float *z32, int first, cudaStream_t s) {
    if (amg_last_step_fusable(a)) {
        launch_amg_vcycle_but_last(a, r32, z32, d.sc, s);
        if (first)
            launch_pdl(k_jacobi_rz<1>, d.grid.update, kThreads, s, d, a.lev[0], r32, z32);
        else
            launch_pdl(k_jacobi_rz<0>, d.grid.update, kThreads, s, d, a.lev[0], r32, z32);
    } else {
        launch_amg_vcycle(a, r32, z32, d.sc, s);
        launch_pdl(k_rz_amg<true>, d.grid.update, kThreads, s, d, z32, first);
    }
}

void launch_pcg_setup_amg_mixed(const PcgDev &d, const AmgDev32 &a, const double *b, float *r32, float *z32,
                                cudaStream_t s) {
    launch_pdl(k_setup_amg<true>, d.grid.setup, kThreads, s, d, b, r32);
    vcycle_rz(d, a, r32, z32, 1, s);
}

void launch_pcg_continue(cudaGraphConditionalHandle cond, const PcgScalars *sc, cudaStream_t s) {
    k_pcg_continue<<<1, 1, 0, s>>>(cond, sc);
}

bool pcg_rotated_ok(const AmgDev32 &a) { return amg_last_step_fusable(a); }

void launch_pcg_residual_amg_mixed(const PcgDev &d, const double *b, float *r32, cudaStream_t s) {
    launch_pdl(k_setup_amg<true>, d.grid.setup, kThreads, s, d, b, r32);
}

void launch_pcg_rotated_iteration_amg_mixed(PcgDev &d, const AmgDev32 &a, float *r32, float *z32, cudaStream_t s) {
    launch_amg_vcycle_but_last(a, r32, z32, d.sc, s);
    launch_pdl(k_jacobi_rz<2>, d.grid.update, kThreads, s, d, a.lev[0], r32, z32);
    launch_pdl(k_pupdate_m, d.grid.pupdate, kThreads, s, d, z32);
    launch_pdl(k_spmv_dot, d.grid.spmv, kThreads, s, d);
    launch_pdl(k_update_amg<true>, d.grid.update, kThreads, s, d, r32);
}

void launch_pcg_iteration_amg_mixed(PcgDev &d, const AmgDev32 &a, float *r32, float *z32, cudaStream_t s) {
    launch_pdl(k_spmv_dot, d.grid.spmv, kThreads, s, d);
    launch_pdl(k_update_amg<true>, d.grid.update, kThreads, s, d, r32);
    vcycle_rz(d, a, r32, z32, 0, s);
    launch_pdl(k_pupdate_m, d.grid.pupdate, kThreads, s, d, z32);
}

void launch_pcg_iteration(PcgDev &d, cudaStream_t s) {
    launch_pdl(k_spmv_dot, d.grid.spmv, kThreads, s, d);
    launch_pdl(k_update, d.grid.update, kThreads, s, d);
    launch_pdl(k_pupdate, d.grid.pupdate, kThreads, s, d);
}

// Entries that are exactly zero off the diagonal are left out (the P1
// stiffness of a Kuhn-split lattice is the 7-point stencil: 8 of its 15
// structural couplings per row are exact zeros); a product with an exact
// zero adds nothing to a sum, so A x is unchanged.
template <class RP>
void build_sell32_t(int64_t n, const RP *row_ptr, const int32_t *col, const double *val,
                    std::vector<int64_t> &slice_ptr, std::vector<int32_t> &scol, std::vector<double> &sval) {
    auto kept = [&](int64_t r, int64_t k) { return val[k] != 0.0 || col[k] == r; };
    std::vector<int64_t> len(n, 0);
    for (int64_t r = 0; r < n; ++r)
        for (int64_t k = int64_t(row_ptr[r]); k < int64_t(row_ptr[r + 1]); ++k) len[r] += kept(r, k) ? 1 : 0;
    const int64_t ns = (n + 31) / 32;
    slice_ptr.assign(ns + 1, 0);
    for (int64_t sl = 0; sl < ns; ++sl) {
        int64_t w = 0;
        for (int64_t r = sl * 32; r < std::min(n, sl * 32 + 32); ++r) w = std::max(w, len[r]);
        slice_ptr[sl + 1] = slice_ptr[sl] + 32 * w;
    }
    scol.assign(slice_ptr[ns], 0);
    sval.assign(slice_ptr[ns], 0.0);
    for (int64_t sl = 0; sl < ns; ++sl) {
        const int64_t w = (slice_ptr[sl + 1] - slice_ptr[sl]) / 32;
        for (int64_t l = 0; l < 32; ++l) {
            const int64_t r = sl * 32 + l;
            int64_t j = 0;
            int32_t first = 0;
            if (r < n)
                for (int64_t k = int64_t(row_ptr[r]); k < int64_t(row_ptr[r + 1]); ++k) {
                    if (!kept(r, k)) continue;
                    const int64_t o = slice_ptr[sl] + 32 * j + l;
                    scol[o] = col[k];
                    sval[o] = val[k];
                    if (j == 0) first = col[k];
                    ++j;
                }
            // padding: value 0 at a column the row already reads (or column
            // 0), always inside x also for a rectangular matrix
            for (; j < w; ++j) {
                const int64_t o = slice_ptr[sl] + 32 * j + l;
                scol[o] = first;
                sval[o] = 0.0;
            }
        }
    }
}

void build_sell32(int64_t n, const int32_t *row_ptr, const int32_t *col, const double *val,
                  std::vector<int64_t> &slice_ptr, std::vector<int32_t> &scol, std::vector<double> &sval) {
    build_sell32_t(n, row_ptr, col, val, slice_ptr, scol, sval);
}
void build_sell32(int64_t n, const int64_t *row_ptr, const int32_t *col, const double *val,
                  std::vector<int64_t> &slice_ptr, std::vector<int32_t> &scol, std::vector<double> &sval) {
    build_sell32_t(n, row_ptr, col, val, slice_ptr, scol, sval);
}

}  // namespace spg

namespace spg {

void launch_refine_setup(const PcgDev &d, const PcgDev32 &f, const double *b, cudaStream_t s) {
    launch_pdl(k_refine_setup, f.grid.setup, kThreads, s, d, f, b);
}

void launch_pcg32_iteration(PcgDev32 &f, cudaStream_t s) {
    launch_pdl(k_spmv_dot32, f.grid.spmv, kThreads, s, f);
    launch_pdl(k_update32, f.grid.update, kThreads, s, f);
    launch_pdl(k_pupdate32, f.grid.pupdate, kThreads, s, f);
}

PcgGrid pcg_grid32(int64_t n) {
    PcgGrid g;
    g.setup = wave(k_refine_setup, n);
    g.spmv = wave(k_spmv_dot32, n);
    g.update = wave(k_update32, n);
    g.pupdate = wave(k_pupdate32, n);
    return g;
}

void launch_refine_apply(double *x, const float *e, int64_t n, cudaStream_t s) {
    k_refine_apply<<<unsigned((n + 255) / 256), 256, 0, s>>>(x, e, n);
}

}  // namespace spg

namespace spg {

namespace {
// Shifts the history (prev2 <- prev, prev <- phi) and sets phi to the
// extrapolation of order `order` (0: phi itself, 1: 2 phi - prev, 2: 3 phi
// - 3 prev + prev2).
__global__ void k_extrapolate(double *__restrict__ phi, double *__restrict__ prev, double *__restrict__ prev2,
                              int64_t n, int order) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double t = phi[i], p1 = prev[i];
    if (order == 1)
        phi[i] = fma(2.0, t, -p1);
    else if (order == 2)
        phi[i] = fma(3.0, t - p1, prev2[i]);
    prev2[i] = p1;
    prev[i] = t;
}
}  // namespace

void launch_extrapolate(double *phi, double *prev, double *prev2, int64_t n, int order, cudaStream_t s) {
    k_extrapolate<<<unsigned((n + 255) / 256), 256, 0, s>>>(phi, prev, prev2, n, order < 0 ? 0 : order);
}

}  // namespace spg
