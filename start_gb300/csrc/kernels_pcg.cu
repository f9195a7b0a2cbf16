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
__device__ bool block_reduce2(double a, double b, double *partials, PcgScalars *sc, double tot[2]) {
    __shared__ double sa[kThreads / 32], sb[kThreads / 32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    a = warp_sum(a);
    b = warp_sum(b);
    if (lane == 0) {
        sa[wid] = a;
        sb[wid] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ta = 0.0, tb = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) {
            ta += sa[w];
            tb += sb[w];
        }
        partials[2 * blockIdx.x] = ta;
        partials[2 * blockIdx.x + 1] = tb;
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
    ta = warp_sum(ta);
    tb = warp_sum(tb);
    __syncthreads();
    if (lane == 0) {
        sa[wid] = ta;
        sb[wid] = tb;
    }
    __syncthreads();
    if (threadIdx.x != 0) return false;
    ta = 0.0;
    tb = 0.0;
    for (int w = 0; w < kThreads / 32; ++w) {
        ta += sa[w];
        tb += sb[w];
    }
    tot[0] = ta;
    tot[1] = tb;
    return true;
}

// Row i of A x in SELL-32 storage: rows are grouped in slices of 32 (one
// warp), each slice padded to its longest row and stored column-major, so
// lane l of a warp reads entry j of its row at slice_ptr[s] + 32 j + l and a
// warp's 32 loads of one j are contiguous. Padding entries have value 0.
// Four entries per trip with their loads issued before the FMAs and two
// accumulators, so each thread keeps several gathers in flight.
__device__ __forceinline__ double spmv_row(const PcgDev &d, const double *__restrict__ x, int64_t i) {
    const int64_t s = i >> 5;
    int64_t k = __ldg(d.slice_ptr + s) + (i & 31);
    const int64_t k1 = __ldg(d.slice_ptr + s + 1);
    double a0 = 0.0, a1 = 0.0;
    for (; k + 96 < k1; k += 128) {
        const int32_t c0 = __ldg(d.scol + k), c1 = __ldg(d.scol + k + 32);
        const int32_t c2 = __ldg(d.scol + k + 64), c3 = __ldg(d.scol + k + 96);
        const double v0 = __ldg(d.sval + k), v1 = __ldg(d.sval + k + 32);
        const double v2 = __ldg(d.sval + k + 64), v3 = __ldg(d.sval + k + 96);
        const double x0 = __ldg(x + c0), x1 = __ldg(x + c1), x2 = __ldg(x + c2), x3 = __ldg(x + c3);
        a0 = fma(v0, x0, a0);
        a1 = fma(v1, x1, a1);
        a0 = fma(v2, x2, a0);
        a1 = fma(v3, x3, a1);
    }
    for (; k < k1; k += 32) a0 = fma(__ldg(d.sval + k), __ldg(x + __ldg(d.scol + k)), a0);
    return a0 + a1;
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

// r = b - A x, z = D^-1 r, p = z; rz = r.z, bb = b.b, rr = r.r
__global__ void __launch_bounds__(kThreads) k_setup(PcgDev d, const double *__restrict__ b) {
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
    if (d.sc->converged) return;
    const double beta = d.sc->beta;
    for (int64_t i = int64_t(blockIdx.x) * kThreads + threadIdx.x; i < d.n; i += int64_t(gridDim.x) * kThreads)
        d.p[i] = d.z[i] + beta * d.p[i];
}

// ------------------------------------------------- mixed precision (SPG_MIXED)
// FP32 SpMV PCG for the correction e in A e = r, inside FP64 iterative
// refinement x <- x + e on r = b - A x (FP64 SpMV). Dot products are FP64:
// each warp sums its FP32 products in FP32, the warp sum is promoted and all
// further accumulation is FP64.

__device__ __forceinline__ float spmv_row32(const PcgDev32 &d, const float *__restrict__ x, int64_t i) {
    const int64_t s = i >> 5;
    int64_t k = __ldg(d.slice_ptr + s) + (i & 31);
    const int64_t k1 = __ldg(d.slice_ptr + s + 1);
    float a0 = 0.0f, a1 = 0.0f;
    for (; k + 96 < k1; k += 128) {
        const int32_t c0 = __ldg(d.scol + k), c1 = __ldg(d.scol + k + 32);
        const int32_t c2 = __ldg(d.scol + k + 64), c3 = __ldg(d.scol + k + 96);
        const float v0 = __ldg(d.sval + k), v1 = __ldg(d.sval + k + 32);
        const float v2 = __ldg(d.sval + k + 64), v3 = __ldg(d.sval + k + 96);
        const float x0 = __ldg(x + c0), x1 = __ldg(x + c1), x2 = __ldg(x + c2), x3 = __ldg(x + c3);
        a0 = fmaf(v0, x0, a0);
        a1 = fmaf(v1, x1, a1);
        a0 = fmaf(v2, x2, a0);
        a1 = fmaf(v3, x3, a1);
    }
    for (; k < k1; k += 32) a0 = fmaf(__ldg(d.sval + k), __ldg(x + __ldg(d.scol + k)), a0);
    return a0 + a1;
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

// Four 256-thread blocks per SM: each thread then handles several rows, so
// the FP64 shuffle reductions of the dot products (which issue per warp at
// the FP64 rate) are amortised over several rows.
int pcg_blocks(int64_t n) {
    const int64_t want = (n + kThreads - 1) / kThreads;
    return int(want < 152 * 4 ? (want < 1 ? 1 : want) : 152 * 4);
}

void launch_pcg_rhs(const double *node_q, double inv_eps0, const double *lift, const uint8_t *is_dir,
                    const double *dir_value, double *b, int64_t n, cudaStream_t s) {
    k_rhs<<<unsigned((n + 255) / 256), 256, 0, s>>>(node_q, inv_eps0, lift, is_dir, dir_value, b, n);
}

void launch_node_rho(const double *node_q, const double *dual_vol, double *rho, int64_t n, cudaStream_t s) {
    k_node_rho<<<unsigned((n + 255) / 256), 256, 0, s>>>(node_q, dual_vol, rho, n);
}

void launch_pcg_setup(const PcgDev &d, const double *b, cudaStream_t s) {
    k_setup<<<d.blocks, kThreads, 0, s>>>(d, b);
}

void launch_pcg_iteration(PcgDev &d, cudaStream_t s) {
    k_spmv_dot<<<d.blocks, kThreads, 0, s>>>(d);
    k_update<<<d.blocks, kThreads, 0, s>>>(d);
    k_pupdate<<<d.blocks, kThreads, 0, s>>>(d);
}

void build_sell32(int64_t n, const int32_t *row_ptr, const int32_t *col, const double *val,
                  std::vector<int64_t> &slice_ptr, std::vector<int32_t> &scol, std::vector<double> &sval) {
    const int64_t ns = (n + 31) / 32;
    slice_ptr.assign(ns + 1, 0);
    for (int64_t sl = 0; sl < ns; ++sl) {
        int32_t w = 0;
        for (int64_t r = sl * 32; r < std::min(n, sl * 32 + 32); ++r) w = std::max(w, row_ptr[r + 1] - row_ptr[r]);
        slice_ptr[sl + 1] = slice_ptr[sl] + 32 * int64_t(w);
    }
    scol.assign(slice_ptr[ns], 0);
    sval.assign(slice_ptr[ns], 0.0);
    for (int64_t sl = 0; sl < ns; ++sl) {
        const int64_t w = (slice_ptr[sl + 1] - slice_ptr[sl]) / 32;
        for (int64_t l = 0; l < 32; ++l) {
            const int64_t r = sl * 32 + l;
            const int32_t len = r < n ? row_ptr[r + 1] - row_ptr[r] : 0;
            for (int64_t j = 0; j < w; ++j) {
                const int64_t k = slice_ptr[sl] + 32 * j + l;
                if (j < len) {
                    scol[k] = col[row_ptr[r] + j];
                    sval[k] = val[row_ptr[r] + j];
                } else {
                    scol[k] = r < n ? int32_t(r) : 0;
                    sval[k] = 0.0;
                }
            }
        }
    }
}

}  // namespace spg

namespace spg {

void launch_refine_setup(const PcgDev &d, const PcgDev32 &f, const double *b, cudaStream_t s) {
    k_refine_setup<<<d.blocks, kThreads, 0, s>>>(d, f, b);
}

void launch_pcg32_iteration(PcgDev32 &f, cudaStream_t s) {
    k_spmv_dot32<<<f.blocks, kThreads, 0, s>>>(f);
    k_update32<<<f.blocks, kThreads, 0, s>>>(f);
    k_pupdate32<<<f.blocks, kThreads, 0, s>>>(f);
}

void launch_refine_apply(double *x, const float *e, int64_t n, cudaStream_t s) {
    k_refine_apply<<<unsigned((n + 255) / 256), 256, 0, s>>>(x, e, n);
}

}  // namespace spg
