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

__device__ __forceinline__ double spmv_row(const int32_t *__restrict__ row_ptr, const int32_t *__restrict__ col,
                                           const double *__restrict__ val, const double *__restrict__ x, int64_t i) {
    const int32_t k0 = __ldg(row_ptr + i), k1 = __ldg(row_ptr + i + 1);
    double s = 0.0;
    for (int32_t k = k0; k < k1; ++k) s += __ldg(val + k) * __ldg(x + __ldg(col + k));
    return s;
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
        const double ri = bi - spmv_row(d.row_ptr, d.col, d.val, d.x, i);
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
        const double qi = spmv_row(d.row_ptr, d.col, d.val, d.p, i);
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

}  // namespace

int pcg_blocks(int64_t n) {
    const int64_t want = (n + kThreads - 1) / kThreads;
    return int(want < 152 * 16 ? (want < 1 ? 1 : want) : 152 * 16);
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

}  // namespace spg
