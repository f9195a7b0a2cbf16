// spg_pcg_solve_noalloc: the Jacobi-PCG Poisson solve on a caller-provided
// CSR matrix, with all of its working memory in one file-scope device array,
// so the call allocates nothing.
//
// Who needs it: callers that must not call cudaMalloc/cudaFree. One kind owns
// every byte of device memory through its own pool, as a PyTorch caching
// allocator or a fixed arena does. The other runs in a loop where the device
// synchronisation that cudaMalloc and cudaFree can imply is not allowed.
// Such a caller already holds the matrix, the right-hand side and the solution
// vector in memory it allocated itself; this entry point needs nothing else.
//
// The scratch array (r, z, p, q, the Jacobi inverse diagonal, per-block
// partial sums and the CG scalars) is sized for kNoAllocMaxRows rows:
// 5 * 131072 doubles + 3 * 512 block partials + scalars, about 5.3 MB, which
// every GPU that loads the library keeps until the process exits.
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "spg_internal.h"

namespace spg {

namespace {

constexpr int64_t kNoAllocMaxRows = int64_t(1) << 17;
constexpr int kNaThreads = 256;
constexpr int kNaMaxBlocks = 512;
constexpr int kNaChunk = 8;  // iterations launched between convergence checks
constexpr int64_t kScalarWords = 16;
constexpr int64_t kScratchWords = 5 * kNoAllocMaxRows + 3 * kNaMaxBlocks + kScalarWords;
static_assert(sizeof(PcgScalars) <= kScalarWords * sizeof(double), "scalar slot too small");

// The one scratch array shared by every call on a device.
static __device__ __align__(256) double g_pcg_scratch[kScratchWords];

constexpr unsigned kFull = 0xffffffffu;

struct NaArgs {
    int64_t n;
    const int32_t *row_ptr, *col;
    const double *val, *b;
    double *x;
    double *r, *z, *p, *q, *dinv, *partials;
    PcgScalars *sc;
};

__device__ __forceinline__ double na_warp_sum(double v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(kFull, v, off);
    return v;
}

// Two block sums into partials, then the last block (ticket) totals them in
// block order; true in thread 0 of that block.
__device__ bool na_reduce2(double a, double b, double *partials, PcgScalars *sc, double tot[2]) {
    __shared__ double sa[kNaThreads / 32], sb[kNaThreads / 32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    a = na_warp_sum(a);
    b = na_warp_sum(b);
    if (lane == 0) {
        sa[wid] = a;
        sb[wid] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ta = 0.0, tb = 0.0;
        for (int w = 0; w < kNaThreads / 32; ++w) {
            ta += sa[w];
            tb += sb[w];
        }
        partials[2 * blockIdx.x] = ta;
        partials[2 * blockIdx.x + 1] = tb;
        __threadfence();
        last = atomicInc(&sc->ticket, gridDim.x - 1) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return false;
    __threadfence();
    double ta = 0.0, tb = 0.0;
    for (unsigned k = 0; k < gridDim.x; ++k) {
        ta += __ldcg(partials + 2 * k);
        tb += __ldcg(partials + 2 * k + 1);
    }
    tot[0] = ta;
    tot[1] = tb;
    return true;
}

__device__ __forceinline__ double na_row(const NaArgs &a, const double *__restrict__ v, int64_t i) {
    double s = 0.0;
    for (int32_t k = a.row_ptr[i]; k < a.row_ptr[i + 1]; ++k) s = fma(a.val[k], v[a.col[k]], s);
    return s;
}

// Jacobi inverse diagonal, r = b - A x, z = D^-1 r, p = z; rz, bb; then rr.
// A row without a stored diagonal, or with a zero or non-finite one, sets
// bit 0 of sc->flags and the host refuses the solve.
__global__ void __launch_bounds__(kNaThreads) k_na_setup(NaArgs a) {
    double rz = 0.0, bb = 0.0;
    bool bad = false;
    for (int64_t i = int64_t(blockIdx.x) * kNaThreads + threadIdx.x; i < a.n; i += int64_t(gridDim.x) * kNaThreads) {
        double d = 0.0;
        bool found = false;
        for (int32_t k = a.row_ptr[i]; k < a.row_ptr[i + 1]; ++k)
            if (a.col[k] == i) {
                d = a.val[k];
                found = true;
            }
        if (!found || !(fabs(d) > 0.0) || !isfinite(d)) {
            bad = true;
            d = 1.0;
        }
        const double di = 1.0 / d;
        const double ri = a.b[i] - na_row(a, a.x, i);
        const double zi = ri * di;
        a.dinv[i] = di;
        a.r[i] = ri;
        a.z[i] = zi;
        a.p[i] = zi;
        rz += ri * zi;
        bb += a.b[i] * a.b[i];
    }
    if (bad) atomicOr(&a.sc->flags, 1);
    double tot[2];
    if (na_reduce2(rz, bb, a.partials, a.sc, tot)) {
        a.sc->rz = tot[0];
        a.sc->bb = tot[1];
        a.sc->iters = 0;
        a.sc->converged = tot[1] == 0.0 ? 1 : 0;
    }
}

// rr of the initial residual (separate pass: the setup kernel's reduction
// slot carries rz and bb).
__global__ void __launch_bounds__(kNaThreads) k_na_rr(NaArgs a) {
    double rr = 0.0;
    for (int64_t i = int64_t(blockIdx.x) * kNaThreads + threadIdx.x; i < a.n; i += int64_t(gridDim.x) * kNaThreads)
        rr += a.r[i] * a.r[i];
    double tot[2];
    if (na_reduce2(rr, 0.0, a.partials, a.sc, tot)) {
        a.sc->rr = tot[0];
        if (tot[0] <= a.sc->tol2 * a.sc->bb) a.sc->converged = 1;
    }
}

__global__ void __launch_bounds__(kNaThreads) k_na_spmv_dot(NaArgs a) {
    if (a.sc->converged) return;
    double pq = 0.0;
    for (int64_t i = int64_t(blockIdx.x) * kNaThreads + threadIdx.x; i < a.n; i += int64_t(gridDim.x) * kNaThreads) {
        const double qi = na_row(a, a.p, i);
        a.q[i] = qi;
        pq += a.p[i] * qi;
    }
    double tot[2];
    if (na_reduce2(pq, 0.0, a.partials, a.sc, tot)) {
        if (tot[0] > 0.0) {
            a.sc->alpha = a.sc->rz / tot[0];
        } else {
            a.sc->alpha = 0.0;
            a.sc->converged = 3;  // breakdown: p.Aq <= 0 (A not SPD on this subspace, or NaN)
        }
    }
}

__global__ void __launch_bounds__(kNaThreads) k_na_update(NaArgs a) {
    if (a.sc->converged) return;
    const double alpha = a.sc->alpha;
    double rz = 0.0, rr = 0.0;
    for (int64_t i = int64_t(blockIdx.x) * kNaThreads + threadIdx.x; i < a.n; i += int64_t(gridDim.x) * kNaThreads) {
        a.x[i] += alpha * a.p[i];
        const double ri = a.r[i] - alpha * a.q[i];
        const double zi = ri * a.dinv[i];
        a.r[i] = ri;
        a.z[i] = zi;
        rz += ri * zi;
        rr += ri * ri;
    }
    double tot[2];
    if (na_reduce2(rz, rr, a.partials, a.sc, tot)) {
        PcgScalars *sc = a.sc;
        sc->iters += 1;
        sc->rr = tot[1];
        if (tot[1] <= sc->tol2 * sc->bb) {
            sc->converged = 1;
        } else if (sc->iters >= sc->max_iter) {
            sc->converged = 2;
        } else {
            sc->beta = tot[0] / sc->rz;
            sc->rz = tot[0];
        }
    }
}

// b = 0: the solution is x = 0 whatever the initial guess.
__global__ void __launch_bounds__(kNaThreads) k_na_zero_x(NaArgs a) {
    if (a.sc->bb != 0.0) return;
    for (int64_t i = int64_t(blockIdx.x) * kNaThreads + threadIdx.x; i < a.n; i += int64_t(gridDim.x) * kNaThreads)
        a.x[i] = 0.0;
}

__global__ void __launch_bounds__(kNaThreads) k_na_pupdate(NaArgs a) {
    if (a.sc->converged) return;
    const double beta = a.sc->beta;
    for (int64_t i = int64_t(blockIdx.x) * kNaThreads + threadIdx.x; i < a.n; i += int64_t(gridDim.x) * kNaThreads)
        a.p[i] = a.z[i] + beta * a.p[i];
}

int na_fail(int code, const std::string &msg) {
    set_thread_error(msg);
    return code;
}

// Device address of g_pcg_scratch, looked up once per device with that
// device current (the host-side symbol is only a stand-in for it).
std::mutex g_na_mutex;
double *g_na_ptr[64] = {nullptr};

int na_scratch(double **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return na_fail(SPG_E_NO_DEVICE, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= 64) return na_fail(SPG_E_NO_DEVICE, "device ordinal above 63");
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_ptr[dev]) {
        void *ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_pcg_scratch);
        if (e != cudaSuccess || !ptr)
            return na_fail(SPG_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_na_ptr[dev] = static_cast<double *>(ptr);
    }
    *out = g_na_ptr[dev];
    return SPG_OK;
}

}  // namespace

}  // namespace spg

extern "C" int spg_pcg_solve_noalloc(int64_t n, const int32_t *row_ptr, const int32_t *col, const double *val,
                                     const double *b, double *x, double rtol, int32_t max_iter, void *stream,
                                     int32_t *iters, double *relres) {
    using namespace spg;
    if (n <= 0 || !row_ptr || !col || !val || !b || !x)
        return na_fail(SPG_E_INVALID, "spg_pcg_solve_noalloc: n must be positive and all arrays non-null");
    if (n > kNoAllocMaxRows)
        return na_fail(SPG_E_INVALID, "spg_pcg_solve_noalloc: n = " + std::to_string(n) + " exceeds the " +
                                          std::to_string(kNoAllocMaxRows) + "-row scratch of this entry point");
    if (!(rtol > 0.0) || max_iter < 1)
        return na_fail(SPG_E_INVALID, "spg_pcg_solve_noalloc: rtol must be > 0 and max_iter >= 1");
    double *base = nullptr;
    int rc = na_scratch(&base);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    NaArgs a;
    a.n = n;
    a.row_ptr = row_ptr;
    a.col = col;
    a.val = val;
    a.b = b;
    a.x = x;
    a.r = base;
    a.z = base + kNoAllocMaxRows;
    a.p = base + 2 * kNoAllocMaxRows;
    a.q = base + 3 * kNoAllocMaxRows;
    a.dinv = base + 4 * kNoAllocMaxRows;
    a.partials = base + 5 * kNoAllocMaxRows;
    a.sc = reinterpret_cast<PcgScalars *>(base + 5 * kNoAllocMaxRows + 3 * kNaMaxBlocks);
    // The scalars keep the previous call's values: start from a clean block
    // (ticket 0, not converged) every call.
    PcgScalars init;
    std::memset(&init, 0, sizeof(init));
    init.tol2 = rtol * rtol;
    init.max_iter = max_iter;
    cudaError_t e = cudaMemcpyAsync(a.sc, &init, sizeof(init), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return na_fail(SPG_E_CUDA, std::string("scalar reset: ") + cudaGetErrorString(e));
    const int64_t want = (n + kNaThreads - 1) / kNaThreads;
    const unsigned blocks = unsigned(want < kNaMaxBlocks ? want : kNaMaxBlocks);
    k_na_setup<<<blocks, kNaThreads, 0, s>>>(a);
    k_na_rr<<<blocks, kNaThreads, 0, s>>>(a);
    k_na_zero_x<<<blocks, kNaThreads, 0, s>>>(a);
    PcgScalars hs;
    for (;;) {
        e = cudaMemcpyAsync(&hs, a.sc, sizeof(hs), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return na_fail(SPG_E_CUDA, std::string("PCG: ") + cudaGetErrorString(e));
        if (hs.flags)
            return na_fail(SPG_E_INVALID,
                           "spg_pcg_solve_noalloc: a row has no stored diagonal entry, or a zero or non-finite one");
        if (hs.converged) break;
        for (int k = 0; k < kNaChunk; ++k) {
            k_na_spmv_dot<<<blocks, kNaThreads, 0, s>>>(a);
            k_na_update<<<blocks, kNaThreads, 0, s>>>(a);
            k_na_pupdate<<<blocks, kNaThreads, 0, s>>>(a);
        }
        e = cudaGetLastError();
        if (e != cudaSuccess) return na_fail(SPG_E_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    }
    if (iters) *iters = hs.iters;
    if (relres) *relres = hs.bb > 0.0 ? std::sqrt(hs.rr / hs.bb) : 0.0;
    if (hs.converged == 2)
        return na_fail(SPG_E_NOT_CONVERGED, "spg_pcg_solve_noalloc: PCG did not converge within max_iter");
    if (hs.converged == 3)
        return na_fail(SPG_E_NOT_CONVERGED,
                       "spg_pcg_solve_noalloc: CG breakdown (p.Ap <= 0 after " + std::to_string(hs.iters) +
                           " iterations): the matrix is not SPD, or the data hold NaN");
    return SPG_OK;
}
