// Smoothed-aggregation algebraic multigrid hierarchy for the Poisson
// stiffness matrix (host C++, built once per mesh).
//
// The reference solves K phi = b with Belos CG preconditioned by MueLu
// (src/FiniteElementMethod/Solvers/MatrixEquationSolver.cpp:359-427), whose
// default is smoothed aggregation with Chebyshev smoothing. This builds that
// kind of hierarchy for the GPU V-cycle in kernels_amg.cu:
//   * strength of connection |a_ij| >= theta sqrt(|a_ii a_jj|), theta = 0.08;
//   * three-pass greedy aggregation in row order (deterministic); rows with
//     no strong neighbour (the identity rows of Dirichlet nodes) belong to no
//     aggregate and stay on the fine level;
//   * tentative prolongator: the normalised constant on each aggregate;
//   * P = (I - omega D^-1 A) T with omega = 4 / (3 lambda_max(D^-1 A));
//   * A_c = P^T A P (weak couplings optionally lumped onto the diagonal),
//     R = P^T; levels until at most AmgOptions::coarse_rows rows remain;
//   * the coarsest operator is inverted densely (Cholesky).
// lambda_max comes from 30 power iterations on D^-1 A (times 1.1), the same
// bound the Chebyshev smoother uses.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include <omp.h>

#include "spg_internal.h"

namespace spg {

namespace {

constexpr int kMaxLevels = 12;
constexpr int kPowerIters = 30;

void transpose(const AmgCsr &A, AmgCsr &T) {
    T.n = A.m;
    T.m = A.n;
    T.rp.assign(T.n + 1, 0);
    for (int32_t c : A.ci) T.rp[c + 1]++;
    for (int64_t i = 0; i < T.n; ++i) T.rp[i + 1] += T.rp[i];
    T.ci.resize(A.ci.size());
    T.v.resize(A.v.size());
    std::vector<int64_t> pos(T.rp.begin(), T.rp.end() - 1);
    for (int64_t i = 0; i < A.n; ++i)
        for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k) {
            const int64_t o = pos[A.ci[k]]++;
            T.ci[o] = int32_t(i);
            T.v[o] = A.v[k];
        }
}

// C = A B (row-wise, columns sorted), OpenMP over rows with a dense marker
// per thread; two passes (count, fill) so the result is independent of the
// thread count.
void spgemm(const AmgCsr &A, const AmgCsr &B, AmgCsr &C) {
    C.n = A.n;
    C.m = B.m;
    C.rp.assign(C.n + 1, 0);
    const int nth = omp_get_max_threads();
    std::vector<std::vector<int64_t>> mark(nth, std::vector<int64_t>(B.m, -1));
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < A.n; ++i) {
        auto &mk = mark[omp_get_thread_num()];
        int64_t cnt = 0;
        for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k) {
            const int32_t j = A.ci[k];
            for (int64_t l = B.rp[j]; l < B.rp[j + 1]; ++l)
                if (mk[B.ci[l]] != i) {
                    mk[B.ci[l]] = i;
                    cnt++;
                }
        }
        C.rp[i + 1] = cnt;
    }
    for (int64_t i = 0; i < C.n; ++i) C.rp[i + 1] += C.rp[i];
    C.ci.resize(C.rp[C.n]);
    C.v.resize(C.rp[C.n]);
    for (auto &mk : mark) std::fill(mk.begin(), mk.end(), -1);
    std::vector<std::vector<double>> acc(nth, std::vector<double>(B.m, 0.0));
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < A.n; ++i) {
        auto &mk = mark[omp_get_thread_num()];
        auto &ac = acc[omp_get_thread_num()];
        int64_t o = C.rp[i];
        for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k) {
            const int32_t j = A.ci[k];
            const double a = A.v[k];
            for (int64_t l = B.rp[j]; l < B.rp[j + 1]; ++l) {
                const int32_t c = B.ci[l];
                if (mk[c] != i) {
                    mk[c] = i;
                    C.ci[o++] = c;
                    ac[c] = 0.0;
                }
                ac[c] += a * B.v[l];
            }
        }
        std::sort(C.ci.begin() + C.rp[i], C.ci.begin() + C.rp[i + 1]);
        for (int64_t q = C.rp[i]; q < C.rp[i + 1]; ++q) C.v[q] = ac[C.ci[q]];
    }
}

// Removes exactly-zero entries (the diagonal stays).
void drop_zeros(AmgCsr &A) {
    int64_t o = 0;
    std::vector<int64_t> rp(A.n + 1, 0);
    for (int64_t i = 0; i < A.n; ++i) {
        for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k)
            if (A.v[k] != 0.0 || (A.n == A.m && A.ci[k] == i)) {
                A.ci[o] = A.ci[k];
                A.v[o] = A.v[k];
                ++o;
            }
        rp[i + 1] = o;
    }
    A.rp.swap(rp);
    A.ci.resize(o);
    A.v.resize(o);
}

double lambda_max(const AmgCsr &A, const std::vector<double> &dinv) {
    const int64_t n = A.n;
    std::vector<double> x(n), y(n);
    for (int64_t i = 0; i < n; ++i) x[i] = 1.0 + 0.37 * double((i * 7919) % 101) / 101.0;
    double lam = 1.0;
    for (int it = 0; it < kPowerIters; ++it) {
        double nx = 0.0;
        for (int64_t i = 0; i < n; ++i) nx += x[i] * x[i];
        nx = std::sqrt(nx);
        if (!(nx > 0.0)) break;
        for (int64_t i = 0; i < n; ++i) x[i] /= nx;
#pragma omp parallel for
        for (int64_t i = 0; i < n; ++i) {
            double s = 0.0;
            for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k) s += A.v[k] * x[A.ci[k]];
            y[i] = dinv[i] * s;
        }
        double num = 0.0;
        for (int64_t i = 0; i < n; ++i) num += x[i] * y[i];
        lam = num;
        x.swap(y);
    }
    return lam;
}

// Aggregates of the strength graph; agg[i] = -1 for rows with no strong
// neighbour. Returns the number of aggregates.
int64_t aggregate(const AmgCsr &A, double theta, std::vector<int64_t> &agg) {
    const int64_t n = A.n;
    std::vector<double> d(n, 0.0);
    for (int64_t i = 0; i < n; ++i)
        for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k)
            if (A.ci[k] == i) d[i] = std::fabs(A.v[k]);
    std::vector<int64_t> srp(n + 1, 0);
    std::vector<int32_t> sci;
    sci.reserve(A.ci.size());
    for (int64_t i = 0; i < n; ++i) {
        for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k) {
            const int32_t j = A.ci[k];
            if (j != i && std::fabs(A.v[k]) >= theta * std::sqrt(d[i] * d[j])) sci.push_back(j);
        }
        srp[i + 1] = int64_t(sci.size());
    }
    agg.assign(n, -1);
    int64_t na = 0;
    // pass 1: a row whose strong neighbours are all free starts an aggregate with them
    for (int64_t i = 0; i < n; ++i) {
        if (agg[i] >= 0 || srp[i + 1] == srp[i]) continue;
        bool free_nb = true;
        for (int64_t k = srp[i]; k < srp[i + 1] && free_nb; ++k) free_nb = agg[sci[k]] < 0;
        if (!free_nb) continue;
        agg[i] = na;
        for (int64_t k = srp[i]; k < srp[i + 1]; ++k) agg[sci[k]] = na;
        na++;
    }
    // pass 2: remaining rows join the aggregate of their strongest aggregated neighbour
    std::vector<int64_t> a2 = agg;
    for (int64_t i = 0; i < n; ++i) {
        if (agg[i] >= 0 || srp[i + 1] == srp[i]) continue;
        double best = -1.0;
        for (int64_t k = srp[i]; k < srp[i + 1]; ++k) {
            const int32_t j = sci[k];
            if (agg[j] < 0) continue;
            double w = 0.0;
            for (int64_t q = A.rp[i]; q < A.rp[i + 1]; ++q)
                if (A.ci[q] == j) w = std::fabs(A.v[q]);
            if (w > best) {
                best = w;
                a2[i] = agg[j];
            }
        }
    }
    agg.swap(a2);
    // pass 3: rows still free start aggregates with their free strong neighbours
    for (int64_t i = 0; i < n; ++i) {
        if (agg[i] >= 0 || srp[i + 1] == srp[i]) continue;
        agg[i] = na;
        for (int64_t k = srp[i]; k < srp[i + 1]; ++k)
            if (agg[sci[k]] < 0) agg[sci[k]] = na;
        na++;
    }
    return na;
}

// Moves the weak positive couplings 0 < a_ij < eps sqrt(|a_ii a_jj|) of a
// coarse operator onto the diagonal. Row sums, hence the constant near-null
// space, are kept; the criterion is symmetric, so the operator stays
// symmetric; and the change for one pair, a_ij (e_i - e_j)(e_i - e_j)^T, is
// positive semidefinite, so the operator stays positive definite.
void filter_weak(AmgCsr &A, double eps) {
    std::vector<double> d(A.n, 0.0);
    for (int64_t i = 0; i < A.n; ++i)
        for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k)
            if (A.ci[k] == i) d[i] = A.v[k];
    std::vector<int64_t> rp(A.n + 1, 0);
    int64_t o = 0;
    for (int64_t i = 0; i < A.n; ++i) {
        double lump = 0.0;
        const int64_t start = o;
        int64_t diag = -1;
        for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k) {
            const int32_t j = A.ci[k];
            if (j != i && A.v[k] > 0.0 && A.v[k] < eps * std::sqrt(std::fabs(d[i] * d[j]))) {
                lump += A.v[k];
                continue;
            }
            if (j == i) diag = o;
            A.ci[o] = j;
            A.v[o] = A.v[k];
            ++o;
        }
        if (diag >= 0) A.v[diag] += lump;
        (void)start;
        rp[i + 1] = o;
    }
    A.rp.swap(rp);
    A.ci.resize(o);
    A.v.resize(o);
}

// In-place Cholesky of a dense SPD matrix (lower), then its inverse.
bool dense_inverse(int64_t n, std::vector<double> &a, std::vector<double> &inv) {
    for (int64_t j = 0; j < n; ++j) {
        double s = a[j * n + j];
        for (int64_t k = 0; k < j; ++k) s -= a[j * n + k] * a[j * n + k];
        if (!(s > 0.0)) return false;
        const double l = std::sqrt(s);
        a[j * n + j] = l;
#pragma omp parallel for schedule(static)
        for (int64_t i = j + 1; i < n; ++i) {
            double t = a[i * n + j];
            for (int64_t k = 0; k < j; ++k) t -= a[i * n + k] * a[j * n + k];
            a[i * n + j] = t / l;
        }
    }
    inv.assign(n * n, 0.0);
#pragma omp parallel for schedule(dynamic, 8)
    for (int64_t c = 0; c < n; ++c) {
        std::vector<double> e(n, 0.0);
        e[c] = 1.0;
        for (int64_t i = 0; i < n; ++i) {  // L y = e
            double t = e[i];
            for (int64_t k = 0; k < i; ++k) t -= a[i * n + k] * e[k];
            e[i] = t / a[i * n + i];
        }
        for (int64_t i = n - 1; i >= 0; --i) {  // L^T x = y
            double t = e[i];
            for (int64_t k = i + 1; k < n; ++k) t -= a[k * n + i] * e[k];
            e[i] = t / a[i * n + i];
        }
        for (int64_t i = 0; i < n; ++i) inv[i * n + c] = e[i];
    }
    return true;
}

}  // namespace

int amg_setup(int64_t n, const int32_t *row_ptr, const int32_t *col, const double *val, AmgHost &out,
              std::string &err, const AmgOptions &opt) {
    out = AmgHost{};
    AmgCsr A;
    A.n = A.m = n;
    A.rp.assign(row_ptr, row_ptr + n + 1);
    A.ci.assign(col, col + row_ptr[n]);
    A.v.assign(val, val + row_ptr[n]);
    drop_zeros(A);
    for (int lev = 0; lev < kMaxLevels; ++lev) {
        AmgLevelHost L;
        L.dinv.assign(A.n, 0.0);
        for (int64_t i = 0; i < A.n; ++i)
            for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k)
                if (A.ci[k] == i) L.dinv[i] = A.v[k] != 0.0 ? 1.0 / A.v[k] : 0.0;
        L.lam = 1.1 * lambda_max(A, L.dinv);
        if (A.n <= opt.coarse_rows) {
            // coarsest level: dense inverse
            std::vector<double> dense(A.n * A.n, 0.0);
            for (int64_t i = 0; i < A.n; ++i)
                for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k) dense[i * A.n + A.ci[k]] = A.v[k];
            out.nc = A.n;
            if (!dense_inverse(A.n, dense, out.coarse_inv)) {
                err = "amg: coarsest operator is not positive definite";
                return SPG_E_INVALID;
            }
            L.A = std::move(A);
            out.levels.push_back(std::move(L));
            return SPG_OK;
        }
        std::vector<int64_t> agg;
        const int64_t na = aggregate(A, opt.theta, agg);
        if (na == 0 || na * 5 > A.n * 4) {  // no coarsening progress: stop here with a dense coarse level
            if (A.n > 8 * opt.coarse_rows) {
                err = "amg: aggregation stalled at " + std::to_string(A.n) + " rows";
                return SPG_E_INVALID;
            }
            std::vector<double> dense(A.n * A.n, 0.0);
            for (int64_t i = 0; i < A.n; ++i)
                for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k) dense[i * A.n + A.ci[k]] = A.v[k];
            out.nc = A.n;
            if (!dense_inverse(A.n, dense, out.coarse_inv)) {
                err = "amg: coarsest operator is not positive definite";
                return SPG_E_INVALID;
            }
            L.A = std::move(A);
            out.levels.push_back(std::move(L));
            return SPG_OK;
        }
        // tentative prolongator
        std::vector<int64_t> size(na, 0);
        for (int64_t i = 0; i < A.n; ++i)
            if (agg[i] >= 0) size[agg[i]]++;
        AmgCsr T;
        T.n = A.n;
        T.m = na;
        T.rp.assign(A.n + 1, 0);
        for (int64_t i = 0; i < A.n; ++i) {
            T.rp[i + 1] = T.rp[i] + (agg[i] >= 0 ? 1 : 0);
            if (agg[i] >= 0) {
                T.ci.push_back(int32_t(agg[i]));
                T.v.push_back(1.0 / std::sqrt(double(size[agg[i]])));
            }
        }
        // P = T - omega D^-1 A T (P = T past opt.smooth_levels)
        AmgCsr AT;
        spgemm(A, T, AT);
        const double omega = lev < opt.smooth_levels ? 4.0 / (3.0 * L.lam) : 0.0;
        AmgCsr P;
        P.n = A.n;
        P.m = na;
        P.rp.assign(A.n + 1, 0);
        for (int64_t i = 0; i < A.n; ++i) {
            // merge row i of T (at most one entry) and of -omega D^-1 AT (sorted)
            const double s = -omega * L.dinv[i];
            const bool has_t = T.rp[i + 1] > T.rp[i];
            const int32_t tc = has_t ? T.ci[T.rp[i]] : -1;
            bool placed = !has_t;
            for (int64_t k = AT.rp[i]; k < AT.rp[i + 1]; ++k) {
                const int32_t c = AT.ci[k];
                if (!placed && tc < c) {
                    P.ci.push_back(tc);
                    P.v.push_back(T.v[T.rp[i]]);
                    placed = true;
                }
                double v = s * AT.v[k];
                if (c == tc) {
                    v += T.v[T.rp[i]];
                    placed = true;
                }
                P.ci.push_back(c);
                P.v.push_back(v);
            }
            if (!placed) {
                P.ci.push_back(tc);
                P.v.push_back(T.v[T.rp[i]]);
            }
            P.rp[i + 1] = int64_t(P.ci.size());
        }
        drop_zeros(P);
        AmgCsr R, AP, Ac;
        transpose(P, R);
        spgemm(A, P, AP);
        spgemm(R, AP, Ac);
        drop_zeros(Ac);
        if (opt.filter > 0.0) filter_weak(Ac, opt.filter);
        L.A = std::move(A);
        L.P = std::move(P);
        L.R = std::move(R);
        out.levels.push_back(std::move(L));
        A = std::move(Ac);
    }
    err = "amg: too many levels";
    return SPG_E_INVALID;
}

}  // namespace spg
