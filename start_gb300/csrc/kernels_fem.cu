// FEM set-up on the GPU: the P1 element maps and volumes, the node -> tet
// incidence with the dual volumes, and the stiffness matrix in CSR with the
// Dirichlet rows replaced by identity rows and the Dirichlet columns moved to
// the right-hand side (the lifting and the eliminated couplings). This is the
// work of GSMAssembler (src/FiniteElementMethod/Assemblers/GSMAssembler.cpp:10-72)
// and MatrixBoundaryConditionsManager (src/FiniteElementMethod/BoundaryConditions/
// MatrixBoundaryConditionsManager.cpp:5-39), done per row instead of per
// element: row i sums the contributions of its incident tets in increasing
// tet order, so there is no atomic on a value and the matrix is the same on
// every run, bit for bit equal to the CPU oracle's (same expressions, built
// with --fmad=false). Face matching, surface triangles and the point-location
// grid stay on the host.
#include <algorithm>
#include <vector>

#include "spg_internal.h"

namespace spg {

namespace {

// Rows of J^-1, J = [x1-x0, x2-x0, x3-x0]; returns det J (0: degenerate).
__device__ double tet_map_dev(const double *x0, const double *x1, const double *x2, const double *x3, double M[9]) {
    const double a0 = x1[0] - x0[0], a1 = x1[1] - x0[1], a2 = x1[2] - x0[2];
    const double b0 = x2[0] - x0[0], b1 = x2[1] - x0[1], b2 = x2[2] - x0[2];
    const double c0 = x3[0] - x0[0], c1 = x3[1] - x0[1], c2 = x3[2] - x0[2];
    const double bc0 = b1 * c2 - b2 * c1, bc1 = b2 * c0 - b0 * c2, bc2 = b0 * c1 - b1 * c0;
    const double det = a0 * bc0 + a1 * bc1 + a2 * bc2;
    if (det == 0.0) return 0.0;
    M[0] = bc0 / det;
    M[1] = bc1 / det;
    M[2] = bc2 / det;
    M[3] = (c1 * a2 - c2 * a1) / det;
    M[4] = (c2 * a0 - c0 * a2) / det;
    M[5] = (c0 * a1 - c1 * a0) / det;
    M[6] = (a1 * b2 - a2 * b1) / det;
    M[7] = (a2 * b0 - a0 * b2) / det;
    M[8] = (a0 * b1 - a1 * b0) / det;
    return det;
}

// Orientation (nodes 2 and 3 swapped when det < 0), map, origin and volume of
// each tet; *bad receives the lowest tet with a bad node index or zero volume.
__global__ void k_elements(const double *__restrict__ xyz, int32_t *__restrict__ tn, int64_t nt, int64_t nn,
                           TetRec *__restrict__ rec, double *__restrict__ vol, int *bad) {
    const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    int32_t v[4];
    for (int k = 0; k < 4; ++k) {
        v[k] = tn[4 * t + k];
        if (v[k] < 0 || v[k] >= nn) {
            atomicMin(bad, int(t));
            return;
        }
    }
    const double *p[4];
    for (int k = 0; k < 4; ++k) p[k] = xyz + 3 * int64_t(v[k]);
    double M[9];
    double det = tet_map_dev(p[0], p[1], p[2], p[3], M);
    if (det < 0.0) {
        tn[4 * t + 2] = v[3];
        tn[4 * t + 3] = v[2];
        const double *q = p[2];
        p[2] = p[3];
        p[3] = q;
        det = tet_map_dev(p[0], p[1], p[2], p[3], M);
    }
    if (!(det > 0.0)) {
        atomicMin(bad, int(t));
        return;
    }
    TetRec &r = rec[t];
    for (int k = 0; k < 9; ++k) r.M[k] = M[k];
    for (int k = 0; k < 3; ++k) {
        r.x0[k] = p[0][k];
        r.H[k] = 0.0;
    }
    r.ezero = 0u;
    r.pad = 0u;
    vol[t] = det / 6.0;
}

__global__ void k_inc_count(const int32_t *__restrict__ tn, int64_t n4, int32_t *__restrict__ cnt) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n4) atomicAdd(cnt + tn[i], 1);
}

__global__ void k_inc_fill(const int32_t *__restrict__ tn, int64_t n4, int64_t *__restrict__ cur,
                           int32_t *__restrict__ ntet) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n4) ntet[atomicAdd(reinterpret_cast<unsigned long long *>(cur + tn[i]), 1ull)] = int32_t(i);
}

template <class T>
__device__ void insertion_sort(T *a, int64_t n) {
    for (int64_t k = 1; k < n; ++k) {
        const T x = a[k];
        int64_t j = k - 1;
        while (j >= 0 && a[j] > x) {
            a[j + 1] = a[j];
            --j;
        }
        a[j + 1] = x;
    }
}

// Each node's incident (tet * 4 + vertex) list in increasing order, and its
// dual volume: a quarter of the incident volumes summed in that order.
__global__ void k_inc_sort_dual(const int64_t *__restrict__ nstart, int32_t *__restrict__ ntet, int64_t nn,
                                const double *__restrict__ vol, double *__restrict__ dual) {
    const int64_t n = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (n >= nn) return;
    const int64_t k0 = nstart[n], k1 = nstart[n + 1];
    insertion_sort(ntet + k0, k1 - k0);
    double s = 0.0;
    for (int64_t k = k0; k < k1; ++k) s += vol[ntet[k] >> 2];
    dual[n] = 0.25 * s;
}

// Row structure: the free nodes of the incident tets of a free node, sorted
// and unique, left at the start of its candidate segment (4 entries per
// incidence); a Dirichlet row has the one diagonal entry.
__global__ void k_row_cols(const int64_t *__restrict__ nstart, const int32_t *__restrict__ ntet,
                           const int32_t *__restrict__ tn, const uint8_t *__restrict__ is_dir, int64_t nn,
                           int32_t *__restrict__ cand, int32_t *__restrict__ rowlen) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    if (is_dir[i]) {
        rowlen[i] = 1;
        return;
    }
    // Each candidate goes into the sorted unique list c[0, u) unless present:
    // the writes are the list's own shifts, not a sort of every candidate.
    int32_t *c = cand + 4 * nstart[i];
    int64_t u = 0;
    for (int64_t k = nstart[i]; k < nstart[i + 1]; ++k) {
        const int32_t *v = tn + 4 * int64_t(ntet[k] >> 2);
        for (int q = 0; q < 4; ++q) {
            const int32_t x = v[q];
            if (is_dir[x]) continue;
            int64_t j = u;
            while (j > 0 && c[j - 1] > x) --j;
            if (j > 0 && c[j - 1] == x) continue;
            for (int64_t r = u; r > j; --r) c[r] = c[r - 1];
            c[j] = x;
            ++u;
        }
    }
    rowlen[i] = int32_t(u);
}

// Values, diagonal, lifting and eliminated couplings of row i: kab =
// vol (G_a . G_b) of each incident tet in increasing tet order; a free column
// adds to its entry, a Dirichlet column to the lifting (times its value) and
// to the row's eliminated coupling with that node (kept in order of first
// appearance, then sorted by node).
__global__ void k_row_values(const int64_t *__restrict__ nstart, const int32_t *__restrict__ ntet,
                             const int32_t *__restrict__ tn, const uint8_t *__restrict__ is_dir,
                             const double *__restrict__ dir_value, const TetRec *__restrict__ rec,
                             const double *__restrict__ vol, int64_t nn, const int32_t *__restrict__ cand,
                             const int32_t *__restrict__ row_ptr, int32_t *__restrict__ col, double *__restrict__ val,
                             double *__restrict__ diag, double *__restrict__ lift, int32_t *__restrict__ ecol,
                             double *__restrict__ eval, int32_t *__restrict__ ecnt) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    const int32_t r0 = row_ptr[i], len = row_ptr[i + 1] - r0;
    int32_t *c0 = col + r0;
    double *v0 = val + r0;
    if (is_dir[i]) {
        c0[0] = int32_t(i);
        v0[0] = 1.0;
        diag[i] = 1.0;
        lift[i] = 0.0;
        ecnt[i] = 0;
        return;
    }
    const int32_t *c = cand + 4 * nstart[i];
    for (int32_t k = 0; k < len; ++k) {
        c0[k] = c[k];
        v0[k] = 0.0;
    }
    int32_t *ec = ecol + 4 * nstart[i];
    double *ev = eval + 4 * nstart[i];
    int32_t ne = 0;
    double lf = 0.0;
    for (int64_t k = nstart[i]; k < nstart[i + 1]; ++k) {
        const int64_t t = ntet[k] >> 2;
        const int a = ntet[k] & 3;
        const TetRec &r = rec[t];
        double G[4][3];
        for (int q = 0; q < 3; ++q) {
            G[1][q] = r.M[q];
            G[2][q] = r.M[3 + q];
            G[3][q] = r.M[6 + q];
            G[0][q] = -(G[1][q] + G[2][q] + G[3][q]);
        }
        const int32_t *v = tn + 4 * t;
        for (int b = 0; b < 4; ++b) {
            const double kab = vol[t] * (G[a][0] * G[b][0] + G[a][1] * G[b][1] + G[a][2] * G[b][2]);
            const int32_t j = v[b];
            if (is_dir[j]) {
                lf += kab * dir_value[j];
                int32_t e = 0;
                while (e < ne && ec[e] != j) ++e;
                if (e == ne) {
                    ec[ne] = j;
                    ev[ne] = kab;
                    ++ne;
                } else {
                    ev[e] += kab;
                }
            } else {
                int32_t lo = 0, hi = len;  // lower bound of j among the row's columns
                while (lo < hi) {
                    const int32_t mid = (lo + hi) >> 1;
                    if (c0[mid] < j)
                        lo = mid + 1;
                    else
                        hi = mid;
                }
                v0[lo] += kab;
            }
        }
    }
    lift[i] = lf;
    double d = 1.0;
    for (int32_t k = 0; k < len; ++k)
        if (c0[k] == int32_t(i)) d = v0[k];
    diag[i] = d;
    for (int32_t q = 1; q < ne; ++q) {  // sort the eliminated couplings by node
        const int32_t x = ec[q];
        const double y = ev[q];
        int32_t j = q - 1;
        while (j >= 0 && ec[j] > x) {
            ec[j + 1] = ec[j];
            ev[j + 1] = ev[j];
            --j;
        }
        ec[j + 1] = x;
        ev[j + 1] = y;
    }
    ecnt[i] = ne;
}

__global__ void k_elim_fill(const int64_t *__restrict__ nstart, const int32_t *__restrict__ ecol,
                            const double *__restrict__ eval, const int64_t *__restrict__ eoff, int64_t nn,
                            int32_t *__restrict__ out_row, int32_t *__restrict__ out_col, double *__restrict__ out_val) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    const int64_t o = eoff[i], ne = eoff[i + 1] - o;
    for (int64_t q = 0; q < ne; ++q) {
        out_row[o + q] = int32_t(i);
        out_col[o + q] = ecol[4 * nstart[i] + q];
        out_val[o + q] = eval[4 * nstart[i] + q];
    }
}

inline unsigned blocks(int64_t n) { return unsigned((n + 255) / 256); }

// RAII device buffer for the set-up (freed on every return path).
template <class T>
struct DevBuf {
    T *p = nullptr;
    ~DevBuf() { cudaFree(p); }
    cudaError_t alloc(int64_t n) { return cudaMalloc(reinterpret_cast<void **>(&p), sizeof(T) * size_t(n > 0 ? n : 1)); }
};

#define FEM_CK(x)                                                   \
    do {                                                            \
        const cudaError_t e_ = (x);                                 \
        if (e_ != cudaSuccess) {                                    \
            err = std::string("fem: ") + cudaGetErrorString(e_);    \
            return e_ == cudaErrorMemoryAllocation ? SPG_E_OOM : SPG_E_CUDA; \
        }                                                           \
    } while (0)

std::vector<int64_t> exclusive_scan(const std::vector<int32_t> &c) {
    std::vector<int64_t> s(c.size() + 1, 0);
    for (size_t k = 0; k < c.size(); ++k) s[k + 1] = s[k] + c[k];
    return s;
}

}  // namespace

int fem_elements_gpu(HostMesh &m, std::string &err, int64_t &bad_tet) {
    const int64_t nn = m.n_nodes, nt = m.n_tets;
    DevBuf<double> xyz, vol;
    DevBuf<int32_t> tn;
    DevBuf<TetRec> rec;
    DevBuf<int> bad;
    FEM_CK(xyz.alloc(3 * nn));
    FEM_CK(tn.alloc(4 * nt));
    FEM_CK(rec.alloc(nt));
    FEM_CK(vol.alloc(nt));
    FEM_CK(bad.alloc(1));
    FEM_CK(cudaMemcpy(xyz.p, m.node_xyz.data(), 8 * size_t(3 * nn), cudaMemcpyHostToDevice));
    FEM_CK(cudaMemcpy(tn.p, m.tet_nodes.data(), 4 * size_t(4 * nt), cudaMemcpyHostToDevice));
    const int none = 0x7fffffff;
    FEM_CK(cudaMemcpy(bad.p, &none, sizeof(int), cudaMemcpyHostToDevice));
    k_elements<<<blocks(nt), 256>>>(xyz.p, tn.p, nt, nn, rec.p, vol.p, bad.p);
    FEM_CK(cudaGetLastError());
    int b = none;
    FEM_CK(cudaMemcpy(&b, bad.p, sizeof(int), cudaMemcpyDeviceToHost));
    bad_tet = b == none ? -1 : b;
    if (bad_tet >= 0) return SPG_OK;
    m.rec.resize(nt);
    m.vol.resize(nt);
    FEM_CK(cudaMemcpy(m.tet_nodes.data(), tn.p, 4 * size_t(4 * nt), cudaMemcpyDeviceToHost));
    FEM_CK(cudaMemcpy(m.rec.data(), rec.p, sizeof(TetRec) * size_t(nt), cudaMemcpyDeviceToHost));
    FEM_CK(cudaMemcpy(m.vol.data(), vol.p, 8 * size_t(nt), cudaMemcpyDeviceToHost));
    return SPG_OK;
}

int fem_stiffness_gpu(HostMesh &m, std::string &err) {
    const int64_t nn = m.n_nodes, nt = m.n_tets, n4 = 4 * nt;
    DevBuf<int32_t> tn, cnt, ntet, cand, rowlen, row_ptr, col, ecol, ecnt, orow, ocol;
    DevBuf<int64_t> nstart, cur, eoff;
    DevBuf<double> vol, dual, dirv, val, diag, lift, eval, oval;
    DevBuf<uint8_t> isd;
    DevBuf<TetRec> rec;
    FEM_CK(tn.alloc(n4));
    FEM_CK(cnt.alloc(nn));
    FEM_CK(ntet.alloc(n4));
    FEM_CK(nstart.alloc(nn + 1));
    FEM_CK(cur.alloc(nn));
    FEM_CK(vol.alloc(nt));
    FEM_CK(dual.alloc(nn));
    FEM_CK(rec.alloc(nt));
    FEM_CK(isd.alloc(nn));
    FEM_CK(dirv.alloc(nn));
    FEM_CK(cudaMemcpy(tn.p, m.tet_nodes.data(), 4 * size_t(n4), cudaMemcpyHostToDevice));
    FEM_CK(cudaMemcpy(vol.p, m.vol.data(), 8 * size_t(nt), cudaMemcpyHostToDevice));
    FEM_CK(cudaMemcpy(rec.p, m.rec.data(), sizeof(TetRec) * size_t(nt), cudaMemcpyHostToDevice));
    FEM_CK(cudaMemcpy(isd.p, m.is_dir.data(), size_t(nn), cudaMemcpyHostToDevice));
    FEM_CK(cudaMemcpy(dirv.p, m.dir_value.data(), 8 * size_t(nn), cudaMemcpyHostToDevice));
    // node -> tet incidence
    FEM_CK(cudaMemset(cnt.p, 0, 4 * size_t(nn)));
    k_inc_count<<<blocks(n4), 256>>>(tn.p, n4, cnt.p);
    std::vector<int32_t> hc(nn);
    FEM_CK(cudaMemcpy(hc.data(), cnt.p, 4 * size_t(nn), cudaMemcpyDeviceToHost));
    const std::vector<int64_t> hs = exclusive_scan(hc);
    FEM_CK(cudaMemcpy(nstart.p, hs.data(), 8 * size_t(nn + 1), cudaMemcpyHostToDevice));
    FEM_CK(cudaMemcpy(cur.p, hs.data(), 8 * size_t(nn), cudaMemcpyHostToDevice));
    k_inc_fill<<<blocks(n4), 256>>>(tn.p, n4, cur.p, ntet.p);
    k_inc_sort_dual<<<blocks(nn), 256>>>(nstart.p, ntet.p, nn, vol.p, dual.p);
    FEM_CK(cudaGetLastError());
    m.dual_vol.resize(nn);
    FEM_CK(cudaMemcpy(m.dual_vol.data(), dual.p, 8 * size_t(nn), cudaMemcpyDeviceToHost));
    // row structure
    FEM_CK(cand.alloc(4 * n4));
    FEM_CK(rowlen.alloc(nn));
    k_row_cols<<<blocks(nn), 256>>>(nstart.p, ntet.p, tn.p, isd.p, nn, cand.p, rowlen.p);
    FEM_CK(cudaGetLastError());
    std::vector<int32_t> hl(nn);
    FEM_CK(cudaMemcpy(hl.data(), rowlen.p, 4 * size_t(nn), cudaMemcpyDeviceToHost));
    const std::vector<int64_t> rp64 = exclusive_scan(hl);
    const int64_t nnz = rp64[nn];
    if (nnz >= (int64_t(1) << 31)) {
        err = "mesh: stiffness has more than 2^31 non-zeros";
        return SPG_E_INVALID;
    }
    m.row_ptr.assign(rp64.begin(), rp64.end());
    FEM_CK(row_ptr.alloc(nn + 1));
    FEM_CK(cudaMemcpy(row_ptr.p, m.row_ptr.data(), 4 * size_t(nn + 1), cudaMemcpyHostToDevice));
    // values, diagonal, lifting, eliminated couplings
    FEM_CK(col.alloc(nnz));
    FEM_CK(val.alloc(nnz));
    FEM_CK(diag.alloc(nn));
    FEM_CK(lift.alloc(nn));
    FEM_CK(ecol.alloc(4 * n4));
    FEM_CK(eval.alloc(4 * n4));
    FEM_CK(ecnt.alloc(nn));
    k_row_values<<<blocks(nn), 256>>>(nstart.p, ntet.p, tn.p, isd.p, dirv.p, rec.p, vol.p, nn, cand.p, row_ptr.p,
                                      col.p, val.p, diag.p, lift.p, ecol.p, eval.p, ecnt.p);
    FEM_CK(cudaGetLastError());
    m.col.resize(nnz);
    m.val.resize(nnz);
    m.diag.resize(nn);
    m.lift.resize(nn);
    FEM_CK(cudaMemcpy(m.col.data(), col.p, 4 * size_t(nnz), cudaMemcpyDeviceToHost));
    FEM_CK(cudaMemcpy(m.val.data(), val.p, 8 * size_t(nnz), cudaMemcpyDeviceToHost));
    FEM_CK(cudaMemcpy(m.diag.data(), diag.p, 8 * size_t(nn), cudaMemcpyDeviceToHost));
    FEM_CK(cudaMemcpy(m.lift.data(), lift.p, 8 * size_t(nn), cudaMemcpyDeviceToHost));
    std::vector<int32_t> he(nn);
    FEM_CK(cudaMemcpy(he.data(), ecnt.p, 4 * size_t(nn), cudaMemcpyDeviceToHost));
    const std::vector<int64_t> eo = exclusive_scan(he);
    const int64_t ne = eo[nn];
    FEM_CK(eoff.alloc(nn + 1));
    FEM_CK(cudaMemcpy(eoff.p, eo.data(), 8 * size_t(nn + 1), cudaMemcpyHostToDevice));
    FEM_CK(orow.alloc(ne));
    FEM_CK(ocol.alloc(ne));
    FEM_CK(oval.alloc(ne));
    k_elim_fill<<<blocks(nn), 256>>>(nstart.p, ecol.p, eval.p, eoff.p, nn, orow.p, ocol.p, oval.p);
    FEM_CK(cudaGetLastError());
    m.elim_row.resize(ne);
    m.elim_col.resize(ne);
    m.elim_val.resize(ne);
    if (ne) {
        FEM_CK(cudaMemcpy(m.elim_row.data(), orow.p, 4 * size_t(ne), cudaMemcpyDeviceToHost));
        FEM_CK(cudaMemcpy(m.elim_col.data(), ocol.p, 4 * size_t(ne), cudaMemcpyDeviceToHost));
        FEM_CK(cudaMemcpy(m.elim_val.data(), oval.p, 8 * size_t(ne), cudaMemcpyDeviceToHost));
    }
    return SPG_OK;
}

}  // namespace spg
