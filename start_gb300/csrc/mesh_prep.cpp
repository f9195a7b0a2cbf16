// Host-side mesh preparation for libstart_gpu.so.
//
// Replaces the reference's initialisation chain:
//   VolumetricMesh read + per-tet data        src/Geometry/Mesh/Volumetric/VolumetricMesh.cpp:35-121
//   local stiffness + nabla phi (Intrepid2)    VolumetricMesh.cpp:306-380
//   global CRS assembly, row/col = tag - 1     src/FiniteElementMethod/Assemblers/GSMAssembler.cpp:10-118
//   Dirichlet rows                             src/FiniteElementMethod/BoundaryConditions/MatrixBoundaryConditionsManager.cpp:5-39
//   surface triangles (AABB tree source)       src/Geometry/Mesh/Surface/SurfaceMesh.cpp:55-66
//   global bounding box test                   SurfaceMesh.cpp:92-134
//   CubicGrid voxel buckets                    src/Geometry/Mesh/Cubic/CubicGrid.cpp:10-57
//
// P1 elements are assembled in closed form: K_e = V * G G^T with G the four
// barycentric gradients, which is what one-point cubature of constant
// gradients integrates exactly. Dirichlet rows become identity rows and the
// Dirichlet columns move to the right-hand side, which keeps K symmetric
// positive definite for CG (the reference only replaces rows).
//
// Compiled with -ffp-contract=off: the barycentric map computed here feeds the
// FP64 walk, which must agree bit for bit with the CPU oracle.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <numeric>
#include <sstream>

#include "spg_internal.h"

namespace spg {

namespace {

struct FaceRef {
    int32_t b, c;  // two larger node ids of the sorted triple
    int32_t tf;    // tet*4 + local face
};

// Node indices of local face f (opposite local vertex f).
inline void face_nodes(const int32_t *tn, int f, int32_t out[3]) {
    int k = 0;
    for (int v = 0; v < 4; ++v)
        if (v != f) out[k++] = tn[v];
}

inline void sort3(int32_t v[3]) {
    if (v[0] > v[1]) std::swap(v[0], v[1]);
    if (v[1] > v[2]) std::swap(v[1], v[2]);
    if (v[0] > v[1]) std::swap(v[0], v[1]);
}

}  // namespace

// Barycentric map of one tet: rows of J^{-1} where J = [x1-x0, x2-x0, x3-x0].
// Row 0 = (b x c)/det, row 1 = (c x a)/det, row 2 = (a x b)/det.
// The CPU oracle evaluates the same expressions in the same order.
static double tet_map(const double *x0, const double *x1, const double *x2, const double *x3, double M[9]) {
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

int prepare_mesh(const spg_mesh_desc &d, double bbox_expansion, HostMesh &m, std::string &err) {
    std::ostringstream es;
    if (d.n_nodes <= 0 || d.n_tets <= 0 || !d.node_xyz || !d.tet_nodes) {
        err = "mesh: n_nodes, n_tets, node_xyz and tet_nodes are required";
        return SPG_E_INVALID;
    }
    if (d.n_nodes >= (int64_t(1) << 31) || d.n_tets >= (int64_t(1) << 29)) {
        err = "mesh: too large (n_nodes < 2^31, n_tets < 2^29)";
        return SPG_E_INVALID;
    }
    if (d.n_triangles < 0 || (d.n_triangles > 0 && !d.tri_nodes) || d.n_dirichlet < 0 ||
        (d.n_dirichlet > 0 && (!d.dirichlet_nodes || !d.dirichlet_values))) {
        err = "mesh: triangle or Dirichlet arrays missing";
        return SPG_E_INVALID;
    }
    const int64_t Nn = d.n_nodes, Nt = d.n_tets, Ntri = d.n_triangles;
    m.n_nodes = Nn;
    m.n_tets = Nt;
    m.n_tris = Ntri;
    m.node_xyz.assign(d.node_xyz, d.node_xyz + 3 * Nn);
    m.tet_nodes.assign(d.tet_nodes, d.tet_nodes + 4 * Nt);
    m.rec.assign(Nt, TetRec{});
    m.vol.assign(Nt, 0.0);

    // 1. Orientation, barycentric maps, volumes.
    int bad = -1;
    for (int64_t t = 0; t < Nt; ++t) {
        int32_t *tn = &m.tet_nodes[4 * t];
        for (int k = 0; k < 4; ++k)
            if (tn[k] < 0 || tn[k] >= Nn) bad = int(t);
        if (bad >= 0) break;
        const double *p[4];
        for (int k = 0; k < 4; ++k) p[k] = &m.node_xyz[3 * int64_t(tn[k])];
        double M[9];
        double det = tet_map(p[0], p[1], p[2], p[3], M);
        if (det < 0.0) {
            std::swap(tn[2], tn[3]);
            std::swap(p[2], p[3]);
            det = tet_map(p[0], p[1], p[2], p[3], M);
        }
        if (!(det > 0.0)) {
            bad = int(t);
            break;
        }
        TetRec &r = m.rec[t];
        std::memcpy(r.M, M, sizeof(M));
        r.x0[0] = p[0][0];
        r.x0[1] = p[0][1];
        r.x0[2] = p[0][2];
        m.vol[t] = det / 6.0;
    }
    if (bad >= 0) {
        es << "mesh: tet " << bad << " has a bad node index or zero volume";
        err = es.str();
        return SPG_E_BAD_MESH;
    }

    // 2. Face matching: bucket faces by their smallest node id.
    std::vector<int64_t> bstart(Nn + 1, 0);
    for (int64_t t = 0; t < Nt; ++t)
        for (int f = 0; f < 4; ++f) {
            int32_t v[3];
            face_nodes(&m.tet_nodes[4 * t], f, v);
            sort3(v);
            bstart[v[0] + 1]++;
        }
    for (int64_t i = 0; i < Nn; ++i) bstart[i + 1] += bstart[i];
    std::vector<FaceRef> faces(4 * Nt);
    {
        std::vector<int64_t> cur(bstart.begin(), bstart.end() - 1);
        for (int64_t t = 0; t < Nt; ++t)
            for (int f = 0; f < 4; ++f) {
                int32_t v[3];
                face_nodes(&m.tet_nodes[4 * t], f, v);
                sort3(v);
                faces[cur[v[0]]++] = FaceRef{v[1], v[2], int32_t(4 * t + f)};
            }
    }
    m.nbr.assign(4 * Nt, -1);
    m.ftri.assign(4 * Nt, -1);
    int64_t nonmanifold = 0, boundary = 0;
#pragma omp parallel for schedule(dynamic, 4096) reduction(+ : nonmanifold, boundary)
    for (int64_t a = 0; a < Nn; ++a) {
        FaceRef *f0 = faces.data() + bstart[a], *f1 = faces.data() + bstart[a + 1];
        std::sort(f0, f1, [](const FaceRef &x, const FaceRef &y) {
            return x.b != y.b ? x.b < y.b : (x.c != y.c ? x.c < y.c : x.tf < y.tf);
        });
        for (FaceRef *f = f0; f < f1;) {
            FaceRef *g = f + 1;
            while (g < f1 && g->b == f->b && g->c == f->c) ++g;
            const int64_t k = g - f;
            if (k == 2) {
                m.nbr[f[0].tf] = f[1].tf;
                m.nbr[f[1].tf] = f[0].tf;
            } else if (k == 1) {
                boundary++;
            } else {
                nonmanifold++;
            }
            f = g;
        }
    }
    if (nonmanifold) {
        es << "mesh: " << nonmanifold << " faces are shared by more than two tets";
        err = es.str();
        return SPG_E_BAD_MESH;
    }
    m.n_boundary_faces = boundary;

    // 3. Surface triangles onto tet faces (all faces carrying the triangle).
    for (int64_t k = 0; k < Ntri; ++k) {
        int32_t v[3] = {d.tri_nodes[3 * k], d.tri_nodes[3 * k + 1], d.tri_nodes[3 * k + 2]};
        if (v[0] < 0 || v[0] >= Nn || v[1] < 0 || v[1] >= Nn || v[2] < 0 || v[2] >= Nn) {
            es << "mesh: triangle " << k << " has a bad node index";
            err = es.str();
            return SPG_E_BAD_MESH;
        }
        sort3(v);
        const FaceRef *f0 = faces.data() + bstart[v[0]], *f1 = faces.data() + bstart[v[0] + 1];
        int hits = 0;
        for (const FaceRef *f = f0; f < f1; ++f)
            if (f->b == v[1] && f->c == v[2]) {
                m.ftri[f->tf] = int32_t(k);
                hits++;
            }
        if (!hits) {
            es << "mesh: triangle " << k << " is not a face of any tet";
            err = es.str();
            return SPG_E_BAD_MESH;
        }
    }
    faces.clear();
    faces.shrink_to_fit();

    // 4. Node -> tet incidence, dual volumes.
    std::vector<int64_t> nstart(Nn + 1, 0);
    for (int64_t i = 0; i < 4 * Nt; ++i) nstart[m.tet_nodes[i] + 1]++;
    for (int64_t i = 0; i < Nn; ++i) nstart[i + 1] += nstart[i];
    std::vector<int32_t> ntet(4 * Nt);  // tet*4 + local vertex
    {
        std::vector<int64_t> cur(nstart.begin(), nstart.end() - 1);
        for (int64_t i = 0; i < 4 * Nt; ++i) ntet[cur[m.tet_nodes[i]]++] = int32_t(i);
    }
    m.dual_vol.assign(Nn, 0.0);
    for (int64_t n = 0; n < Nn; ++n) {
        double s = 0.0;
        for (int64_t k = nstart[n]; k < nstart[n + 1]; ++k) s += m.vol[ntet[k] >> 2];
        m.dual_vol[n] = 0.25 * s;
    }

    // 5. Dirichlet nodes.
    m.is_dir.assign(Nn, 0);
    m.dir_value.assign(Nn, 0.0);
    m.n_dirichlet = 0;
    for (int64_t k = 0; k < d.n_dirichlet; ++k) {
        const int32_t n = d.dirichlet_nodes[k];
        if (n < 0 || n >= Nn) {
            es << "mesh: Dirichlet node " << n << " out of range";
            err = es.str();
            return SPG_E_INVALID;
        }
        if (!m.is_dir[n]) m.n_dirichlet++;
        m.is_dir[n] = 1;
        m.dir_value[n] = d.dirichlet_values[k];
    }

    // 6. CSR stiffness. Row i holds the nodes of its incident tets, sorted.
    m.row_ptr.assign(Nn + 1, 0);
    std::vector<int32_t> rowlen(Nn, 0);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < Nn; ++i) {
        if (m.is_dir[i]) {
            rowlen[i] = 1;
            continue;
        }
        std::vector<int32_t> cols;
        cols.reserve(32);
        for (int64_t k = nstart[i]; k < nstart[i + 1]; ++k) {
            const int32_t *tn = &m.tet_nodes[4 * int64_t(ntet[k] >> 2)];
            for (int v = 0; v < 4; ++v)
                if (!m.is_dir[tn[v]]) cols.push_back(tn[v]);
        }
        std::sort(cols.begin(), cols.end());
        rowlen[i] = int32_t(std::unique(cols.begin(), cols.end()) - cols.begin());
    }
    for (int64_t i = 0; i < Nn; ++i) m.row_ptr[i + 1] = m.row_ptr[i] + rowlen[i];
    const int64_t nnz = m.row_ptr[Nn];
    if (nnz >= (int64_t(1) << 31)) {
        err = "mesh: stiffness has more than 2^31 non-zeros";
        return SPG_E_INVALID;
    }
    m.col.assign(nnz, 0);
    m.val.assign(nnz, 0.0);
    m.diag.assign(Nn, 1.0);
    m.lift.assign(Nn, 0.0);
    std::vector<std::vector<std::pair<int32_t, double>>> elim(Nn);  // free row -> (Dirichlet col, K)
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < Nn; ++i) {
        int32_t *c0 = &m.col[m.row_ptr[i]];
        double *v0 = &m.val[m.row_ptr[i]];
        const int32_t len = rowlen[i];
        if (m.is_dir[i]) {
            c0[0] = int32_t(i);
            v0[0] = 1.0;
            m.diag[i] = 1.0;
            continue;
        }
        {
            std::vector<int32_t> cols;
            cols.reserve(32);
            for (int64_t k = nstart[i]; k < nstart[i + 1]; ++k) {
                const int32_t *tn = &m.tet_nodes[4 * int64_t(ntet[k] >> 2)];
                for (int v = 0; v < 4; ++v)
                    if (!m.is_dir[tn[v]]) cols.push_back(tn[v]);
            }
            std::sort(cols.begin(), cols.end());
            cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
            std::copy(cols.begin(), cols.end(), c0);
        }
        double lift = 0.0;
        for (int64_t k = nstart[i]; k < nstart[i + 1]; ++k) {
            const int64_t t = ntet[k] >> 2;
            const int a = ntet[k] & 3;
            const TetRec &r = m.rec[t];
            double G[4][3];
            for (int c = 0; c < 3; ++c) {
                G[1][c] = r.M[c];
                G[2][c] = r.M[3 + c];
                G[3][c] = r.M[6 + c];
                G[0][c] = -(G[1][c] + G[2][c] + G[3][c]);
            }
            const int32_t *tn = &m.tet_nodes[4 * t];
            for (int b = 0; b < 4; ++b) {
                const double kab = m.vol[t] * (G[a][0] * G[b][0] + G[a][1] * G[b][1] + G[a][2] * G[b][2]);
                const int32_t j = tn[b];
                if (m.is_dir[j]) {
                    lift += kab * m.dir_value[j];
                    auto &e = elim[i];
                    auto it = std::find_if(e.begin(), e.end(), [j](const std::pair<int32_t, double> &x) {
                        return x.first == j;
                    });
                    if (it == e.end())
                        e.emplace_back(j, kab);
                    else
                        it->second += kab;
                } else {
                    const int32_t *pos = std::lower_bound(c0, c0 + len, j);
                    v0[pos - c0] += kab;
                }
            }
        }
        m.lift[i] = lift;
        for (int32_t k = 0; k < len; ++k)
            if (c0[k] == i) m.diag[i] = v0[k];
    }

    // Eliminated couplings K_fd (free row f, Dirichlet column d): the lifting
    // vector for new Dirichlet values and the adjoint of the lifting.
    m.elim_row.clear();
    m.elim_col.clear();
    m.elim_val.clear();
    for (int64_t i = 0; i < Nn; ++i) {
        std::sort(elim[i].begin(), elim[i].end());
        for (const auto &e : elim[i]) {
            m.elim_row.push_back(int32_t(i));
            m.elim_col.push_back(e.first);
            m.elim_val.push_back(e.second);
        }
    }

    // 7. Expanded global bounding box of the surface triangles
    //    (SurfaceMesh::isParticleWithinModelingSpace); the node box when there
    //    are no triangles.
    double lo[3] = {HUGE_VAL, HUGE_VAL, HUGE_VAL}, hi[3] = {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL};
    auto grow = [&](int32_t n) {
        for (int c = 0; c < 3; ++c) {
            lo[c] = std::min(lo[c], m.node_xyz[3 * int64_t(n) + c]);
            hi[c] = std::max(hi[c], m.node_xyz[3 * int64_t(n) + c]);
        }
    };
    if (Ntri > 0)
        for (int64_t k = 0; k < 3 * Ntri; ++k) grow(d.tri_nodes[k]);
    else
        for (int64_t n = 0; n < Nn; ++n) grow(int32_t(n));
    for (int c = 0; c < 3; ++c) {
        const double centre = (lo[c] + hi[c]) / 2.0;
        const double half = ((hi[c] - lo[c]) / 2.0) * bbox_expansion;
        m.bbox_lo[c] = centre - half;
        m.bbox_hi[c] = centre + half;
    }

    // 8. Voxel seed grid over the node box: about one voxel per six tets.
    double nlo[3] = {HUGE_VAL, HUGE_VAL, HUGE_VAL}, nhi[3] = {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL};
    for (int64_t n = 0; n < Nn; ++n)
        for (int c = 0; c < 3; ++c) {
            nlo[c] = std::min(nlo[c], m.node_xyz[3 * n + c]);
            nhi[c] = std::max(nhi[c], m.node_xyz[3 * n + c]);
        }
    double total_vol = 0.0;
    for (int64_t t = 0; t < Nt; ++t) total_vol += m.vol[t];
    const double edge = std::cbrt(6.0 * total_vol / double(Nt));
    int64_t nvox = 1;
    for (int c = 0; c < 3; ++c) {
        const double ext = std::max(nhi[c] - nlo[c], edge);
        m.vox_dims[c] = int32_t(std::max(1.0, std::min(1024.0, std::ceil(ext / edge))));
        m.vox_origin[c] = nlo[c];
        m.vox_inv[c] = double(m.vox_dims[c]) / ext;
        nvox *= m.vox_dims[c];
    }
    m.vox_seed.assign(nvox, -1);
    for (int64_t t = 0; t < Nt; ++t) {
        double cen[3] = {0, 0, 0};
        for (int k = 0; k < 4; ++k)
            for (int c = 0; c < 3; ++c) cen[c] += m.node_xyz[3 * int64_t(m.tet_nodes[4 * t + k]) + c];
        int32_t iv[3];
        for (int c = 0; c < 3; ++c) {
            const double u = (0.25 * cen[c] - m.vox_origin[c]) * m.vox_inv[c];
            iv[c] = int32_t(std::min<double>(m.vox_dims[c] - 1, std::max(0.0, std::floor(u))));
        }
        const int64_t v = iv[0] + int64_t(m.vox_dims[0]) * (iv[1] + int64_t(m.vox_dims[1]) * iv[2]);
        if (m.vox_seed[v] < 0 || m.vox_seed[v] > t) m.vox_seed[v] = int32_t(t);
    }
    // Fill empty voxels from face neighbours until none is empty.
    for (bool changed = true; changed;) {
        changed = false;
        std::vector<int32_t> next = m.vox_seed;
        const int32_t dx = m.vox_dims[0], dy = m.vox_dims[1], dz = m.vox_dims[2];
        for (int32_t k = 0; k < dz; ++k)
            for (int32_t j = 0; j < dy; ++j)
                for (int32_t i = 0; i < dx; ++i) {
                    const int64_t v = i + int64_t(dx) * (j + int64_t(dy) * k);
                    if (m.vox_seed[v] >= 0) continue;
                    const int64_t cand[6] = {i > 0 ? v - 1 : -1,
                                             i + 1 < dx ? v + 1 : -1,
                                             j > 0 ? v - dx : -1,
                                             j + 1 < dy ? v + dx : -1,
                                             k > 0 ? v - int64_t(dx) * dy : -1,
                                             k + 1 < dz ? v + int64_t(dx) * dy : -1};
                    for (int64_t cv : cand)
                        if (cv >= 0 && m.vox_seed[cv] >= 0) {
                            next[v] = m.vox_seed[cv];
                            changed = true;
                            break;
                        }
                }
        m.vox_seed.swap(next);
    }
    return SPG_OK;
}

}  // namespace spg
