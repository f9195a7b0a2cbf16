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
// positive definite for CG (the reference only replaces rows). The element
// maps and volumes, the node -> tet incidence and the stiffness assembly run
// on the GPU (kernels_fem.cu); the face matching, the surface triangles, the
// bounding box and the point-location grid stay here.
//
// Compiled with -ffp-contract=off, like the oracle: the geometry feeds the
// FP64 walk, which must agree bit for bit with the CPU oracle.
#include <algorithm>
#include <array>
#include <chrono>
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

namespace {
double ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}
}  // namespace

int prepare_mesh(const spg_mesh_desc &d, double bbox_expansion, HostMesh &m, std::string &err) {
    const auto t_start = std::chrono::steady_clock::now();
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

    // 1. Orientation, barycentric maps, volumes (on the GPU, kernels_fem.cu).
    for (int64_t k = 0; k < 4 * Nt; ++k)
        if (m.tet_nodes[k] < 0 || m.tet_nodes[k] >= Nn) {
            es << "mesh: tet " << k / 4 << " has a bad node index or zero volume";
            err = es.str();
            return SPG_E_BAD_MESH;
        }
    {
        int64_t bad = -1;
        const auto t0 = std::chrono::steady_clock::now();
        const int rc = fem_elements_gpu(m, err, bad);
        m.prep_ms[0] = ms_since(t0);
        if (rc) return rc;
        if (bad >= 0) {
            es << "mesh: tet " << bad << " has a bad node index or zero volume";
            err = es.str();
            return SPG_E_BAD_MESH;
        }
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

    // 4. Node -> tet incidence and dual volumes; CSR stiffness with the
    //    Dirichlet rows as identity rows, the lifting and the eliminated
    //    couplings (on the GPU, kernels_fem.cu).
    {
        const auto t0 = std::chrono::steady_clock::now();
        const int rc = fem_stiffness_gpu(m, err);
        m.prep_ms[1] = ms_since(t0);
        if (rc) return rc;
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
    m.prep_ms[2] = ms_since(t_start);
    return SPG_OK;
}

}  // namespace spg
