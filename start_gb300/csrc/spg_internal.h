// Internal declarations shared by the host-side preparation (mesh_prep.cpp),
// the C ABI (capi.cpp) and the device kernels (*.cu) of libstart_gpu.so.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/start_gpu.h"

namespace spg {

// Particle id and state share one 32-bit word: bits 0..27 id, 28 settled, 29 lost.
constexpr uint32_t kIdMask = 0x0FFFFFFFu;
constexpr uint32_t kSettled = 1u << 28;
constexpr uint32_t kLost = 1u << 29;
constexpr uint32_t kDead = kSettled | kLost;
constexpr int64_t kMaxParticles = int64_t(kIdMask) + 1;

// Per-tet record read by the push and the walk: barycentric map and E.
// lambda_{1..3}(p) = M * (p - x0), lambda_0 = 1 - lambda_1 - lambda_2 - lambda_3.
// Row r of M is grad(lambda_{r+1}); E = -sum_i phi_i grad(lambda_i).
struct alignas(128) TetRec {
    double M[9];
    double x0[3];
    double E[3];
    double pad;
};
static_assert(sizeof(TetRec) == 128, "TetRec must be one 128-byte line");

// Neighbour across local face f (opposite local vertex f): nb*4 + g where g is
// the same face's local index in nb; -1 on the mesh boundary.
// Surface triangle on local face f: triangle id, or -1.

// Host copy of everything mesh_prep derives from spg_mesh_desc.
struct HostMesh {
    int64_t n_nodes = 0, n_tets = 0, n_tris = 0, n_boundary_faces = 0, n_dirichlet = 0;
    std::vector<double> node_xyz;   // 3*Nn
    std::vector<int32_t> tet_nodes; // 4*Nt, positively oriented
    std::vector<TetRec> rec;        // Nt (E = 0)
    std::vector<int32_t> nbr;       // 4*Nt packed
    std::vector<int32_t> ftri;      // 4*Nt
    std::vector<double> vol;        // Nt
    std::vector<double> dual_vol;   // Nn: 1/4 sum of incident tet volumes
    // Stiffness with Dirichlet rows replaced by identity and Dirichlet columns
    // moved to the right-hand side (symmetric elimination).
    std::vector<int32_t> row_ptr, col;
    std::vector<double> val, diag;
    std::vector<uint8_t> is_dir;
    std::vector<double> dir_value;  // Nn (0 on free nodes)
    std::vector<double> lift;       // Nn: sum_{j in D} K_ij g_j on free rows, 0 on D rows
    // Reference global bounding box test (SurfaceMesh.cpp:104-134), expanded.
    double bbox_lo[3] = {0, 0, 0}, bbox_hi[3] = {0, 0, 0};
    // Voxel seed grid for point location.
    double vox_origin[3] = {0, 0, 0}, vox_inv[3] = {1, 1, 1};
    int32_t vox_dims[3] = {1, 1, 1};
    std::vector<int32_t> vox_seed;
};

// Returns SPG_OK or SPG_E_BAD_MESH / SPG_E_INVALID with a message in err.
int prepare_mesh(const spg_mesh_desc &desc, double bbox_expansion, HostMesh &out, std::string &err);

// ---------------------------------------------------------------- device side

struct DevParticles {
    double *x, *y, *z, *vx, *vy, *vz;
    int32_t *tet;
    uint32_t *idf;
};

// Cumulative device counters (one struct in device memory).
struct DevCounters {
    unsigned long long processed;   // alive particles seen by the step kernel
    unsigned long long tet_runs;    // runs of equal tet ids in particle order
    unsigned long long collisions;
    unsigned long long crossings;
    unsigned long long settled;
    unsigned long long lost;
    unsigned long long capped;      // walks stopped at max_crossings
    unsigned long long pad;
};

struct StepConst {
    double dt, q_over_m, charge, mass;
    double vmin;
    double lo[3], hi[3];
    int32_t model;
    int32_t max_cross;
    // collisions
    double gas_n, mass_cp, mass_ct, sigma_hs;
    double vhs_c1;     // dref^2 / Gamma(5/2 - omega)
    double two_kT;     // 2 * kT_ref
    double mr;         // reduced mass
    double expo;       // omega - 1/2
    double inv_alpha;  // 1 / alpha
    uint32_t seed_lo, seed_hi;
    int64_t step;
};

struct MeshDev {
    const TetRec *rec;
    const int4 *nbr;
    const int4 *ftri;
    const int4 *tet_nodes;
    const double *node_xyz;
    int64_t n_tets, n_nodes;
};

// Kernel launchers (kernels_particles.cu).
void launch_step64(const DevParticles &p, int64_t n, const MeshDev &m, const StepConst &c,
                   unsigned int *tri_count, DevCounters *ctr, cudaStream_t s);
void launch_deposit64(const DevParticles &p, int64_t n, const MeshDev &m, double wq, double *node_q,
                      cudaStream_t s);
void launch_efield64(const MeshDev &m, TetRec *rec, const double *phi, cudaStream_t s);
void launch_locate(const double *pos, int64_t n, const MeshDev &m, const int32_t *vox_seed,
                   const double *vox_origin_inv, const int32_t *vox_dims, int max_cross,
                   int32_t *tet_out, cudaStream_t s);
void launch_zero_efield(TetRec *rec, int64_t n_tets, cudaStream_t s);
void launch_count_lost(const int32_t *tet, int64_t n, unsigned long long *out, cudaStream_t s);
void launch_init_particles(const double *pos, const double *vel, const int32_t *tet, int64_t n,
                           DevParticles p, cudaStream_t s);
void launch_gather_by_id(const DevParticles &p, int64_t n, double *pos, double *vel, int32_t *tet,
                         uint32_t *flags, cudaStream_t s);
// Re-sort: histogram, exclusive scan, scatter. Writes the number of alive
// particles to *n_alive_dev. scratch must hold sort_scratch_words(n_tets) ints, 8-byte aligned.
int64_t sort_scratch_words(int64_t n_tets);
// Number of tets holding at least one alive particle at the last re-sort.
unsigned long long *sort_occupied_counter(int32_t *scratch);
void launch_resort(const DevParticles &src, DevParticles dst, int64_t n, int64_t n_tets, int32_t *scratch,
                   int64_t *n_alive_dev, cudaStream_t s);

// PCG (kernels_pcg.cu).
// tol2 is set to rtol^2 by the host and scaled by ||b||^2 in the setup kernel.
struct PcgScalars {
    double rz, pq, alpha, beta, rr, bb, tol2;
    int32_t iters, converged, max_iter, pad;
    unsigned int ticket;
    unsigned int pad2;
};
struct PcgDev {
    int64_t n;
    const int32_t *row_ptr, *col;
    const double *val, *inv_diag;
    double *x, *r, *z, *p, *p2, *q;
    double *partials;  // 3 doubles per block
    PcgScalars *sc;
    int blocks;
};
int pcg_blocks(int64_t n);
// b = node_q/eps0 - lift on free rows, g on Dirichlet rows
void launch_pcg_rhs(const double *node_q, double inv_eps0, const double *lift, const uint8_t *is_dir,
                    const double *dir_value, double *b, int64_t n, cudaStream_t s);
void launch_pcg_setup(const PcgDev &d, const double *b, cudaStream_t s);
void launch_pcg_iteration(PcgDev &d, cudaStream_t s);
void launch_node_rho(const double *node_q, const double *dual_vol, double *rho, int64_t n, cudaStream_t s);

}  // namespace spg
