// Internal declarations shared by the host-side preparation (mesh_prep.cpp),
// the C ABI (capi.cpp) and the device kernels (*.cu) of libstart_gpu.so.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/start_gpu.h"
#include "screen.h"

namespace spg {

// Particle id and state share one 32-bit word: bits 0..27 id, 28 settled, 29 lost.
constexpr uint32_t kIdMask = 0x0FFFFFFFu;
constexpr uint32_t kSettled = 1u << 28;
constexpr uint32_t kLost = 1u << 29;
constexpr uint32_t kDead = kSettled | kLost;
constexpr int64_t kMaxParticles = int64_t(kIdMask) + 1;

// Per-tet record read by the push and the walk: barycentric map and the
// push increment. lambda_{1..3}(p) = M * (p - x0), lambda_0 = 1 - sum.
// Row r of M is grad(lambda_{r+1}). H = ((q E / m) dt) / 2 per component is
// the Boris half-step velocity increment for B = 0, computed once per tet
// after each solve with the same operations the per-particle formula uses;
// ezero = 1 when E is exactly zero (the reference then skips the push).
struct alignas(128) TetRec {
    double M[9];
    double x0[3];
    double H[3];
    uint32_t ezero;
    uint32_t pad;
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
    std::vector<int32_t> elim_row, elim_col;  // eliminated couplings K_fd, f free, d Dirichlet
    std::vector<double> elim_val;
    // Reference global bounding box test (SurfaceMesh.cpp:104-134), expanded.
    double bbox_lo[3] = {0, 0, 0}, bbox_hi[3] = {0, 0, 0};
    // Voxel seed grid for point location.
    double vox_origin[3] = {0, 0, 0}, vox_inv[3] = {1, 1, 1};
    int32_t vox_dims[3] = {1, 1, 1};
    std::vector<int32_t> vox_seed;
    // Set-up wall times (ms): GPU element maps, GPU incidence + stiffness,
    // the whole preparation.
    double prep_ms[3] = {0, 0, 0};
};

// Order-preserving map of a double to int64: a < b <=> key(a) < key(b) for
// non-NaN values, with -0 and +0 mapped to the same key.
inline long long order_key_host(double x) {
    long long b;
    static_assert(sizeof(b) == sizeof(x), "");
    __builtin_memcpy(&b, &x, sizeof(b));
    if (b == (long long)0x8000000000000000ULL) b = 0;
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}

// Message returned by spg_last_error(NULL) on the calling thread.
void set_thread_error(const std::string &msg);

// Returns SPG_OK or SPG_E_BAD_MESH / SPG_E_INVALID with a message in err.
int prepare_mesh(const spg_mesh_desc &desc, double bbox_expansion, HostMesh &out, std::string &err);
// FEM set-up on the current device (kernels_fem.cu): element maps, volumes
// and orientation (bad_tet: lowest bad tet or -1); incidence, dual volumes
// and the CSR stiffness with its Dirichlet elimination.
int fem_elements_gpu(HostMesh &m, std::string &err, int64_t &bad_tet);
int fem_stiffness_gpu(HostMesh &m, std::string &err);

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
    // order-preserving integer keys of lo/hi (exact bbox test without FP64 compares)
    long long lo_key[3], hi_key[3];
    // bit pattern of 2*vmin: |v_k| above it means |v| >= vmin for certain
    long long two_vmin_bits;
    // FP32 screen of the collision probability: P ~= kp * (v^2)^pexp
    float kp_f, pexp_f;
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
    // FP32 copies for the mixed form (rounded once on the host, so no thread
    // spends FP64-pipe conversions on them)
    float lo_f[3], hi_f[3], vmin_f, dt_f, mass_cp_f, mass_ct_f, inv_alpha_f;
    // v^2 at or below which kp (v^2)^pexp < q (1 - 2e-4), q = 1/256: a step
    // that is no collision candidate needs no probability there (-1: none)
    float v2_cand_f;
};

struct MeshDev {
    const TetRec *rec;
    const TetScreen *screen;  // hi_float of rec's M and x0 (inside screen of the FP64 step)
    const int4 *nbr;
    const int4 *ftri;
    const int4 *tet_nodes;
    const double *node_xyz;
    int64_t n_tets, n_nodes;
};

// A particle whose move needs the exact tet walk: its index and start point.
struct WalkItem {
    int32_t i;
    int32_t pad;
    double x0, y0, z0;
};

// Landing record of a settled particle (adjoint of the landing point): step
// of the crossing, exit face of the final tet, hit fraction s of the move
// segment; step = -1 while the particle has not landed.
struct LandRec {
    int32_t step;
    int32_t face;
    int32_t tet;  // tet whose face was crossed
    int32_t pad;
    double s;
};

// Per-step record of a checkpoint window (adjoint recompute): tet (-1 when
// the particle is dead) and velocity at the start of each step, [k][i].
struct AdjHist {
    int32_t *tet;
    double *vx, *vy, *vz;
};

// kernels_adjoint.cu
void launch_record(const DevParticles &p, int64_t n, const AdjHist &h, int k, cudaStream_t s);
void launch_objective(const DevParticles &p, int64_t n, const LandRec *land, const double *target, double sigma,
                      double *gr, double *sums, cudaStream_t s);
// G (nullable): per-tet gradient of the recovered field (launch_field_gradient);
// with it the position adjoint also carries the push's dependence on the
// particle's position.
void launch_backward(const DevParticles &p, int64_t n, const AdjHist &h, int k0, int k1, const TetRec *rec,
                     const LandRec *land, const double *gr, double gscale, double *ax, double *av, double *gE,
                     const StepConst &c, cudaStream_t s, const double *G = nullptr);
// G[9 t + 3 d + c] = dE_d/dx_c of the continuous field whose nodal values are
// the volume averages of the incident tets' E (E: 3 per tet); En (3 nn) and
// Wn (nn) are scratch.
void launch_field_gradient(const int4 *tet_nodes, const TetRec *rec, const double *E, int64_t nt, int64_t nn,
                           double *En, double *Wn, double *G, cudaStream_t s);
void launch_gE_to_nodes(const int4 *tet_nodes, const TetRec *rec, const double *gE, int64_t nt, double *lam,
                        cudaStream_t s);
void launch_adj_rhs(const double *lam, const uint8_t *is_dir, double *b, double *x, int64_t nn, cudaStream_t s);
void launch_dirichlet_grad(const double *lam, const uint8_t *is_dir, const int32_t *er, const int32_t *ec,
                           const double *ev, int64_t ne, const double *mu, double *out, int64_t nn, cudaStream_t s);
void launch_lift(const int64_t *erp, const int32_t *ec, const double *ev, const double *g, double *lift, int64_t nn,
                 cudaStream_t s);
void launch_set_dirichlet(const uint8_t *is_dir, const double *g, double *dir_value, double *phi, int64_t nn,
                          cudaStream_t s);
void launch_gather_adj(const DevParticles &p, int64_t n, const double *ax, const double *av, double *dx, double *dv,
                       cudaStream_t s);

struct FieldArgs;
// List of the tets that hold particles at a deposit (the tets whose field the
// next solve of a run must compute): gen_of[t] == gen marks a listed tet.
struct OccList {
    int32_t *list;  // nullptr: no list is kept
    unsigned int *n;
    uint32_t *gen_of;
    uint32_t gen;
};
// Kernel launchers (kernels_particles.cu).
// Step kernel plus the exact walk of the queued particles (wq holds up to n
// items); land (nullable) receives the landing records; a walk that brings a
// particle into a tet with an older field computes that tet's field (f).
void launch_step64(const DevParticles &p, int64_t n, const MeshDev &m, const StepConst &c,
                   unsigned int *tri_count, WalkItem *wq, unsigned int *wq_n, DevCounters *ctr, const FieldArgs &f,
                   cudaStream_t s, LandRec *land = nullptr);
// Fixed-point P1 deposit: node_fix[n] += round(lambda_n * 2^k) per alive
// particle (lambda_0 takes the remainder so each particle adds exactly 2^k).
// occ (list nullable) collects the tets holding particles.
void launch_deposit64(const DevParticles &p, int64_t n, const MeshDev &m, int k, unsigned long long *node_fix,
                      const OccList &occ, cudaStream_t s);
// node_q = node_fix * scale
void launch_fix_to_charge(const unsigned long long *node_fix, double scale, double *node_q, int64_t n,
                          cudaStream_t s);
void launch_locate(const double *pos, int64_t n, const MeshDev &m, const int32_t *vox_seed,
                   const double *vox_origin_inv, const int32_t *vox_dims, int max_cross,
                   int32_t *tet_out, cudaStream_t s);
// E = 0 and H = 0 in every tet, stamped with f.epoch (both forms' records).
void launch_zero_field(const FieldArgs &f, int64_t n_tets, cudaStream_t s);
void launch_count_lost(const int32_t *tet, int64_t n, unsigned long long *out, cudaStream_t s);
// Installs n particles at slots [id_base, id_base + n) with ids id_base + i.
void launch_init_particles(const double *pos, const double *vel, const int32_t *tet, int64_t n,
                           DevParticles p, cudaStream_t s, int64_t id_base = 0);
// Slot of each particle id; the gathers below write in id order through it
// (slot: n words of scratch).
void launch_slot_of_id(const uint32_t *idf, int64_t n, int32_t *slot, cudaStream_t s);
void launch_gather_by_id(const DevParticles &p, int64_t n, int32_t *slot, double *pos, double *vel,
                         int32_t *tet, uint32_t *flags, cudaStream_t s);
// Re-sort: histogram, exclusive scan, scatter. Writes the number of alive
// particles to *n_alive_dev. scratch must hold sort_scratch_words(n_tets) ints, 8-byte aligned.
int64_t sort_scratch_words(int64_t n_tets);
// Number of tets holding at least one alive particle at the last re-sort.
unsigned long long *sort_occupied_counter(int32_t *scratch);
void launch_resort(const DevParticles &src, DevParticles dst, int64_t n, int64_t n_tets, int32_t *scratch,
                   int64_t *n_alive_dev, cudaStream_t s);
// Histogram + exclusive scan of the sort keys; sort_offsets(scratch) then
// holds the first slot of every key (tets, then n_tets for dead particles).
void launch_sort_prepare(const int32_t *tet, const uint32_t *idf, int64_t n, int64_t n_tets, int32_t *scratch,
                         int64_t *n_alive_dev, cudaStream_t s);
int32_t *sort_offsets(int32_t *scratch);

// ---------------------------------------------------------- mixed precision
// Per-tet record of the mixed form (64 B): FP32 barycentric map about the
// centroid, lambda_{1..3} = 1/4 + M (x - c); FP32 push increment; FP32
// centroid (modelling-box test only); flags: kRecEzero (E = 0, no push) and
// kRecInterior (the tet lies inside the modelling box with a margin far above
// the FP32 rounding of centroid + local position, so a particle inside it
// passes the box test: the test is skipped).
constexpr uint32_t kRecEzero = 1u;
constexpr uint32_t kRecInterior = 2u;
struct alignas(64) TetRec32 {
    float M[9];
    float H[3];
    float cen[3];
    uint32_t ezero;  // kRecEzero | kRecInterior
};
static_assert(sizeof(TetRec32) == 64, "TetRec32 must be 64 bytes");

// Per-tet field (E and the push increment H with its E-null flag) of the
// current potential. A full update computes every tet. After a solve inside
// spg_run only the tets holding particles are computed (launch_refresh*),
// and a walk that brings a particle into a tet whose field belongs to an
// older potential (stamp[t] != epoch) computes that tet there: the first
// lane to swap the stamp computes, the values are those of the full update,
// and the next step (a later launch) reads them.
struct FieldArgs {
    const int4 *tet_nodes;
    const double *phi;
    double *efield;    // 3 per tet
    TetRec *rec;       // FP64 map (read); H and ezero written in the FP64 form
    TetRec32 *rec32;   // mixed form: FP32 H and ezero written; nullptr in the FP64 form
    uint32_t *stamp;   // per tet: epoch of its field
    uint32_t epoch;
    double charge, mass, inv_mass, dt;
    double c32;        // mixed form: q dt / (2 m)
};
void launch_field64_full(const FieldArgs &f, int64_t n_tets, cudaStream_t s);
void launch_field32_full(const FieldArgs &f, int64_t n_tets, cudaStream_t s);
void launch_refresh64(const DevParticles &p, int64_t n, const FieldArgs &f, cudaStream_t s);
// The field of the tets a deposit listed (list_n entries on the device).
void launch_field64_list(const FieldArgs &f, const int32_t *list, const unsigned int *list_n, cudaStream_t s);
void launch_field32_list(const FieldArgs &f, const int32_t *list, const unsigned int *list_n, cudaStream_t s);

// 32 B per particle: position relative to the owning tet's centroid.
struct DevParticles32 {
    float *x, *y, *z, *vx, *vy, *vz;
    int32_t *tet;
    uint32_t *idf;
};

// Upload and location in one kernel from device-readable caller arrays of n
// particles (ids 0..n-1): the FP64 form's state into p (cen == nullptr) or
// the mixed form's into q (cen: FP64 centroids); lost (zeroed by the caller)
// receives the count of particles outside the mesh.
void launch_upload(const double *pos, const double *vel, int64_t n, const MeshDev &m, const int32_t *vox_seed,
                   const double *oi, const int32_t *dims, int max_cross, const DevParticles &p,
                   const DevParticles32 &q, const double *cen, unsigned long long *lost, cudaStream_t s);

struct MeshDev32 {
    const TetRec32 *rec;
    const TetRec *rec64;  // FP64 map for near-zero barycentric tests
    const double *cen;    // FP64 centroids, 3 per tet
    const float *cen_lo;  // 3 per tet: cen - float(cen), for re-basing in FP32 pairs
    const int4 *nbr, *ftri, *tet_nodes;
    int64_t n_tets;
};

// kernels_mixed.cu
void launch_step32(const DevParticles32 &p, int64_t n, const MeshDev32 &m, const StepConst &c,
                   unsigned int *tri_count, void *wq, unsigned int *wq_n, DevCounters *ctr, const FieldArgs &f,
                   cudaStream_t s, LandRec *land = nullptr);
void launch_refresh32(const DevParticles32 &p, int64_t n, const FieldArgs &f, cudaStream_t s);
// Steps c.step .. c.step + L - 1 of the mixed form with nothing between them
// (no solve, re-sort, track record or landing record), bit-identical to L
// launch_step32 calls: wq holds n items of 20 B, rq n int2, q_n 2 L + 1
// counters. Returns the number of kernels launched.
int launch_segment32(const DevParticles32 &p, int64_t n, const MeshDev32 &m, const StepConst &c, int L,
                     unsigned int *tri_count, void *wq, int2 *rq, unsigned int *q_n, DevCounters *ctr,
                     const FieldArgs &f, cudaStream_t s);

// adjoint of the FP32 form (kernels_mixed.cu)
void launch_record32(const DevParticles32 &p, int64_t n, const AdjHist &h, int k, cudaStream_t s);
void launch_objective32(const DevParticles32 &p, int64_t n, const MeshDev32 &m, const LandRec *land,
                        const double *target, double sigma, double *gr, double *sums, cudaStream_t s);
void launch_backward32(const DevParticles32 &p, int64_t n, const MeshDev32 &m, const AdjHist &h, int k0, int k1,
                       const LandRec *land, const double *gr, double gscale, double *ax, double *av, double *gE,
                       const StepConst &c, cudaStream_t s, const double *G = nullptr);
void launch_gather_adj32(const DevParticles32 &p, int64_t n, const double *ax, const double *av, double *dx,
                         double *dv, cudaStream_t s);
void launch_deposit32(const DevParticles32 &p, int64_t n, const MeshDev32 &m, int k, unsigned long long *node_fix,
                      const OccList &occ, cudaStream_t s);
void launch_to_local(const double *pos, const double *vel, const int32_t *tet, const double *cen, int64_t n,
                     DevParticles32 p, cudaStream_t s, int64_t id_base = 0);
void launch_gather32(const DevParticles32 &p, int64_t n, int32_t *slot, const double *cen, double *pos, double *vel,
                     int32_t *tet, uint32_t *flags, cudaStream_t s);
void launch_resort32(const DevParticles32 &src, DevParticles32 dst, int64_t n, int64_t n_tets, int32_t *scratch,
                     int64_t *n_alive_dev, cudaStream_t s);
size_t walk_item32_bytes();

// PCG (kernels_pcg.cu).
// tol2 is set to rtol^2 by the host and scaled by ||b||^2 in the setup kernel.
struct PcgScalars {
    double rz, pq, alpha, beta, rr, bb, tol2;
    int32_t iters, converged, max_iter, flags;  // flags: bad-diagonal mark of the allocation-free solve
    unsigned int ticket;
    unsigned int pad2;
};
// Grid of each PCG kernel: SMs x resident blocks per SM (occupancy of that
// kernel), capped by the rows; every kernel loops over rows grid-stride.
struct PcgGrid {
    int setup = 1, spmv = 1, update = 1, pupdate = 1;
};
struct PcgDev {
    int64_t n;
    const int32_t *row_ptr, *col;
    const double *val, *inv_diag;
    const int64_t *slice_ptr;  // SELL-32: n_slices + 1 offsets
    const int32_t *scol;
    const double *sval;
    double *x, *r, *z, *p, *p2, *q;
    double *partials;  // 3 doubles per block
    PcgScalars *sc;
    PcgGrid grid;
};
struct PcgDev32 {
    int64_t n;
    const int64_t *slice_ptr;
    const int32_t *scol;
    const float *sval;
    const float *inv_diag;
    float *e, *r, *z, *p, *q;
    double *partials;  // 3 doubles per block (separate from the FP64 solver's)
    PcgScalars *sc;
    PcgGrid grid;
};
// Upper bound of any PCG grid (partials sizing) and the per-kernel grids.
int pcg_blocks(int64_t n);
PcgGrid pcg_grid64(int64_t n);
PcgGrid pcg_grid32(int64_t n);
// Mixed-precision solve pieces (kernels_pcg.cu).
void launch_refine_setup(const PcgDev &d, const PcgDev32 &f, const double *b, cudaStream_t s);
void launch_pcg32_iteration(PcgDev32 &f, cudaStream_t s);
void launch_refine_apply(double *x, const float *e, int64_t n, cudaStream_t s);
// Initial guess of a run solve: the history shifts (prev2 <- prev <- phi) and
// phi becomes the polynomial extrapolation of order `order` (0: unchanged,
// 1: 2 phi - prev, 2: 3 phi - 3 prev + prev2).
void launch_extrapolate(double *phi, double *prev, double *prev2, int64_t n, int order, cudaStream_t s);
// CSR -> SELL-32 (slices of 32 rows, column-major, zero padding).
void build_sell32(int64_t n, const int32_t *row_ptr, const int32_t *col, const double *val,
                  std::vector<int64_t> &slice_ptr, std::vector<int32_t> &scol, std::vector<double> &sval);
void build_sell32(int64_t n, const int64_t *row_ptr, const int32_t *col, const double *val,
                  std::vector<int64_t> &slice_ptr, std::vector<int32_t> &scol, std::vector<double> &sval);

// ---------------------------------------------------------------- sources
// A particle source on the device (kernels_sources.cu): the spg_source with
// its frame (e1, e2, normal) and energy constants formed on the host.
struct SourceConst {
    int32_t shape, directions, energy;
    double centre[3], e1[3], e2[3], nrm[3];
    double radius, xlim[2], ylim[2], z;
    double one_minus_cos;  // 1 - cos(half_angle)
    double speed_mono;     // sqrt(2 E / m) of the monoenergetic source
    double binding_j, s_max, mass;  // Thompson: U [J], Emax/(Emax+U); particle mass
    double displacement;
    uint32_t seed_lo, seed_hi;
    int64_t id_base;       // Philox counter of particle i is id_base + i (its particle id)
    double theta0, phi0;   // SPG_DIR_FAN: polar and azimuthal angle of the normal
    double expansion;      // SPG_DIR_FAN: polar spread
    double fan_shift[3];   // SPG_DIR_FAN point source: its one displacement vector
    // SPG_SRC_CELLS: per cell centre xyz, theta0, phi0 and its displacement
    // vector (8 doubles), and the first particle index of each cell
    // (n_cells + 1 prefix offsets)
    int32_t n_cells;
    const double *cells;
    const int64_t *cell_first;
};
void launch_generate(const SourceConst &c, int64_t n, double *pos, double *vel, cudaStream_t s);

// ---------------------------------------------------------------- tracks
// Trajectory sampling of a fixed set of particle ids (kernels_track.cu).
void launch_track_map(const int64_t *ids, int k, int32_t *track_of_id, cudaStream_t s);
// track_of_id holds table_n ids; particles with larger ids (injected later) are not tracked.
void launch_track_find(const uint32_t *idf, int64_t n, const int32_t *track_of_id, int64_t table_n, int32_t *slot,
                       cudaStream_t s);
void launch_track_record64(const DevParticles &p, const int32_t *slot, int k, int cap, int32_t *count, double *xyz,
                           cudaStream_t s);
void launch_track_record32(const DevParticles32 &p, const double *cen, const int32_t *slot, int k, int cap,
                           int32_t *count, double *xyz, cudaStream_t s);
void launch_track_current64(const DevParticles &p, const int32_t *slot, int k, double *xyz, uint32_t *flags,
                            cudaStream_t s);
void launch_track_current32(const DevParticles32 &p, const double *cen, const int32_t *slot, int k, double *xyz,
                            uint32_t *flags, cudaStream_t s);

// ---------------------------------------------------------------- AMG
// Smoothed-aggregation hierarchy (amg_setup.cpp) and its GPU V-cycle
// (kernels_amg.cu), the preconditioner of SPG_PRECOND_AMG.
struct AmgCsr {
    int64_t n = 0, m = 0;
    std::vector<int64_t> rp;
    std::vector<int32_t> ci;
    std::vector<double> v;
};
struct AmgLevelHost {
    AmgCsr A, P, R;  // P, R empty on the coarsest level
    std::vector<double> dinv;
    double lam = 0.0;  // upper bound of the spectrum of D^-1 A
};
struct AmgHost {
    std::vector<AmgLevelHost> levels;  // levels[0].A is the solver's matrix
    int64_t nc = 0;                    // rows of the coarsest level
    std::vector<double> coarse_inv;    // its dense inverse, row-major
};
struct AmgOptions {
    double theta = 0.08;   // strength of connection
    double filter = 0.0;   // coarse operators: couplings below filter * sqrt(|a_ii a_jj|) move to the diagonal
    int64_t coarse_rows = 1500;
    int smooth_levels = 99;  // levels whose prolongator is smoothed (the rest use plain aggregation)
};
int amg_setup(int64_t n, const int32_t *row_ptr, const int32_t *col, const double *val, AmgHost &out,
              std::string &err, const AmgOptions &opt = AmgOptions{});

constexpr int kAmgMaxLevels = 12;
// A V-cycle operator on the device: SELL-32 with one thread per row (g = 0,
// short rows), or CSR with g lanes per row (g = 4, 8, 16 or 32; the long rows
// of coarse operators and of the restriction). T: double (FP64 form) or
// float (the inner solve of the mixed form).
template <class T>
struct DevSellT {
    int64_t n = 0;
    int g = 0;
    const int64_t *slice_ptr = nullptr;  // SELL: slice offsets; CSR: row offsets
    const int32_t *scol = nullptr;
    const T *sval = nullptr;
};
// One level of the V-cycle on the device. Jacobi-Chebyshev smoothing on
// D^-1 A: degree 2 over [lam/30, lam], or degree 1 (damped Jacobi,
// 1/theta = 1.6/lam) over [lam/4, lam]; theta = (hi+lo)/2, delta = (hi-lo)/2.
template <class T>
struct AmgLevelDevT {
    int64_t n = 0;
    int degree = 2;
    DevSellT<T> A, P, R;  // P: n x n_next, R: n_next x n
    const T *dinv = nullptr;
    T *x[2] = {nullptr, nullptr};  // iterate ping-pong
    T *b = nullptr, *r = nullptr, *d = nullptr;
    double inv_theta = 0.0, cheb_a = 0.0, cheb_b = 0.0;  // step 2: d = a d + b D^-1 r
};
template <class T>
struct AmgDevT {
    int levels = 0;  // including the coarsest (dense) level
    AmgLevelDevT<T> lev[kAmgMaxLevels];
    int64_t nc = 0;
    const T *coarse_inv = nullptr;
};
using DevSell = DevSellT<double>;
using AmgLevelDev = AmgLevelDevT<double>;
using AmgDev = AmgDevT<double>;
using AmgDev32 = AmgDevT<float>;
// z = M^-1 r by one V-cycle (level 0 vectors: b = r, x[0] = z, x[1] scratch);
// every kernel returns at once when sc->converged is set (sc->converged == 3,
// the inner cap of the mixed form, also stops it).
void launch_amg_vcycle(const AmgDev &a, const double *r, double *z, const PcgScalars *sc, cudaStream_t s);
void launch_amg_vcycle(const AmgDev32 &a, const float *r, float *z, const PcgScalars *sc, cudaStream_t s);
// The FP32 V-cycle without level 0's last Jacobi step, which the mixed PCG
// then runs fused with r.z (possible when level 0 is degree 1 in SELL-32).
bool amg_last_step_fusable(const AmgDev32 &a);
void launch_amg_vcycle_but_last(const AmgDev32 &a, const float *r, float *z, const PcgScalars *sc, cudaStream_t s);
// PCG with the V-cycle: setup and one iteration (spmv_dot, update, V-cycle,
// r.z and beta, p update).
void launch_pcg_setup_amg(const PcgDev &d, const AmgDev &a, const double *b, cudaStream_t s);
void launch_pcg_iteration_amg(PcgDev &d, const AmgDev &a, cudaStream_t s);
// The mixed form's PCG: FP64 SpMV, vectors and sums with the FP32 V-cycle as
// the preconditioner (r32 = float(r) in, z32 out).
void launch_pcg_setup_amg_mixed(const PcgDev &d, const AmgDev32 &a, const double *b, float *r32, float *z32,
                                cudaStream_t s);
void launch_pcg_iteration_amg_mixed(PcgDev &d, const AmgDev32 &a, float *r32, float *z32, cudaStream_t s);
// The same PCG rotated for the while-graph, so that the loop stops right
// after the update that converges: the setup only forms r (and r32); an
// iteration is the V-cycle, r.z and beta (p = z in the first), the p update,
// q = A p and the update of x and r with the stop test. Needs a level 0 that
// fuses its last step with r.z (pcg_rotated_ok).
bool pcg_rotated_ok(const AmgDev32 &a);
void launch_pcg_residual_amg_mixed(const PcgDev &d, const double *b, float *r32, cudaStream_t s);
void launch_pcg_rotated_iteration_amg_mixed(PcgDev &d, const AmgDev32 &a, float *r32, float *z32, cudaStream_t s);
// Last node of a PCG while-graph body: the condition stays 1 until sc->converged.
void launch_pcg_continue(cudaGraphConditionalHandle cond, const PcgScalars *sc, cudaStream_t s);
// b = node_q/eps0 - lift on free rows, g on Dirichlet rows
void launch_pcg_rhs(const double *node_q, double inv_eps0, const double *lift, const uint8_t *is_dir,
                    const double *dir_value, double *b, int64_t n, cudaStream_t s);
void launch_pcg_setup(const PcgDev &d, const double *b, cudaStream_t s);
void launch_pcg_iteration(PcgDev &d, cudaStream_t s);
void launch_node_rho(const double *node_q, const double *dual_vol, double *rho, int64_t n, cudaStream_t s);
// node_q = rho * dual_vol (a density given by the caller)
void launch_node_q_from_rho(const double *rho, const double *dual_vol, double *node_q, int64_t n, cudaStream_t s);

}  // namespace spg
