// C ABI of libstart_gpu.so (declared in include/start_gpu.h).
//
// One handle = one mesh, one particle population and one CUDA stream. The
// time loop mirrors ModelingMainDriver::startModeling
// (src/ModelingMainDriver.cpp:132-220): per step, gather (deposit) and solve
// when due, then process; plus the periodic re-sort that has no reference
// counterpart (it only changes memory order).
#include <algorithm>
#include <chrono>
#include <random>
#include <cmath>
#include <cstring>
#include <memory>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "spg_internal.h"

using namespace spg;

namespace {

thread_local std::string g_create_error;

constexpr int kEventPool = 8192;
constexpr int kPcgChunk = 8;
// Solver scalars held back per run (pinned host records, read when the run
// ends or the records are full).
constexpr int kSolveRecs = 64;
// Order of the extrapolated initial guess of the AMG run solves (1: linear
// in the last two potentials, 2: quadratic in the last three).
constexpr int kExtrapOrder = 2;
// Mixed form: FP32 inner PCG to 1e-4 of the outer residual (about what an
// FP32 matrix can resolve for kappa ~ 1e4), at most this many inner
// iterations per correction and outer refinement steps per solve.
constexpr double kInnerRtol = 1e-4;
constexpr int kInnerMaxIter = 2000;
constexpr int kOuterMax = 40;

struct EventSeries {
    std::vector<cudaEvent_t> start, stop;
    int used = 0;
    double ms = 0.0;
    int64_t launches = 0;
};

}  // namespace

namespace spg {
void set_thread_error(const std::string &msg) { g_create_error = msg; }
}  // namespace spg

struct spg_handle {
    spg_params prm{};
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;

    // mesh
    int64_t n_nodes = 0, n_tets = 0, n_tris = 0, n_boundary_faces = 0, nnz = 0, n_dirichlet = 0;
    double bbox_lo[3], bbox_hi[3];
    double vox_oi[6];
    int32_t vox_dims[3];
    TetRec *rec = nullptr;
    TetScreen *screen = nullptr;  // hi_float of rec's M and x0, the FP64 step's inside screen
    int4 *nbr = nullptr, *ftri = nullptr, *tet_nodes = nullptr;
    double *node_xyz = nullptr;
    int32_t *row_ptr = nullptr, *col = nullptr;
    int64_t *slice_ptr = nullptr;
    int32_t *scol = nullptr;
    double *sval = nullptr;
    int64_t sell_entries = 0;
    int64_t nnz_kept = 0;  // stiffness entries in the device format (exact zeros off the diagonal dropped)
    double *val = nullptr, *inv_diag = nullptr, *dir_value = nullptr, *lift = nullptr, *dual_vol = nullptr;
    uint8_t *is_dir = nullptr;
    int32_t *vox_seed = nullptr;
    std::vector<double> phi_init;  // Dirichlet values, 0 elsewhere
    // With AMG: the electrode field (the potential of the Dirichlet values
    // with no charge), the starting potential of every new particle set.
    double *phi_vac = nullptr;
    bool vac_valid = false;

    // fields
    double *node_q = nullptr, *rho = nullptr, *phi = nullptr, *b = nullptr, *r = nullptr, *z = nullptr,
           *p = nullptr, *q = nullptr, *partials = nullptr;
    // phi of the two previous solves of spg_run and the number of run solves
    // they have seen (the AMG solves start from an extrapolation of the last
    // kExtrapOrder + 1 solutions once there are that many)
    double *phi_prev = nullptr, *phi_prev2 = nullptr;
    int32_t phi_hist = 0;
    double *efield = nullptr;                 // 3 per tet
    uint32_t *tet_stamp = nullptr;            // per tet: epoch of its field (E, H)
    uint32_t field_epoch = 0;                 // epoch of the current potential's field
    bool field_full = true;                   // every tet's field is of field_epoch
    bool in_run = false;                      // inside spg_run: solves refresh the occupied tets only
    // Inside spg_run a while-graph solve does not wait for the host: its
    // scalars go to a pinned record, read when the run ends.
    bool defer_solves = false;
    PcgScalars *solve_rec = nullptr;          // pinned, kSolveRecs records
    uint8_t solve_kind[kSolveRecs] = {};      // 0: do_solve64, 1: do_solve_mixed_amg
    int n_solve_rec = 0;
    bool deferred_capped = false;             // a drained record had hit max_iter
    bool occ_fresh = false;                   // no particle has moved since the deposit listed the tets
    int64_t resorted_at = -1;                 // step of the last periodic re-sort
    int32_t *occ_list = nullptr;              // tets holding particles at the last deposit
    unsigned int *occ_n = nullptr;
    uint32_t *occ_gen = nullptr;              // per tet: generation of the list that holds it
    uint32_t occ_epoch = 0;                   // field epoch the list was made for
    uint32_t occ_count = 0;                   // deposits so far (the list generation)
    unsigned long long *node_fix = nullptr;   // fixed-point deposit accumulators
    int fix_bits = 40;                        // deposit quantum 2^-fix_bits of one particle's charge
    PcgScalars *sc = nullptr;
    int pcg_blocks = 1;
    PcgGrid grid64, grid32;
    // PCG iterations are replayed as a CUDA graph of kPcgChunk iterations
    // (3 kernels each); converged solves turn the remaining kernels into no-ops.
    cudaGraphExec_t pcg_graph = nullptr;
    // AMG preconditioner (prm.preconditioner == SPG_PRECOND_AMG)
    // trajectory sampling (spg_track_particles)
    int32_t track_k = 0, track_cap = 0;
    int64_t *track_ids = nullptr;
    int32_t *track_of_id = nullptr, *track_slot = nullptr, *track_count = nullptr;
    int64_t track_table_n = 0;  // ids the id -> track table covers (particles injected later are not tracked)
    double *track_xyz = nullptr, *track_cur = nullptr;
    uint32_t *track_flags = nullptr;
    bool amg = false, amg32 = false;
    AmgDev amgd{};
    AmgDev32 amgd32{};
    std::vector<void *> amg_alloc;
    std::vector<int64_t> amg_rows, amg_nnz;
    int amg_launches = 0;         // kernel launches of one V-cycle
    double amg_bytes = 0.0;       // algorithmic bytes of one V-cycle

    // mixed form (precision == SPG_MIXED)
    bool mixed = false;
    double pbytes = 56.0;  // bytes per particle in HBM
    TetRec32 *rec32 = nullptr;
    double *cen = nullptr;  // 3 per tet
    float *cen_lo = nullptr;  // 3 per tet: cen - float(cen)
    DevParticles32 Q[2]{};
    float *sval32 = nullptr, *inv_diag32 = nullptr;
    float *e32 = nullptr, *r32 = nullptr, *z32 = nullptr, *p32 = nullptr, *q32 = nullptr;
    double *partials32 = nullptr;
    PcgScalars *sc32 = nullptr;
    cudaGraphExec_t pcg32_graph = nullptr;
    // FP64 PCG with the FP32 V-cycle as one graph: a while node repeats an
    // iteration until the device scalars say converged (no host round trip)
    cudaGraphExec_t pcg_while = nullptr, pcg64_while = nullptr;  // FP32 V-cycle; FP64 V-cycle or Jacobi
    bool pcg_while_failed = false, pcg64_while_failed = false;

    // particles
    DevParticles P[2]{};
    int cur = 0;
    int64_t cap = 0, np = 0, n_active = 0, init_lost = 0;
    unsigned int *tri_count = nullptr;
    DevCounters *ctr = nullptr;
    WalkItem *walkq = nullptr;       // capacity cap (particles)
    unsigned int *walkq_n = nullptr;
    // segmented steps of the mixed form: at most seg_max steps per segment
    // (1: one launch per step); resumed-particle list and per-round counters
    int seg_max = 32;
    int2 *seg_rq = nullptr;
    int64_t seg_rq_cap = 0;
    unsigned int *seg_qn = nullptr;
    int seg_qn_cap = 0;
    int64_t *n_alive_dev = nullptr;
    int32_t *sort_scratch = nullptr;
    // Staging for particles that cross the host boundary or come from a
    // source (set/get/generate/inject): 60 B per particle + 16, kept between
    // calls so that a copy or an injection allocates nothing once grown.
    unsigned char *io = nullptr;
    size_t io_bytes = 0;
    // direct host access: the device reads pageable memory through the host
    // page tables (address translation over the C2C link)
    bool ats = false;
    int32_t *id_slot = nullptr;  // slot of each id for direct downloads
    int64_t id_slot_cap = 0;
    unsigned long long *io_counter = nullptr;
    double setup_ms[6] = {0, 0, 0, 0, 0, 0};  // spg_setup_times
    int64_t occupied = 0;
    bool have_particles = false;
    bool charge_valid = false;

    // loop state
    int64_t step = 0;
    int32_t cg_iters_last = 0, cg_solves = 0;
    int64_t cg_iters_total = 0;
    double cg_relres_last = 0.0;

    // profiling
    bool prof = false;
    EventSeries ev_step, ev_dep, ev_pcg, ev_ef, ev_sort;
    double step_bytes = 0, dep_bytes = 0, pcg_bytes = 0, sort_bytes = 0;
    int64_t pcg_iters_prof = 0;
    unsigned long long processed_at_reset = 0;
    int64_t launches = 0;  // kernels launched (all phases), reset with the profile

    // Dirichlet data for spg_set_dirichlet and the adjoint of the lifting:
    // eliminated couplings K_fd as CSR over free rows.
    int64_t n_elim = 0;
    int64_t *elim_rp = nullptr;
    int32_t *elim_row = nullptr, *elim_col = nullptr;
    double *elim_val = nullptr;
    uint8_t *is_dir_host = nullptr;

    // gradient state (spg_grad_forward / spg_grad_backward)
    std::vector<DevParticles> ckpt;   // particle state at steps 0, ce, 2 ce, ...
    int32_t grad_steps = 0, grad_every = 0;
    int64_t grad_step0 = 0;
    LandRec *land = nullptr;
    double *gr = nullptr, *adj_x = nullptr, *adj_v = nullptr, *gE = nullptr, *lam = nullptr, *mu = nullptr,
           *dJdg = nullptr, *sums = nullptr;
    AdjHist hist{};
    unsigned int *tri_scratch = nullptr;
    DevCounters *ctr_scratch = nullptr;
    std::vector<DevParticles32> ckpt32;  // the same for the FP32 form
    int64_t ckpt_cap = 0, land_cap = 0, hist_cap = 0;  // particles (x window steps for hist) allocated
    double grad_inv_n = 0.0;                            // 1 / landed count of the last forward
    bool grad_ready = false;
    // spg_grad_field_gradient: per-tet gradient of the recovered field and its scratch
    bool grad_fg = false;
    double *grad_G = nullptr, *grad_En = nullptr;
};

namespace {

int fail(spg_handle *h, int code, const std::string &msg) {
    if (h)
        h->err = msg;
    else
        g_create_error = msg;
    return code;
}

#define CK(call)                                                                                     \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess)                                                                       \
            return fail(h, e_ == cudaErrorMemoryAllocation ? SPG_E_OOM : SPG_E_CUDA,                 \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                         \
    } while (0)

template <class T>
cudaError_t dalloc(T **ptr, size_t count) {
    return cudaMalloc(reinterpret_cast<void **>(ptr), sizeof(T) * std::max<size_t>(count, 1));
}

template <class T>
cudaError_t upload(T **ptr, const std::vector<T> &v, cudaStream_t s) {
    cudaError_t e = dalloc(ptr, v.size());
    if (e != cudaSuccess) return e;
    if (v.empty()) return cudaSuccess;
    e = cudaMemcpyAsync(*ptr, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(s);
}

// Staging of n particles: pos [3n], vel [3n] doubles, tet [n], flags [n], slot [n]
// 32-bit words and one 64-bit counter.
struct IoStage {
    double *pos, *vel;
    int32_t *tet;
    uint32_t *flags;
    int32_t *slot;  // slot of each id (spg_get_particles)
    unsigned long long *counter;
};

// Device address through which kernels may read the caller's array p: pinned
// (registered) host memory, managed memory, or, where the device walks the
// host page tables, pageable memory. nullptr: copy through the staging buffer.
const void *device_readable(const spg_handle *h, const void *p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeHost && a.devicePointer) return a.devicePointer;
    if (a.type == cudaMemoryTypeManaged) return p;
    if (a.type == cudaMemoryTypeUnregistered && h->ats) return p;
    return nullptr;
}

// Device address through which kernels may write the caller's array p: pinned
// or managed memory only (writes to untouched pageable pages would fault them
// in one by one).
void *device_writable(const void *p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeHost && a.devicePointer) return a.devicePointer;
    if (a.type == cudaMemoryTypeManaged) return const_cast<void *>(p);
    return nullptr;
}

int io_stage(spg_handle *h, int64_t n, IoStage &st) {
    const size_t need = 60 * size_t(n) + 16;
    if (need > h->io_bytes) {
        cudaFree(h->io);
        h->io = nullptr;
        h->io_bytes = 0;
        CK(cudaMalloc(reinterpret_cast<void **>(&h->io), need));
        h->io_bytes = need;
    }
    st.counter = reinterpret_cast<unsigned long long *>(h->io);
    st.pos = reinterpret_cast<double *>(h->io + 16);
    st.vel = st.pos + 3 * n;
    st.tet = reinterpret_cast<int32_t *>(st.vel + 3 * n);
    st.flags = reinterpret_cast<uint32_t *>(st.tet + n);
    st.slot = reinterpret_cast<int32_t *>(st.flags + n);
    return SPG_OK;
}

void free_particles(spg_handle *h) {
    for (auto &P : h->P) {
        cudaFree(P.x);
        cudaFree(P.y);
        cudaFree(P.z);
        cudaFree(P.vx);
        cudaFree(P.vy);
        cudaFree(P.vz);
        cudaFree(P.tet);
        cudaFree(P.idf);
        P = DevParticles{};
    }
    for (auto &Q : h->Q) {
        cudaFree(Q.x);
        cudaFree(Q.y);
        cudaFree(Q.z);
        cudaFree(Q.vx);
        cudaFree(Q.vy);
        cudaFree(Q.vz);
        cudaFree(Q.tet);
        cudaFree(Q.idf);
        Q = DevParticles32{};
    }
    cudaFree(h->walkq);
    h->walkq = nullptr;
    h->cap = 0;
}

MeshDev32 mesh_dev32(const spg_handle *h) {
    MeshDev32 m;
    m.rec = h->rec32;
    m.rec64 = h->rec;
    m.cen = h->cen;
    m.cen_lo = h->cen_lo;
    m.nbr = h->nbr;
    m.ftri = h->ftri;
    m.tet_nodes = h->tet_nodes;
    m.n_tets = h->n_tets;
    return m;
}

PcgDev32 pcg_dev32(spg_handle *h) {
    PcgDev32 f;
    f.n = h->n_nodes;
    f.slice_ptr = h->slice_ptr;
    f.scol = h->scol;
    f.sval = h->sval32;
    f.inv_diag = h->inv_diag32;
    f.e = h->e32;
    f.r = h->r32;
    f.z = h->z32;
    f.p = h->p32;
    f.q = h->q32;
    f.partials = h->partials32;
    f.sc = h->sc32;
    f.grid = h->grid32;
    return f;
}

// Uploads an AMG hierarchy in value type T: every operator as SELL-32 or
// CSR with g lanes per row (level 0 uses the solver's matrix, sval0), D^-1,
// the Chebyshev constants and the work vectors of each level, the dense
// inverse of the coarsest. Returns the V-cycle's launches and bytes.
template <class T>
int upload_amg(spg_handle *h, const AmgHost &ah, const T *sval0, AmgDevT<T> &a) {
    const int L = int(ah.levels.size());
    if (L > kAmgMaxLevels) return fail(h, SPG_E_INVALID, "amg: too many levels");
    cudaStream_t s = h->stream;
    int rc;
    auto keep = [&](void *p) { h->amg_alloc.push_back(p); };
    auto conv = [](const std::vector<double> &v) { return std::vector<T>(v.begin(), v.end()); };
    // short rows: SELL-32, one thread per row; long rows: CSR, g lanes per row
    auto up_mat = [&](const AmgCsr &M, DevSellT<T> &D) -> int {
        std::vector<int64_t> sp;
        std::vector<int32_t> sc;
        std::vector<double> sv;
        const double avg = M.n ? double(M.ci.size()) / double(M.n) : 0.0;
        D.g = 0;
        // FP64: one thread per row up to 48 entries per row, then lanes with
        // about 12 entries each (each FP64 shuffle add of a lane group costs a
        // full warp instruction at the FP64 rate); FP32: lanes from 12
        // entries per row, about 4 entries per lane
        if (sizeof(T) == 8 ? avg > 48.0 : avg > 12.0) {
            const double per_lane = sizeof(T) == 8 ? 12.0 : 4.0;
            D.g = 4;
            while (D.g < 32 && per_lane * D.g < avg) D.g *= 2;
            sp = M.rp;
            sc = M.ci;
            sv = M.v;
        } else {
            build_sell32(M.n, M.rp.data(), M.ci.data(), M.v.data(), sp, sc, sv);
        }
        int64_t *dsp = nullptr;
        int32_t *dsc = nullptr;
        T *dsv = nullptr;
        CK(upload(&dsp, sp, s));
        keep(dsp);
        CK(upload(&dsc, sc, s));
        keep(dsc);
        CK(upload(&dsv, conv(sv), s));
        keep(dsv);
        D.n = M.n;
        D.slice_ptr = dsp;
        D.scol = dsc;
        D.sval = dsv;
        return SPG_OK;
    };
    auto vec = [&](T **p, int64_t n) -> int {
        CK(dalloc(p, std::max<int64_t>(n, 1)));
        keep(*p);
        return SPG_OK;
    };
    a.levels = L;
    h->amg_launches = 0;
    h->amg_bytes = 0.0;
    h->amg_rows.clear();
    h->amg_nnz.clear();
    const double wv = double(sizeof(T)), wm = 4.0 + double(sizeof(T));  // bytes per vector entry / per nonzero
    for (int l = 0; l < L; ++l) {
        const AmgLevelHost &H = ah.levels[l];
        AmgLevelDevT<T> &D = a.lev[l];
        D.n = H.A.n;
        h->amg_rows.push_back(H.A.n);
        h->amg_nnz.push_back(int64_t(H.A.ci.size()));
        if (l == 0) {
            D.A.n = H.A.n;
            D.A.slice_ptr = h->slice_ptr;
            D.A.scol = h->scol;
            D.A.sval = sval0;
        } else if ((rc = up_mat(H.A, D.A))) {
            return rc;
        }
        if (l < L - 1) {
            if ((rc = up_mat(H.P, D.P)) || (rc = up_mat(H.R, D.R))) return rc;
            T *dv = nullptr;
            CK(upload(&dv, conv(H.dinv), s));
            keep(dv);
            D.dinv = dv;
            if ((rc = vec(&D.x[1], D.n)) || (rc = vec(&D.r, D.n)) || (rc = vec(&D.d, D.n))) return rc;
            // degree 1 (damped Jacobi over [lam/4, lam]) on every level: on the
            // 1.03e6-node cube it needs 21 cold iterations against 22 with degree 2
            // on level 0, at 22 % fewer matrix entries per V-cycle
            D.degree = 1;
            const double hi = H.lam, lo = D.degree == 2 ? H.lam / 30.0 : H.lam / 4.0;
            const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo);
            const double sigma = theta / delta, rho0 = 1.0 / sigma, rho1 = 1.0 / (2.0 * sigma - rho0);
            D.inv_theta = 1.0 / theta;
            D.cheb_a = rho1 * rho0;
            D.cheb_b = 2.0 * rho1 / delta;
            const double nnzA = double(H.A.ci.size()), n = double(D.n);
            const double nnzP = double(H.P.ci.size()), nc = double(H.P.m);
            if (D.degree == 2) {
                // cheb0 4 n; three Chebyshev steps (nnz + 6 n each); residual
                // (nnz + 3 n); restriction (nnz(P) + n + nc); prolongation
                // (nnz(P) + 2 n + nc); vector words
                h->amg_bytes += wv * (4.0 * n + 18.0 * n + 3.0 * n + 3.0 * n + 2.0 * nc) + wm * (4.0 * nnzA + 2.0 * nnzP);
                h->amg_launches += 7;
            } else if (sizeof(T) == 4) {
                // residual from x0 = D^-1 b / theta (nnz + 3 n); restriction (nnz(P) +
                // n + nc); prolongation onto x0 (nnz(P) + 3 n + nc); Jacobi step (nnz + 4 n)
                h->amg_bytes += wv * (3.0 * n + n + 3.0 * n + 4.0 * n + 2.0 * nc) + wm * (2.0 * nnzA + 2.0 * nnzP);
                h->amg_launches += 4;
            } else {
                // x0 = D^-1 b / theta (3 n); residual (nnz + 3 n); restriction (nnz(P) +
                // n + nc); prolongation (nnz(P) + 2 n + nc); Jacobi step (nnz + 4 n)
                h->amg_bytes += wv * (3.0 * n + 3.0 * n + n + 2.0 * n + 4.0 * n + 2.0 * nc) +
                                wm * (2.0 * nnzA + 2.0 * nnzP);
                h->amg_launches += 5;
            }
        }
        if (l > 0 && (rc = vec(&D.b, D.n))) return rc;
        if (l > 0 && (rc = vec(&D.x[0], D.n))) return rc;
    }
    a.nc = ah.nc;
    T *inv = nullptr;
    CK(upload(&inv, conv(ah.coarse_inv), s));
    keep(inv);
    a.coarse_inv = inv;
    h->amg_launches += 1;
    h->amg_bytes += wv * double(ah.nc) * double(ah.nc + 2);
    return SPG_OK;
}

// Builds the smoothed-aggregation hierarchy of the stiffness matrix on the
// host and uploads it for the FP64 V-cycle (plain form) or the FP32 V-cycle
// (inner solve of the mixed form).
int setup_amg(spg_handle *h, const HostMesh &hm) {
    AmgHost ah;
    std::string err;
    int rc = amg_setup(hm.n_nodes, hm.row_ptr.data(), hm.col.data(), hm.val.data(), ah, err);
    if (rc) return fail(h, rc, err);
    if (h->mixed || h->prm.preconditioner == SPG_PRECOND_AMG_F32) {
        if ((rc = upload_amg<float>(h, ah, h->sval32, h->amgd32))) return rc;
        h->amg32 = true;
        if (!h->mixed) {  // the FP32 V-cycle's input and output vectors (the mixed form allocates them anyway)
            CK(dalloc(&h->r32, hm.n_nodes));
            CK(dalloc(&h->z32, hm.n_nodes));
        }
    } else {
        if ((rc = upload_amg<double>(h, ah, h->sval, h->amgd))) return rc;
        h->amg = true;
    }
    return SPG_OK;
}

// PCG setup and one iteration with the handle's preconditioner.
void pcg_setup_any(spg_handle *h, const PcgDev &d, const double *b) {
    if (h->amg32)
        launch_pcg_setup_amg_mixed(d, h->amgd32, b, h->r32, h->z32, h->stream);
    else if (h->amg)
        launch_pcg_setup_amg(d, h->amgd, b, h->stream);
    else
        launch_pcg_setup(d, b, h->stream);
}
void pcg_iteration_any(spg_handle *h, PcgDev &d) {
    if (h->amg32)
        launch_pcg_iteration_amg_mixed(d, h->amgd32, h->r32, h->z32, h->stream);
    else if (h->amg)
        launch_pcg_iteration_amg(d, h->amgd, h->stream);
    else
        launch_pcg_iteration(d, h->stream);
}
// (with the FP32 V-cycle the last level-0 step and r.z are one kernel where level 0 allows it)
int pcg_rz_fused(const spg_handle *h) { return h->amg32 && amg_last_step_fusable(h->amgd32) ? 1 : 0; }
int pcg_iter_launches(const spg_handle *h) {
    return (h->amg || h->amg32) ? 4 + h->amg_launches - pcg_rz_fused(h) : 3;
}
int pcg_chunk(const spg_handle *h) { return (h->amg || h->amg32) ? 2 : kPcgChunk; }

// Allocates both particle buffers (and the walk queue) for n particles.
int alloc_particles(spg_handle *h, int64_t n) {
    if (n <= h->cap) return SPG_OK;
    free_particles(h);
    if (h->mixed) {
        for (auto &Q : h->Q) {
            CK(dalloc(&Q.x, n));
            CK(dalloc(&Q.y, n));
            CK(dalloc(&Q.z, n));
            CK(dalloc(&Q.vx, n));
            CK(dalloc(&Q.vy, n));
            CK(dalloc(&Q.vz, n));
            CK(dalloc(&Q.tet, n));
            CK(dalloc(&Q.idf, n));
        }
    } else {
        for (auto &P : h->P) {
            CK(dalloc(&P.x, n));
            CK(dalloc(&P.y, n));
            CK(dalloc(&P.z, n));
            CK(dalloc(&P.vx, n));
            CK(dalloc(&P.vy, n));
            CK(dalloc(&P.vz, n));
            CK(dalloc(&P.tet, n));
            CK(dalloc(&P.idf, n));
        }
    }
    CK(dalloc(&h->walkq, n));
    h->cap = n;
    return SPG_OK;
}

// Capacity for `need` particles keeping the current ones: new buffers (both
// of the re-sort pair), the current set copied into buffer 0.
int grow_particles(spg_handle *h, int64_t need) {
    if (need <= h->cap) return SPG_OK;
    const int64_t cap = std::max<int64_t>(need, h->cap + h->cap / 2);
    const int64_t np = h->np;
    cudaStream_t s = h->stream;
    if (h->mixed) {
        DevParticles32 N[2];
        for (auto &Q : N) {
            CK(dalloc(&Q.x, cap));
            CK(dalloc(&Q.y, cap));
            CK(dalloc(&Q.z, cap));
            CK(dalloc(&Q.vx, cap));
            CK(dalloc(&Q.vy, cap));
            CK(dalloc(&Q.vz, cap));
            CK(dalloc(&Q.tet, cap));
            CK(dalloc(&Q.idf, cap));
        }
        const DevParticles32 &O = h->Q[h->cur];
        void *dst[8] = {N[0].x, N[0].y, N[0].z, N[0].vx, N[0].vy, N[0].vz, N[0].tet, N[0].idf};
        const void *src[8] = {O.x, O.y, O.z, O.vx, O.vy, O.vz, O.tet, O.idf};
        for (int k = 0; k < 8; ++k)
            if (np) CK(cudaMemcpyAsync(dst[k], src[k], 4 * size_t(np), cudaMemcpyDeviceToDevice, s));
        CK(cudaStreamSynchronize(s));
        free_particles(h);
        h->Q[0] = N[0];
        h->Q[1] = N[1];
    } else {
        DevParticles N[2];
        for (auto &P : N) {
            CK(dalloc(&P.x, cap));
            CK(dalloc(&P.y, cap));
            CK(dalloc(&P.z, cap));
            CK(dalloc(&P.vx, cap));
            CK(dalloc(&P.vy, cap));
            CK(dalloc(&P.vz, cap));
            CK(dalloc(&P.tet, cap));
            CK(dalloc(&P.idf, cap));
        }
        const DevParticles &O = h->P[h->cur];
        void *dst[8] = {N[0].x, N[0].y, N[0].z, N[0].vx, N[0].vy, N[0].vz, N[0].tet, N[0].idf};
        const void *src[8] = {O.x, O.y, O.z, O.vx, O.vy, O.vz, O.tet, O.idf};
        const size_t w[8] = {8, 8, 8, 8, 8, 8, 4, 4};
        for (int k = 0; k < 8; ++k)
            if (np) CK(cudaMemcpyAsync(dst[k], src[k], w[k] * size_t(np), cudaMemcpyDeviceToDevice, s));
        CK(cudaStreamSynchronize(s));
        free_particles(h);
        h->P[0] = N[0];
        h->P[1] = N[1];
    }
    CK(dalloc(&h->walkq, cap));
    h->cap = cap;
    h->cur = 0;
    return SPG_OK;
}

MeshDev mesh_dev(const spg_handle *h) {
    MeshDev m;
    m.rec = h->rec;
    m.screen = h->screen;
    m.nbr = h->nbr;
    m.ftri = h->ftri;
    m.tet_nodes = h->tet_nodes;
    m.node_xyz = h->node_xyz;
    m.n_tets = h->n_tets;
    m.n_nodes = h->n_nodes;
    return m;
}

StepConst step_const(const spg_handle *h) {
    const spg_params &p = h->prm;
    StepConst c{};
    c.dt = p.dt;
    c.charge = p.charge;
    c.mass = p.mass;
    c.q_over_m = p.charge / p.mass;
    c.vmin = p.min_velocity;
    for (int k = 0; k < 3; ++k) {
        c.lo[k] = h->bbox_lo[k];
        c.hi[k] = h->bbox_hi[k];
    }
    c.model = p.collision_model;
    c.max_cross = p.max_crossings;
    c.gas_n = p.gas_concentration;
    c.mass_cp = p.mass / (p.gas_mass + p.mass);
    c.mass_ct = p.gas_mass / (p.gas_mass + p.mass);
    c.sigma_hs = 3.14159265358979323846 * (p.hs_diameter * p.hs_diameter);
    c.vhs_c1 = (p.vhs_dref * p.vhs_dref) / std::tgamma(5.0 / 2.0 - p.omega);
    c.two_kT = 2.0 * p.kT_ref;
    c.mr = p.mass * p.gas_mass / (p.mass + p.gas_mass);
    c.expo = p.omega - 1.0 / 2.0;
    c.inv_alpha = 1.0 / p.alpha;
    c.seed_lo = uint32_t(p.seed);
    c.seed_hi = uint32_t(p.seed >> 32);
    c.step = h->step;
    for (int k = 0; k < 3; ++k) {
        c.lo_key[k] = order_key_host(c.lo[k]);
        c.hi_key[k] = order_key_host(c.hi[k]);
    }
    const double two_vmin = 2.0 * std::fabs(p.min_velocity);
    std::memcpy(&c.two_vmin_bits, &two_vmin, sizeof(two_vmin));
    for (int k = 0; k < 3; ++k) {
        c.lo_f[k] = float(c.lo[k]);
        c.hi_f[k] = float(c.hi[k]);
    }
    c.vmin_f = float(c.vmin);
    c.dt_f = float(c.dt);
    c.mass_cp_f = float(c.mass_cp);
    c.mass_ct_f = float(c.mass_ct);
    c.inv_alpha_f = float(c.inv_alpha);
    // FP32 screen of P = sigma |v| n dt: HS kp (v^2)^(1/2); VHS/VSS
    // pi c1 (2 kT/m_r)^(w-1/2) n dt (v^2)^(1-w).
    if (p.collision_model == SPG_COLL_HS) {
        c.kp_f = float(c.sigma_hs * p.gas_concentration * p.dt);
        c.pexp_f = 0.5f;
    } else {
        c.kp_f = float(3.14159265358979323846 * c.vhs_c1 * std::pow(c.two_kT / c.mr, c.expo) * p.gas_concentration *
                       p.dt);
        c.pexp_f = float(0.5 - c.expo);
    }
    // the FP32 probability is increasing in v^2 (pexp > 0) with a relative
    // error far below the 2e-4 margin; rounded down to a float
    {
        const double q = 1.0 / 256.0 * (1.0 - 2e-4), kp = double(c.kp_f), pe = double(c.pexp_f);
        double v2q = -1.0;
        if (p.collision_model != SPG_COLL_NONE && kp > 0.0) {
            if (pe > 0.0)
                v2q = std::pow(q / kp, 1.0 / pe);
            else if (pe == 0.0 && kp < q)
                v2q = HUGE_VAL;
        } else if (p.collision_model != SPG_COLL_NONE) {
            v2q = HUGE_VAL;  // kp = 0: no collision at all
        }
        float f = float(v2q);
        if (double(f) > v2q) f = std::nextafter(f, -HUGE_VALF);
        c.v2_cand_f = f;
    }
    return c;
}

// Fixed-point deposit exponent: every node total stays below 2^63 even if
// all n particles sit on one node.
int fix_bits_for(int64_t n) {
    int k = 52;
    while (k > 8 && double(n + 1) * std::ldexp(1.0, k) >= 9.0e18) --k;
    return k;
}

PcgDev pcg_dev(spg_handle *h) {
    PcgDev d;
    d.n = h->n_nodes;
    d.row_ptr = h->row_ptr;
    d.col = h->col;
    d.val = h->val;
    d.inv_diag = h->inv_diag;
    d.slice_ptr = h->slice_ptr;
    d.scol = h->scol;
    d.sval = h->sval;
    d.x = h->phi;
    d.r = h->r;
    d.z = h->z;
    d.p = h->p;
    d.p2 = nullptr;
    d.q = h->q;
    d.partials = h->partials;
    d.sc = h->sc;
    d.grid = h->grid64;
    return d;
}

// ---- profiling helpers
void ev_begin(spg_handle *h, EventSeries &s) {
    if (!h->prof) return;
    if (s.start.empty()) {
        s.start.resize(kEventPool);
        s.stop.resize(kEventPool);
        for (int k = 0; k < kEventPool; ++k) {
            cudaEventCreate(&s.start[k]);
            cudaEventCreate(&s.stop[k]);
        }
    }
    if (s.used == kEventPool) {  // resolve the pool before reuse
        cudaEventSynchronize(s.stop[kEventPool - 1]);
        for (int k = 0; k < kEventPool; ++k) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, s.start[k], s.stop[k]);
            s.ms += ms;
        }
        s.used = 0;
    }
    cudaEventRecord(s.start[s.used], h->stream);
}
void ev_end(spg_handle *h, EventSeries &s) {
    if (!h->prof) return;
    cudaEventRecord(s.stop[s.used], h->stream);
    s.used++;
    s.launches++;
}
void ev_resolve(EventSeries &s) {
    if (s.used == 0) return;
    cudaEventSynchronize(s.stop[s.used - 1]);
    for (int k = 0; k < s.used; ++k) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, s.start[k], s.stop[k]);
        s.ms += ms;
    }
    s.used = 0;
}
void ev_destroy(EventSeries &s) {
    for (auto e : s.start) cudaEventDestroy(e);
    for (auto e : s.stop) cudaEventDestroy(e);
    s.start.clear();
    s.stop.clear();
}

// ---- phases
template <class T>
int copy_tail(spg_handle *h, T *dst, const T *src, int64_t o, int64_t n) {
    CK(cudaMemcpyAsync(dst + o, src + o, sizeof(T) * n, cudaMemcpyDeviceToDevice, h->stream));
    return SPG_OK;
}

int do_resort(spg_handle *h) {
    if (!h->have_particles || h->np == 0) return SPG_OK;
    ev_begin(h, h->ev_sort);
    const int64_t tail = h->np - h->n_active, o = h->n_active;
    int rc = SPG_OK;
    if (h->mixed) {
        DevParticles32 &src = h->Q[h->cur], &dst = h->Q[1 - h->cur];
        launch_resort32(src, dst, h->n_active, h->n_tets, h->sort_scratch, h->n_alive_dev, h->stream);
        // Particles past n_active are dead already; they keep their slots.
        if (tail > 0)
            for (auto pr : {std::make_pair(dst.x, src.x), std::make_pair(dst.y, src.y), std::make_pair(dst.z, src.z),
                            std::make_pair(dst.vx, src.vx), std::make_pair(dst.vy, src.vy),
                            std::make_pair(dst.vz, src.vz)})
                if ((rc = copy_tail(h, pr.first, pr.second, o, tail))) return rc;
        if (tail > 0 && ((rc = copy_tail(h, dst.tet, src.tet, o, tail)) || (rc = copy_tail(h, dst.idf, src.idf, o, tail))))
            return rc;
    } else {
        DevParticles &src = h->P[h->cur], &dst = h->P[1 - h->cur];
        launch_resort(src, dst, h->n_active, h->n_tets, h->sort_scratch, h->n_alive_dev, h->stream);
        if (tail > 0)
            for (auto pr : {std::make_pair(dst.x, src.x), std::make_pair(dst.y, src.y), std::make_pair(dst.z, src.z),
                            std::make_pair(dst.vx, src.vx), std::make_pair(dst.vy, src.vy),
                            std::make_pair(dst.vz, src.vz)})
                if ((rc = copy_tail(h, pr.first, pr.second, o, tail))) return rc;
        if (tail > 0 && ((rc = copy_tail(h, dst.tet, src.tet, o, tail)) || (rc = copy_tail(h, dst.idf, src.idf, o, tail))))
            return rc;
    }
    ev_end(h, h->ev_sort);
    h->launches += h->n_active > 0 ? 5 : 3;
    CK(cudaGetLastError());
    int64_t na = 0;
    unsigned long long occ = 0;
    CK(cudaMemcpyAsync(&na, h->n_alive_dev, sizeof(na), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(&occ, sort_occupied_counter(h->sort_scratch), sizeof(occ), cudaMemcpyDeviceToHost,
                       h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (h->prof) h->sort_bytes += double(h->n_active) * 2.0 * h->pbytes + 8.0 * double(h->n_tets + 1);
    h->cur = 1 - h->cur;
    h->n_active = na;
    h->occupied = int64_t(occ);
    return SPG_OK;
}

int do_gather(spg_handle *h) {
    if (!h->have_particles) return fail(h, SPG_E_STATE, "gather: no particles set");
    CK(cudaMemsetAsync(h->node_fix, 0, sizeof(unsigned long long) * h->n_nodes, h->stream));
    // the deposit also lists the occupied tets, for the field of the next solve
    CK(cudaMemsetAsync(h->occ_n, 0, sizeof(unsigned int), h->stream));
    h->occ_epoch = h->field_epoch + 1;
    const OccList occ{h->occ_list, h->occ_n, h->occ_gen, ++h->occ_count};
    ev_begin(h, h->ev_dep);
    if (h->mixed)
        launch_deposit32(h->Q[h->cur], h->n_active, mesh_dev32(h), h->fix_bits, h->node_fix, occ, h->stream);
    else
        launch_deposit64(h->P[h->cur], h->n_active, mesh_dev(h), h->fix_bits, h->node_fix, occ, h->stream);
    ev_end(h, h->ev_dep);
    launch_fix_to_charge(h->node_fix, std::ldexp(h->prm.weight * h->prm.charge, -h->fix_bits), h->node_q,
                         h->n_nodes, h->stream);
    h->launches += 1;
    if (h->n_active > 0) h->launches += 1;
    CK(cudaGetLastError());
    if (h->prof)
        h->dep_bytes += (h->mixed ? 20.0 : 32.0) * double(h->n_active) +
                        (h->mixed ? 52.0 : 112.0) * double(h->occupied ? h->occupied : h->n_tets) +
                        16.0 * double(h->n_nodes);
    h->charge_valid = true;
    h->occ_fresh = true;
    return SPG_OK;
}

FieldArgs field_args(const spg_handle *h) {
    FieldArgs f{};
    f.tet_nodes = h->tet_nodes;
    f.phi = h->phi;
    f.efield = h->efield;
    f.rec = h->rec;
    f.rec32 = h->mixed ? h->rec32 : nullptr;
    f.stamp = h->tet_stamp;
    f.epoch = h->field_epoch;
    f.charge = h->prm.charge;
    f.mass = h->prm.mass;
    f.inv_mass = 1.0 / h->prm.mass;
    f.dt = h->prm.dt;
    f.c32 = ((h->prm.charge / h->prm.mass) * h->prm.dt) / 2.0;
    return f;
}

// E from phi for both forms (and the FP32 push increment of the mixed form):
// every tet, or (sparse, the solves of spg_run) only the tets holding
// particles; the walks compute the others as particles enter them.
int update_field(spg_handle *h, bool sparse) {
    ev_begin(h, h->ev_ef);
    h->field_epoch++;
    const FieldArgs f = field_args(h);
    if (sparse && h->occ_epoch == h->field_epoch) {  // the deposit before this solve listed the tets
        if (h->mixed)
            launch_field32_list(f, h->occ_list, h->occ_n, h->stream);
        else
            launch_field64_list(f, h->occ_list, h->occ_n, h->stream);
    } else if (sparse) {
        if (h->mixed)
            launch_refresh32(h->Q[h->cur], h->n_active, f, h->stream);
        else
            launch_refresh64(h->P[h->cur], h->n_active, f, h->stream);
    } else if (h->mixed) {
        launch_field32_full(f, h->n_tets, h->stream);
    } else {
        launch_field64_full(f, h->n_tets, h->stream);
    }
    h->field_full = !sparse;
    h->launches += 1;
    ev_end(h, h->ev_ef);
    CK(cudaGetLastError());
    return SPG_OK;
}

// E = 0 everywhere (no solve yet).
void zero_field(spg_handle *h) {
    h->field_epoch++;
    h->field_full = true;
    launch_zero_field(field_args(h), h->n_tets, h->stream);
}

// The statistics of a finished solve; SPG_E_NOT_CONVERGED if it hit max_iter.
int record_solve(spg_handle *h, int32_t iters, double rr, double bb, bool capped) {
    h->cg_iters_last = iters;
    h->cg_iters_total += iters;
    h->cg_solves++;
    h->cg_relres_last = bb > 0.0 ? std::sqrt(rr / bb) : 0.0;
    if (capped) {
        std::ostringstream os;
        os << "PCG did not converge: " << iters << " iterations, relative residual " << h->cg_relres_last;
        return fail(h, SPG_E_NOT_CONVERGED, os.str());
    }
    return SPG_OK;
}

int finish_solve(spg_handle *h, int32_t iters, double rr, double bb, bool capped) {
    int rc = update_field(h, h->in_run);
    if (rc) return rc;
    return record_solve(h, iters, rr, bb, capped);
}

// Launch count and profiled bytes of a while-graph solve (kind 0: do_solve64,
// 1: do_solve_mixed_amg) that ran hs.iters iterations.
void account_while_solve(spg_handle *h, int kind, const PcgScalars &hs) {
    h->launches += int64_t(hs.iters + 1) * (pcg_iter_launches(h) + 1);
    if (!h->prof) return;
    const double n = double(h->n_nodes), nnz = double(h->nnz_kept);
    h->pcg_iters_prof += hs.iters;
    if (kind == 1)  // spmv_dot 12 nnz + 24 n, update 52 n, FP32 V-cycle, r.z 12 n, p update 20 n
        h->pcg_bytes += double(hs.iters + 1) * (12.0 * nnz + 108.0 * n + h->amg_bytes);
    else if (h->amg)  // spmv_dot 12 nnz + 24 n, update 48 n, V-cycle, r.z 16 n, p update 24 n
        h->pcg_bytes += double(hs.iters + 1) * (12.0 * nnz + 112.0 * n + h->amg_bytes);
    else
        h->pcg_bytes += double(hs.iters) * (12.0 * nnz + 4.0 * (n + 1.0) + 72.0 * n);
}

// The statistics of the solves held back by the run (one synchronisation).
int drain_solves(spg_handle *h) {
    if (h->n_solve_rec == 0) return SPG_OK;
    CK(cudaStreamSynchronize(h->stream));
    const int n = h->n_solve_rec;
    h->n_solve_rec = 0;
    for (int k = 0; k < n; ++k) {
        const PcgScalars hs = h->solve_rec[k];
        account_while_solve(h, h->solve_kind[k], hs);
        if (record_solve(h, hs.iters, hs.rr, hs.bb, hs.converged == 2) == SPG_E_NOT_CONVERGED)
            h->deferred_capped = true;
    }
    return SPG_OK;
}

// After the while graph of a solve inside spg_run: its scalars into the next
// pinned record (stream-ordered, the host goes on), then the field.
int defer_solve(spg_handle *h, int kind) {
    if (!h->solve_rec) CK(cudaHostAlloc(reinterpret_cast<void **>(&h->solve_rec), sizeof(PcgScalars) * kSolveRecs,
                                        cudaHostAllocDefault));
    if (h->n_solve_rec == kSolveRecs) {
        const int rc = drain_solves(h);
        if (rc) return rc;
    }
    CK(cudaMemcpyAsync(&h->solve_rec[h->n_solve_rec], h->sc, sizeof(PcgScalars), cudaMemcpyDeviceToHost, h->stream));
    h->solve_kind[h->n_solve_rec++] = uint8_t(kind);
    ev_end(h, h->ev_pcg);
    return update_field(h, h->in_run);
}

// A PCG as one graph: a while node repeats the body (one iteration, `iterate`)
// until the device scalars say converged, capped or failed, with no host
// round trip per iteration. Built once per solver; if the CUDA runtime refuses a
// conditional node, *failed is set and the caller keeps its chunked graph.
template <class F>
void build_pcg_while(spg_handle *h, F iterate, cudaGraphExec_t *exec, bool *failed) {
    cudaGraph_t g = nullptr;
    cudaGraphConditionalHandle cond = 0;
    cudaGraphNode_t node = nullptr;
    cudaGraphNodeParams np = {};
    bool ok = cudaGraphCreate(&g, 0) == cudaSuccess &&
              cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault) == cudaSuccess;
    if (ok) {
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = cond;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        ok = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np) == cudaSuccess;
    }
    if (ok) {
        cudaGraph_t body = np.conditional.phGraph_out[0];
        ok = cudaStreamBeginCaptureToGraph(h->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
             cudaSuccess;
        if (ok) {
            iterate();
            launch_pcg_continue(cond, h->sc, h->stream);
            ok = cudaStreamEndCapture(h->stream, &body) == cudaSuccess;
        }
    }
    if (ok) ok = cudaGraphInstantiate(exec, g, 0) == cudaSuccess;
    if (g) cudaGraphDestroy(g);
    if (!ok) {
        *exec = nullptr;
        *failed = true;
        cudaGetLastError();
    }
}

int do_solve64(spg_handle *h) {
    const int64_t n = h->n_nodes;
    PcgScalars init{};
    init.tol2 = (h->prm.cg_rtol * h->prm.cg_rtol);
    init.max_iter = h->prm.cg_max_iter;
    CK(cudaMemcpyAsync(h->sc, &init, sizeof(init), cudaMemcpyHostToDevice, h->stream));
    PcgDev d = pcg_dev(h);
    ev_begin(h, h->ev_pcg);
    pcg_setup_any(h, d, h->b);
    h->launches += h->amg ? 2 + h->amg_launches : 1;
    PcgScalars hs{};
    if (!h->pcg64_while && !h->pcg64_while_failed)
        build_pcg_while(h, [&] { pcg_iteration_any(h, d); }, &h->pcg64_while, &h->pcg64_while_failed);
    const int chunk = pcg_chunk(h);
    if (h->pcg64_while) {
        CK(cudaGraphLaunch(h->pcg64_while, h->stream));
        if (h->defer_solves) return defer_solve(h, 0);
        CK(cudaMemcpyAsync(&hs, h->sc, sizeof(hs), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        ev_end(h, h->ev_pcg);
        account_while_solve(h, 0, hs);
        return finish_solve(h, hs.iters, hs.rr, hs.bb, hs.converged == 2);
    } else if (!h->pcg_graph) {
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < chunk; ++k) pcg_iteration_any(h, d);
        CK(cudaStreamEndCapture(h->stream, &g));
        CK(cudaGraphInstantiate(&h->pcg_graph, g, 0));
        cudaGraphDestroy(g);
    }
    for (;;) {
        CK(cudaGraphLaunch(h->pcg_graph, h->stream));
        h->launches += pcg_iter_launches(h) * chunk;
        CK(cudaMemcpyAsync(&hs, h->sc, sizeof(hs), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        if (hs.converged) break;
    }
    ev_end(h, h->ev_pcg);
    if (h->prof) {
        h->pcg_iters_prof += hs.iters;
        if (h->amg)  // spmv_dot 12 nnz + 24 n, update 48 n, V-cycle, r.z 16 n, p update 24 n
            h->pcg_bytes += double(hs.iters + 1) * (12.0 * double(h->nnz_kept) + 112.0 * double(n) + h->amg_bytes);
        else
            h->pcg_bytes += double(hs.iters) * (12.0 * double(h->nnz_kept) + 4.0 * double(n + 1) + 72.0 * double(n));
    }
    return finish_solve(h, hs.iters, hs.rr, hs.bb, hs.converged == 2);
}

// Mixed form with AMG: FP64 PCG (SpMV, vectors, sums, stop test) with the
// FP32 V-cycle as the preconditioner. The V-cycle's rounding perturbs M^-1 by
// about 1e-7 relative, far below what changes the CG iteration count, and the
// iterate converges on the FP64 residual ||b - A x|| <= cg_rtol ||b||.
int do_solve_mixed_amg(spg_handle *h) {
    const int64_t n = h->n_nodes;
    PcgScalars init{};
    init.tol2 = h->prm.cg_rtol * h->prm.cg_rtol;
    init.max_iter = h->prm.cg_max_iter;
    CK(cudaMemcpyAsync(h->sc, &init, sizeof(init), cudaMemcpyHostToDevice, h->stream));
    PcgDev d = pcg_dev(h);
    ev_begin(h, h->ev_pcg);
    const bool rotated = pcg_rotated_ok(h->amgd32);
    if (!h->pcg_while && !h->pcg_while_failed && rotated)
        build_pcg_while(h, [&] { launch_pcg_rotated_iteration_amg_mixed(d, h->amgd32, h->r32, h->z32, h->stream); },
                        &h->pcg_while, &h->pcg_while_failed);
    if (h->pcg_while) {
        // r only; the first iteration of the graph begins with the V-cycle
        launch_pcg_residual_amg_mixed(d, h->b, h->r32, h->stream);
        h->launches += 1;
    } else {
        launch_pcg_setup_amg_mixed(d, h->amgd32, h->b, h->r32, h->z32, h->stream);
        h->launches += 2 + h->amg_launches - pcg_rz_fused(h);
    }
    if (h->pcg_while) {
        CK(cudaGraphLaunch(h->pcg_while, h->stream));
        if (h->defer_solves) return defer_solve(h, 1);
        PcgScalars hs{};
        CK(cudaMemcpyAsync(&hs, h->sc, sizeof(hs), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        ev_end(h, h->ev_pcg);
        account_while_solve(h, 1, hs);
        return finish_solve(h, hs.iters, hs.rr, hs.bb, hs.converged == 2);
    }
    const int chunk = pcg_chunk(h);
    if (!h->pcg32_graph) {
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < chunk; ++k) launch_pcg_iteration_amg_mixed(d, h->amgd32, h->r32, h->z32, h->stream);
        CK(cudaStreamEndCapture(h->stream, &g));
        CK(cudaGraphInstantiate(&h->pcg32_graph, g, 0));
        cudaGraphDestroy(g);
    }
    PcgScalars hs{};
    for (;;) {
        CK(cudaGraphLaunch(h->pcg32_graph, h->stream));
        h->launches += pcg_iter_launches(h) * chunk;
        CK(cudaMemcpyAsync(&hs, h->sc, sizeof(hs), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        if (hs.converged) break;
    }
    ev_end(h, h->ev_pcg);
    if (h->prof) {  // spmv_dot 12 nnz + 24 n, update 52 n, FP32 V-cycle, r.z 12 n, p update 20 n
        h->pcg_iters_prof += hs.iters;
        h->pcg_bytes += double(hs.iters + 1) * (12.0 * double(h->nnz_kept) + 108.0 * double(n) + h->amg_bytes);
    }
    return finish_solve(h, hs.iters, hs.rr, hs.bb, hs.converged == 2);
}

// Mixed form with Jacobi: FP32-SpMV PCG corrections inside FP64 iterative
// refinement, stopped on the FP64 residual ||b - A x|| <= cg_rtol ||b||.
int do_solve_mixed(spg_handle *h) {
    if (h->amg32) return do_solve_mixed_amg(h);
    const int64_t n = h->n_nodes;
    PcgScalars outer{}, inner{};
    outer.tol2 = h->prm.cg_rtol * h->prm.cg_rtol;
    inner.tol2 = kInnerRtol * kInnerRtol;
    inner.max_iter = kInnerMaxIter;
    CK(cudaMemcpyAsync(h->sc, &outer, sizeof(outer), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->sc32, &inner, sizeof(inner), cudaMemcpyHostToDevice, h->stream));
    PcgDev d = pcg_dev(h);
    PcgDev32 f = pcg_dev32(h);
    const int chunk = pcg_chunk(h);
    if (!h->pcg32_graph) {
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < chunk; ++k) launch_pcg32_iteration(f, h->stream);
        CK(cudaStreamEndCapture(h->stream, &g));
        CK(cudaGraphInstantiate(&h->pcg32_graph, g, 0));
        cudaGraphDestroy(g);
    }
    ev_begin(h, h->ev_pcg);
    int32_t total = 0;
    PcgScalars hs{}, hi{};
    bool capped = true;
    for (int outer_it = 0; outer_it <= kOuterMax; ++outer_it) {
        launch_refine_setup(d, f, h->b, h->stream);
        h->launches += 1;
        CK(cudaMemcpyAsync(&hs, h->sc, sizeof(hs), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        if (hs.converged) {
            capped = false;
            break;
        }
        if (outer_it == kOuterMax || total >= h->prm.cg_max_iter) break;
        for (;;) {
            CK(cudaGraphLaunch(h->pcg32_graph, h->stream));
            h->launches += pcg_iter_launches(h) * chunk;
            CK(cudaMemcpyAsync(&hi, h->sc32, sizeof(hi), cudaMemcpyDeviceToHost, h->stream));
            CK(cudaStreamSynchronize(h->stream));
            if (hi.converged) break;
        }
        total += hi.iters;
        launch_refine_apply(h->phi, h->e32, n, h->stream);
        h->launches += 1;
    }
    ev_end(h, h->ev_pcg);
    if (h->prof) {
        h->pcg_iters_prof += total;
        h->pcg_bytes += double(total) * (8.0 * double(h->nnz_kept) + 4.0 * double(n + 1) + 36.0 * double(n));
    }
    return finish_solve(h, total, hs.rr, hs.bb, capped);
}

int do_solve(spg_handle *h) {
    launch_pcg_rhs(h->node_q, 1.0 / h->prm.epsilon0, h->lift, h->is_dir, h->dir_value, h->b, h->n_nodes, h->stream);
    h->launches += 1;
    if (h->amg32) return do_solve_mixed_amg(h);
    return h->mixed ? do_solve_mixed(h) : do_solve64(h);
}

// Appends the position of each tracked particle that is still alive (before
// the step, as the reference records it before the move).
int record_tracks(spg_handle *h) {
    const uint32_t *idf = h->mixed ? h->Q[h->cur].idf : h->P[h->cur].idf;
    launch_track_find(idf, h->np, h->track_of_id, h->track_table_n, h->track_slot, h->stream);
    if (h->mixed)
        launch_track_record32(h->Q[h->cur], h->cen, h->track_slot, h->track_k, h->track_cap, h->track_count,
                              h->track_xyz, h->stream);
    else
        launch_track_record64(h->P[h->cur], h->track_slot, h->track_k, h->track_cap, h->track_count, h->track_xyz,
                              h->stream);
    h->launches += 2;
    CK(cudaGetLastError());
    return SPG_OK;
}

void free_tracks(spg_handle *h) {
    for (void *q : {(void *)h->track_ids, (void *)h->track_of_id, (void *)h->track_slot, (void *)h->track_count,
                    (void *)h->track_xyz, (void *)h->track_cur, (void *)h->track_flags})
        cudaFree(q);
    h->track_ids = nullptr;
    h->track_of_id = h->track_slot = h->track_count = nullptr;
    h->track_xyz = h->track_cur = nullptr;
    h->track_flags = nullptr;
    h->track_k = h->track_cap = 0;
}

int do_process(spg_handle *h) {
    h->occ_fresh = false;
    if (h->track_k > 0) {
        const int rc = record_tracks(h);
        if (rc) return rc;
    }
    StepConst c = step_const(h);
    ev_begin(h, h->ev_step);
    if (h->mixed)
        launch_step32(h->Q[h->cur], h->n_active, mesh_dev32(h), c, h->tri_count, h->walkq, h->walkq_n, h->ctr,
                      field_args(h), h->stream);
    else
        launch_step64(h->P[h->cur], h->n_active, mesh_dev(h), c, h->tri_count, h->walkq, h->walkq_n, h->ctr,
                      field_args(h), h->stream);
    ev_end(h, h->ev_step);
    if (h->n_active > 0) h->launches += 2;  // step kernel + queued walks
    CK(cudaGetLastError());
    if (h->prof)
        h->step_bytes += (h->mixed ? 92.0 : 152.0) *
                         double(h->occupied ? h->occupied : std::min(h->n_tets, h->n_active));
    h->step++;
    return SPG_OK;
}

// Steps h->step .. h->step + l - 1 of the mixed form as one segment (nothing
// of the time loop falls between them).
int do_segment32(spg_handle *h, int l) {
    h->occ_fresh = false;
    if (h->seg_rq_cap < h->cap) {
        cudaFree(h->seg_rq);
        h->seg_rq = nullptr;
        h->seg_rq_cap = 0;
        CK(dalloc(&h->seg_rq, size_t(std::max<int64_t>(h->cap, 1))));
        h->seg_rq_cap = h->cap;
    }
    if (h->seg_qn_cap < 2 * l + 1) {
        cudaFree(h->seg_qn);
        h->seg_qn = nullptr;
        h->seg_qn_cap = 0;
        CK(dalloc(&h->seg_qn, size_t(2 * h->seg_max + 1)));
        h->seg_qn_cap = 2 * h->seg_max + 1;
    }
    StepConst c = step_const(h);
    ev_begin(h, h->ev_step);
    const int nl = launch_segment32(h->Q[h->cur], h->n_active, mesh_dev32(h), c, l, h->tri_count, h->walkq,
                                    h->seg_rq, h->seg_qn, h->ctr, field_args(h), h->stream);
    ev_end(h, h->ev_step);
    h->launches += nl;
    CK(cudaGetLastError());
    if (h->prof)
        h->step_bytes += double(l) * 92.0 * double(h->occupied ? h->occupied : std::min(h->n_tets, h->n_active));
    h->step += l;
    return SPG_OK;
}

// l steps with nothing of the time loop between them: segments of at most
// seg_max steps in the mixed form (without trajectory sampling, which records
// every step), single steps otherwise.
int do_steps(spg_handle *h, int l) {
    if (h->mixed && h->track_k == 0 && h->seg_max > 1 && l > 1) {
        while (l > 0) {
            const int m = std::min(l, h->seg_max);
            const int rc = do_segment32(h, m);
            if (rc) return rc;
            l -= m;
        }
        return SPG_OK;
    }
    for (int k = 0; k < l; ++k) {
        const int rc = do_process(h);
        if (rc) return rc;
    }
    return SPG_OK;
}

// Steps from h->step to the next step at which the time loop does more than
// step (a re-sort, or with `solves` a deposit and solve), at most `left`.
int steps_to_event(const spg_handle *h, int64_t left, bool solves) {
    int64_t l = left;
    const int64_t s = h->step;
    if (solves && h->prm.poisson_every > 0) l = std::min(l, h->prm.poisson_every - s % h->prm.poisson_every);
    if (h->prm.resort_every > 0) l = std::min(l, h->prm.resort_every - s % h->prm.resort_every);
    return int(std::max<int64_t>(l, 1));
}

int read_counters(spg_handle *h, DevCounters &c) {
    CK(cudaMemcpyAsync(&c, h->ctr, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return SPG_OK;
}

int fill_stats(spg_handle *h, spg_stats *st) {
    if (!st) return SPG_OK;
    DevCounters c{};
    int rc = read_counters(h, c);
    if (rc) return rc;
    st->step = h->step;
    st->n_particles = h->np;
    st->n_settled = int64_t(c.settled);
    st->n_lost = int64_t(c.lost) + h->init_lost;
    st->n_alive = h->np - st->n_settled - st->n_lost;
    st->particle_steps = int64_t(c.processed);
    st->collisions = int64_t(c.collisions);
    st->crossings = int64_t(c.crossings);
    st->cg_iters_total = h->cg_iters_total;
    st->cg_iters_last = h->cg_iters_last;
    st->cg_solves = h->cg_solves;
    st->cg_relres_last = h->cg_relres_last;
    return SPG_OK;
}

// The electrode field into phi_vac: one solve from the Dirichlet values with
// no charge. Its iterations are not counted as a run's.
int solve_vacuum(spg_handle *h) {
    const int64_t n = h->n_nodes;
    if (!h->phi_vac) CK(dalloc(&h->phi_vac, n));
    CK(cudaMemcpyAsync(h->phi, h->phi_init.data(), sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemsetAsync(h->node_q, 0, sizeof(double) * n, h->stream));
    h->phi_hist = 0;
    const bool prev = h->in_run;
    h->in_run = false;
    const int rc = do_solve(h);
    h->in_run = prev;
    if (rc == SPG_E_NOT_CONVERGED) return SPG_OK;  // not kept: new particle sets start from phi_init
    if (rc) return rc;
    CK(cudaMemcpyAsync(h->phi_vac, h->phi, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
    h->vac_valid = true;
    return SPG_OK;
}

int reset_run_state(spg_handle *h) {
    if ((h->amg || h->amg32) && !h->vac_valid) {
        const int rc = solve_vacuum(h);
        if (rc) return rc;
    }
    h->step = 0;
    h->cg_iters_last = 0;
    h->cg_solves = 0;
    h->cg_iters_total = 0;
    h->cg_relres_last = 0.0;
    h->charge_valid = false;
    h->occ_fresh = false;
    h->resorted_at = -1;
    CK(cudaMemsetAsync(h->ctr, 0, sizeof(DevCounters), h->stream));
    CK(cudaMemsetAsync(h->tri_count, 0, sizeof(unsigned int) * std::max<int64_t>(h->n_tris, 1), h->stream));
    if (h->vac_valid)  // AMG: a new particle set starts from the electrode field
        CK(cudaMemcpyAsync(h->phi, h->phi_vac, sizeof(double) * h->n_nodes, cudaMemcpyDeviceToDevice, h->stream));
    else
        CK(cudaMemcpyAsync(h->phi, h->phi_init.data(), sizeof(double) * h->n_nodes, cudaMemcpyHostToDevice,
                           h->stream));
    CK(cudaMemsetAsync(h->node_q, 0, sizeof(double) * h->n_nodes, h->stream));
    zero_field(h);
    h->phi_hist = 0;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->stream));
    return SPG_OK;
}

int validate_params(const spg_params *p, std::string &msg) {
    if (!(p->dt > 0.0)) msg = "dt must be > 0";
    else if (!(p->mass > 0.0)) msg = "mass must be > 0";
    else if (!(p->weight > 0.0)) msg = "weight must be > 0";
    else if (!(p->epsilon0 > 0.0)) msg = "epsilon0 must be > 0";
    else if (p->collision_model < SPG_COLL_NONE || p->collision_model > SPG_COLL_VSS) msg = "bad collision_model";
    else if (p->precision != SPG_FP64 && p->precision != SPG_MIXED) msg = "bad precision";
    else if (p->preconditioner != SPG_PRECOND_JACOBI && p->preconditioner != SPG_PRECOND_AMG &&
             p->preconditioner != SPG_PRECOND_AMG_F32)
        msg = "bad preconditioner";
    else if (p->collision_model != SPG_COLL_NONE && !(p->gas_mass > 0.0)) msg = "gas_mass must be > 0";
    else if (p->collision_model != SPG_COLL_NONE && !(p->gas_concentration >= 0.0)) msg = "gas_concentration < 0";
    else if (p->collision_model == SPG_COLL_VSS && !(p->alpha > 0.0)) msg = "alpha must be > 0";
    else if (p->poisson_every < 1) msg = "poisson_every must be >= 1";
    else if (p->resort_every < 0) msg = "resort_every must be >= 0";
    else if (p->max_crossings < 1) msg = "max_crossings must be >= 1";
    else if (p->cg_max_iter < 1) msg = "cg_max_iter must be >= 1";
    else if (!(p->cg_rtol > 0.0)) msg = "cg_rtol must be > 0";
    else return SPG_OK;
    return SPG_E_INVALID;
}

}  // namespace

extern "C" {

const char *spg_version(void) { return "start_gb300 1.0 (sm_103a)"; }

void spg_default_params(spg_params *p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->dt = 1e-8;
    p->charge = 1.602176565e-19;  // Constants.hpp e_charge
    p->mass = 7.9485017e-26;      // Ti
    p->weight = 1.0;
    p->collision_model = SPG_COLL_NONE;
    p->precision = SPG_FP64;
    p->gas_mass = 6.6335209e-26;  // Ar
    p->gas_concentration = 0.0;
    p->hs_diameter = 3.6e-10;
    p->vhs_dref = 4.17e-10;
    p->omega = 0.81;
    p->alpha = 1.40;
    p->kT_ref = 297.0 * 1.380658e-23;  // Constants.hpp:12
    p->epsilon0 = 8.8541878128e-12;
    p->min_velocity = 10.0;  // Constants.hpp:50
    p->bbox_expansion = 1.01;
    p->seed = 0;
    p->poisson_every = 10;
    p->resort_every = 20;
    p->max_crossings = 4096;
    p->cg_max_iter = 20000;
    p->cg_rtol = 1e-10;
    p->device = 0;
    p->preconditioner = SPG_PRECOND_JACOBI;
}

const char *spg_last_error(const spg_handle *h) { return h ? h->err.c_str() : g_create_error.c_str(); }

int spg_create(const spg_mesh_desc *mesh, const spg_params *params, spg_handle **out) {
    spg_handle *h = nullptr;
    if (!mesh || !params || !out) return fail(h, SPG_E_INVALID, "spg_create: null argument");
    *out = nullptr;
    std::string msg;
    if (validate_params(params, msg)) return fail(h, SPG_E_INVALID, "spg_create: " + msg);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(h, SPG_E_NO_DEVICE, "spg_create: no CUDA device");
    if (params->device < 0 || params->device >= ndev) return fail(h, SPG_E_NO_DEVICE, "spg_create: bad device");
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, params->device);
    if (prop.major * 10 + prop.minor != 103) {
        std::ostringstream os;
        os << "spg_create: built for sm_103a (GB300); device is sm_" << prop.major << prop.minor;
        return fail(h, SPG_E_NO_DEVICE, os.str());
    }
    if (cudaSetDevice(params->device) != cudaSuccess) return fail(h, SPG_E_NO_DEVICE, "spg_create: cudaSetDevice");
    const auto t_create = std::chrono::steady_clock::now();
    HostMesh hm;
    std::string err;
    int rc = prepare_mesh(*mesh, params->bbox_expansion, hm, err);
    if (rc) return fail(h, rc, err);

    std::unique_ptr<spg_handle> H(new (std::nothrow) spg_handle());
    if (!H) return fail(h, SPG_E_OOM, "spg_create: host allocation failed");
    h = H.get();
    h->prm = *params;
    h->device = params->device;
    {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccessUsesHostPageTables, params->device) ==
            cudaSuccess)
            h->ats = v != 0;
        cudaGetLastError();
    }
    h->mixed = params->precision == SPG_MIXED;
    h->pbytes = h->mixed ? 32.0 : 56.0;
    CK(cudaSetDevice(h->device));
    CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    h->n_nodes = hm.n_nodes;
    h->n_tets = hm.n_tets;
    h->n_tris = hm.n_tris;
    h->n_boundary_faces = hm.n_boundary_faces;
    h->nnz = int64_t(hm.col.size());
    h->n_dirichlet = hm.n_dirichlet;
    for (int k = 0; k < 3; ++k) {
        h->bbox_lo[k] = hm.bbox_lo[k];
        h->bbox_hi[k] = hm.bbox_hi[k];
        h->vox_oi[k] = hm.vox_origin[k];
        h->vox_oi[3 + k] = hm.vox_inv[k];
        h->vox_dims[k] = hm.vox_dims[k];
    }
    std::vector<double> inv_diag(hm.diag.size());
    for (size_t i = 0; i < hm.diag.size(); ++i) inv_diag[i] = 1.0 / hm.diag[i];
    cudaStream_t s = h->stream;
    CK(upload(&h->rec, hm.rec, s));
    {
        std::vector<TetScreen> scr(hm.n_tets);
        for (int64_t t = 0; t < hm.n_tets; ++t) {
            for (int k = 0; k < 9; ++k) scr[t].M[k] = hi_float(hm.rec[t].M[k]);
            for (int k = 0; k < 3; ++k) scr[t].x0[k] = hi_float(hm.rec[t].x0[k]);
        }
        CK(upload(&h->screen, scr, s));
    }
    CK(upload(reinterpret_cast<int32_t **>(&h->nbr), hm.nbr, s));
    CK(upload(reinterpret_cast<int32_t **>(&h->ftri), hm.ftri, s));
    CK(upload(reinterpret_cast<int32_t **>(&h->tet_nodes), hm.tet_nodes, s));
    CK(upload(&h->node_xyz, hm.node_xyz, s));
    {
        std::vector<int64_t> sp;
        std::vector<int32_t> sc;
        std::vector<double> sv;
        build_sell32(hm.n_nodes, hm.row_ptr.data(), hm.col.data(), hm.val.data(), sp, sc, sv);
        h->sell_entries = int64_t(sv.size());
        h->nnz_kept = 0;
        for (int64_t r = 0; r < hm.n_nodes; ++r)
            for (int32_t k = hm.row_ptr[r]; k < hm.row_ptr[r + 1]; ++k)
                h->nnz_kept += (hm.val[k] != 0.0 || hm.col[k] == r) ? 1 : 0;
        CK(upload(&h->slice_ptr, sp, s));
        CK(upload(&h->scol, sc, s));
        CK(upload(&h->sval, sv, s));
        if (h->mixed || h->prm.preconditioner == SPG_PRECOND_AMG_F32) {
            std::vector<float> sv32(sv.begin(), sv.end());
            CK(upload(&h->sval32, sv32, s));
        }
    }
    if (h->prm.preconditioner == SPG_PRECOND_AMG || h->prm.preconditioner == SPG_PRECOND_AMG_F32) {
        const auto t0 = std::chrono::steady_clock::now();
        int rc = setup_amg(h, hm);
        if (rc) return rc;
        h->setup_ms[4] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    {
        std::vector<int64_t> erp(hm.n_nodes + 1, 0);
        for (int32_t r : hm.elim_row) erp[r + 1]++;
        for (int64_t i = 0; i < hm.n_nodes; ++i) erp[i + 1] += erp[i];
        h->n_elim = int64_t(hm.elim_val.size());
        CK(upload(&h->elim_rp, erp, s));
        CK(upload(&h->elim_row, hm.elim_row, s));
        CK(upload(&h->elim_col, hm.elim_col, s));
        CK(upload(&h->elim_val, hm.elim_val, s));
    }
    CK(upload(&h->row_ptr, hm.row_ptr, s));
    CK(upload(&h->col, hm.col, s));
    CK(upload(&h->val, hm.val, s));
    CK(upload(&h->inv_diag, inv_diag, s));
    CK(upload(&h->is_dir, hm.is_dir, s));
    CK(upload(&h->dir_value, hm.dir_value, s));
    CK(upload(&h->lift, hm.lift, s));
    CK(upload(&h->dual_vol, hm.dual_vol, s));
    CK(upload(&h->vox_seed, hm.vox_seed, s));
    h->phi_init = hm.dir_value;
    if (h->mixed) {
        // FP32 maps about the centroid, FP64 centroids, FP32 inner-solver arrays
        std::vector<TetRec32> r32(hm.n_tets);
        std::vector<double> cen(3 * hm.n_tets);
        std::vector<float> cen_lo(3 * hm.n_tets);
        // Interior tets: every vertex inside the modelling box by 1e-5 of its
        // extent plus its largest coordinate, some hundred times the FP32
        // rounding of a centroid-plus-local position and of the box bounds.
        double margin = 0.0;
        for (int c = 0; c < 3; ++c)
            margin = std::max(margin, 1e-5 * ((hm.bbox_hi[c] - hm.bbox_lo[c]) +
                                              std::max(std::fabs(hm.bbox_lo[c]), std::fabs(hm.bbox_hi[c]))));
        for (int64_t t = 0; t < hm.n_tets; ++t) {
            for (int c = 0; c < 3; ++c) {
                double acc = 0.0;
                for (int k = 0; k < 4; ++k) acc += hm.node_xyz[3 * int64_t(hm.tet_nodes[4 * t + k]) + c];
                cen[3 * t + c] = 0.25 * acc;
            }
            TetRec32 &q = r32[t];
            for (int k = 0; k < 9; ++k) q.M[k] = float(hm.rec[t].M[k]);
            for (int c = 0; c < 3; ++c) {
                q.H[c] = 0.0f;
                q.cen[c] = float(cen[3 * t + c]);
                cen_lo[3 * t + c] = float(cen[3 * t + c] - double(q.cen[c]));
            }
            bool interior = true;
            for (int k = 0; k < 4; ++k)
                for (int c = 0; c < 3; ++c) {
                    const double v = hm.node_xyz[3 * int64_t(hm.tet_nodes[4 * t + k]) + c];
                    interior = interior && v >= hm.bbox_lo[c] + margin && v <= hm.bbox_hi[c] - margin;
                }
            q.ezero = kRecEzero | (interior ? kRecInterior : 0u);
        }
        CK(upload(&h->rec32, r32, s));
        CK(upload(&h->cen, cen, s));
        CK(upload(&h->cen_lo, cen_lo, s));
        std::vector<float> id32(inv_diag.begin(), inv_diag.end());
        CK(upload(&h->inv_diag32, id32, s));
        CK(dalloc(&h->e32, hm.n_nodes));
        CK(dalloc(&h->r32, hm.n_nodes));
        CK(dalloc(&h->z32, hm.n_nodes));
        CK(dalloc(&h->p32, hm.n_nodes));
        CK(dalloc(&h->q32, hm.n_nodes));
    }
    const int64_t n = h->n_nodes;
    CK(dalloc(&h->node_q, n));
    CK(dalloc(&h->node_fix, n));
    CK(dalloc(&h->efield, 3 * size_t(h->n_tets)));
    CK(dalloc(&h->tet_stamp, size_t(h->n_tets)));
    CK(dalloc(&h->occ_list, size_t(h->n_tets)));
    CK(dalloc(&h->occ_n, 1));
    CK(dalloc(&h->occ_gen, size_t(h->n_tets)));
    CK(cudaMemsetAsync(h->occ_gen, 0, sizeof(uint32_t) * size_t(h->n_tets), s));
    CK(cudaMemsetAsync(h->tet_stamp, 0, sizeof(uint32_t) * size_t(h->n_tets), s));
    CK(dalloc(&h->rho, n));
    CK(dalloc(&h->phi, n));
    CK(dalloc(&h->phi_prev, n));
    CK(dalloc(&h->phi_prev2, n));
    CK(dalloc(&h->b, n));
    CK(dalloc(&h->r, n));
    CK(dalloc(&h->z, n));
    CK(dalloc(&h->p, n));
    CK(dalloc(&h->q, n));
    h->pcg_blocks = pcg_blocks(n);
    h->grid64 = pcg_grid64(n);
    h->grid32 = pcg_grid32(n);
    CK(cudaGetLastError());
    CK(dalloc(&h->partials, 3 * size_t(h->pcg_blocks)));
    CK(dalloc(&h->sc, 1));
    CK(dalloc(&h->partials32, 3 * size_t(h->pcg_blocks)));
    CK(dalloc(&h->sc32, 1));
    CK(cudaMemsetAsync(h->sc32, 0, sizeof(PcgScalars), s));
    CK(cudaMemsetAsync(h->sc, 0, sizeof(PcgScalars), s));
    CK(dalloc(&h->tri_count, std::max<int64_t>(h->n_tris, 1)));
    CK(dalloc(&h->ctr, 1));
    CK(dalloc(&h->walkq_n, 1));
    CK(dalloc(&h->n_alive_dev, 1));
    CK(dalloc(&h->sort_scratch, size_t(sort_scratch_words(h->n_tets))));
    rc = reset_run_state(h);
    if (rc) return rc;
    CK(cudaStreamSynchronize(s));
    {
        double *t = h->setup_ms;
        t[0] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_create).count();
        t[1] = hm.prep_ms[0];
        t[2] = hm.prep_ms[1];
        t[3] = hm.prep_ms[2] - hm.prep_ms[0] - hm.prep_ms[1];
        t[5] = t[0] - hm.prep_ms[2] - t[4];
    }
    *out = H.release();
    return SPG_OK;
}

int spg_setup_times(const spg_handle *h, double ms[6]) {
    if (!h || !ms) return SPG_E_INVALID;
    for (int k = 0; k < 6; ++k) ms[k] = h->setup_ms[k];
    return SPG_OK;
}

int spg_destroy(spg_handle *h) {
    if (!h) return SPG_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_particles(h);
    void *ptrs[] = {h->rec,      h->screen,   h->nbr,      h->ftri,     h->tet_nodes, h->node_xyz, h->row_ptr,   h->col,
                    h->val,      h->inv_diag, h->is_dir,   h->dir_value, h->lift,     h->dual_vol,  h->vox_seed,
                    h->node_q,   h->rho,      h->phi,      h->phi_prev,  h->phi_prev2,      h->b,         h->r,        h->z,         h->p,
                    h->phi_vac,  h->id_slot,  h->io_counter, h->grad_G, h->grad_En,
                    h->node_fix, h->efield,   h->tet_stamp, h->occ_list, h->occ_n, h->occ_gen,   h->slice_ptr, h->scol,   h->sval,
                    h->rec32,    h->cen,      h->cen_lo,   h->sval32,   h->inv_diag32, h->e32,     h->r32,       h->z32,
                    h->p32,      h->q32,      h->partials32, h->sc32,
                    h->elim_rp,  h->elim_row, h->elim_col, h->elim_val, h->land, h->gr, h->adj_x, h->adj_v,
                    h->gE,       h->lam,      h->mu,       h->dJdg,    h->sums, h->hist.tet, h->hist.vx,
                    h->hist.vy,  h->hist.vz,  h->tri_scratch, h->ctr_scratch,
                    h->q,        h->partials, h->sc,       h->tri_count, h->ctr,      h->n_alive_dev, h->sort_scratch, h->walkq_n,
                    h->io,       h->seg_rq,   h->seg_qn};
    for (void *ptr : ptrs) cudaFree(ptr);
    for (EventSeries *s : {&h->ev_step, &h->ev_dep, &h->ev_pcg, &h->ev_ef, &h->ev_sort}) ev_destroy(*s);
    for (void *ptr : h->amg_alloc) cudaFree(ptr);
    free_tracks(h);
    if (h->pcg_graph) cudaGraphExecDestroy(h->pcg_graph);
    if (h->pcg32_graph) cudaGraphExecDestroy(h->pcg32_graph);
    if (h->pcg_while) cudaGraphExecDestroy(h->pcg_while);
    if (h->solve_rec) cudaFreeHost(h->solve_rec);
    if (h->pcg64_while) cudaGraphExecDestroy(h->pcg64_while);
    for (auto &P : h->ckpt)
        for (void *q : {(void *)P.x, (void *)P.y, (void *)P.z, (void *)P.vx, (void *)P.vy, (void *)P.vz,
                        (void *)P.tet, (void *)P.idf})
            cudaFree(q);
    for (auto &P : h->ckpt32)
        for (void *q : {(void *)P.x, (void *)P.y, (void *)P.z, (void *)P.vx, (void *)P.vy, (void *)P.vz,
                        (void *)P.tet, (void *)P.idf})
            cudaFree(q);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return SPG_OK;
}

int spg_mesh_info(const spg_handle *h, int64_t info[6]) {
    if (!h || !info) return SPG_E_INVALID;
    info[0] = h->n_nodes;
    info[1] = h->n_tets;
    info[2] = h->n_tris;
    info[3] = h->n_boundary_faces;
    info[4] = h->nnz;
    info[5] = h->n_dirichlet;
    return SPG_OK;
}

int spg_set_particles(spg_handle *h, int64_t n, const double *pos, const double *vel, const int32_t *tet_or_null) {
    if (!h) return SPG_E_INVALID;
    if (n < 0 || n > kMaxParticles) return fail(h, SPG_E_INVALID, "set_particles: n out of range");
    if (n > 0 && (!pos || !vel)) return fail(h, SPG_E_INVALID, "set_particles: null pos/vel");
    CK(cudaSetDevice(h->device));
    h->phi_hist = 0;  // a new state: the next run solve starts from phi itself
    free_tracks(h);  // a new particle set ends any tracking
    cudaStream_t s = h->stream;
    {
        const int rc = alloc_particles(h, n);
        if (rc) return rc;
    }
    h->cur = 0;
    h->np = n;
    h->n_active = n;
    h->init_lost = 0;
    h->occupied = 0;
    const double *rpos = (n > 0 && !tet_or_null) ? static_cast<const double *>(device_readable(h, pos)) : nullptr;
    const double *rvel = rpos ? static_cast<const double *>(device_readable(h, vel)) : nullptr;
    if (rpos && rvel) {
        // the caller's arrays are device-readable: one kernel reads them where
        // they lie, locates each particle and writes the state, so the transfer
        // overlaps the location walks
        if (!h->io_counter) CK(dalloc(&h->io_counter, 2));
        CK(cudaMemsetAsync(h->io_counter, 0, sizeof(unsigned long long), s));
        launch_upload(rpos, rvel, n, mesh_dev(h), h->vox_seed, h->vox_oi, h->vox_dims, h->prm.max_crossings,
                      h->P[0], h->Q[0], h->mixed ? h->cen : nullptr, h->io_counter, s);
        CK(cudaGetLastError());
        unsigned long long lost = 0;
        CK(cudaMemcpyAsync(&lost, h->io_counter, sizeof(lost), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        h->init_lost = int64_t(lost);
    } else if (n > 0) {
        IoStage st;
        {
            const int rc = io_stage(h, n, st);
            if (rc) return rc;
        }
        double *dpos = st.pos, *dvel = st.vel;
        int32_t *dtet = st.tet;
        unsigned long long *dlost = st.counter;
        CK(cudaMemcpyAsync(dpos, pos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dvel, vel, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
        if (tet_or_null) {
            std::vector<int32_t> t(tet_or_null, tet_or_null + n);
            for (auto &v : t)
                if (v >= h->n_tets) v = -1;
            CK(cudaMemcpyAsync(dtet, t.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
            CK(cudaStreamSynchronize(s));
        } else {
            launch_locate(dpos, n, mesh_dev(h), h->vox_seed, h->vox_oi, h->vox_dims, h->prm.max_crossings, dtet, s);
        }
        CK(cudaMemsetAsync(dlost, 0, sizeof(unsigned long long), s));
        launch_count_lost(dtet, n, dlost, s);
        if (h->mixed)
            launch_to_local(dpos, dvel, dtet, h->cen, n, h->Q[0], s);
        else
            launch_init_particles(dpos, dvel, dtet, n, h->P[0], s);
        CK(cudaGetLastError());
        unsigned long long lost = 0;
        CK(cudaMemcpyAsync(&lost, dlost, sizeof(lost), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        h->init_lost = int64_t(lost);
    }
    h->have_particles = true;
    h->fix_bits = fix_bits_for(n);
    return reset_run_state(h);
}

void spg_default_source(spg_source *src) {
    if (!src) return;
    std::memset(src, 0, sizeof(*src));
    src->shape = SPG_SRC_DISK;
    src->directions = SPG_DIR_CONE;
    src->energy = SPG_ENERGY_MONO;
    src->normal[2] = 1.0;
    src->radius = 0.02;
    src->half_angle = 30.0 * 3.14159265358979323846 / 180.0;
    src->energy_ev = 1.0;
    src->binding_ev = 4.9;
    src->emax_ev = 50.0;
    src->displacement = 0.05e-3;
}

namespace {
// ParticleDisplacer::_calculateDisplacement (src/Particle/ParticleDisplacer.cpp:20-35):
// dir / max|dir_k| * amount, zero for a direction below machine epsilon.
void fan_shift(const double dir[3], double amount, double out[3]) {
    const double m = std::max(std::fabs(dir[0]), std::max(std::fabs(dir[1]), std::fabs(dir[2])));
    for (int k = 0; k < 3; ++k) out[k] = m < 2.220446049250313e-16 ? 0.0 : (dir[k] / m) * amount;
}
}  // namespace

// Validates src and samples n particles with ids id_base .. id_base + n - 1
// into the device arrays pos, vel (3 n each); tet (n) receives their tets.
int sample_particles(spg_handle *h, int64_t n, const spg_source *src, int64_t id_base, double *dpos, double *dvel,
                     int32_t *dtet, const char *who) {
    const std::string w(who);
    if (!src) return fail(h, SPG_E_INVALID, w + ": null source");
    if (src->shape < SPG_SRC_DISK || src->shape > SPG_SRC_CELLS) return fail(h, SPG_E_INVALID, w + ": bad shape");
    if (src->directions < SPG_DIR_CONE || src->directions > SPG_DIR_FAN)
        return fail(h, SPG_E_INVALID, w + ": bad directions");
    if (src->energy != SPG_ENERGY_MONO && src->energy != SPG_ENERGY_THOMPSON)
        return fail(h, SPG_E_INVALID, w + ": bad energy law");
    const double eV = 1.60217733000001e-19;  // Constants.hpp eV_J
    if (src->energy == SPG_ENERGY_MONO ? !(src->energy_ev > 0.0) : !(src->binding_ev > 0.0 && src->emax_ev > 0.0))
        return fail(h, SPG_E_INVALID, w + ": energies must be > 0");
    if (src->shape == SPG_SRC_CELLS && (src->n_cells <= 0 || !src->cells))
        return fail(h, SPG_E_INVALID, w + ": a cell source needs n_cells > 0 and cells");
    if (src->directions == SPG_DIR_FAN && !(src->expansion >= 0.0))
        return fail(h, SPG_E_INVALID, w + ": expansion must be >= 0");
    SourceConst c{};
    c.shape = src->shape;
    c.directions = src->directions;
    c.energy = src->energy;
    // frame about the normal (rectangles emit about +z)
    double nv[3] = {src->normal[0], src->normal[1], src->normal[2]};
    if (src->shape == SPG_SRC_RECT) nv[0] = nv[1] = 0.0, nv[2] = 1.0;
    const double nn = std::sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
    if (src->shape != SPG_SRC_CELLS && !(nn > 0.0)) return fail(h, SPG_E_INVALID, w + ": zero normal");
    if (nn > 0.0)
        for (double &x : nv) x /= nn;
    else
        nv[0] = nv[1] = 0.0, nv[2] = 1.0;
    const double t[3] = {std::fabs(nv[0]) < 0.9 ? 1.0 : 0.0, std::fabs(nv[0]) < 0.9 ? 0.0 : 1.0, 0.0};
    double e1[3] = {nv[1] * t[2] - nv[2] * t[1], nv[2] * t[0] - nv[0] * t[2], nv[0] * t[1] - nv[1] * t[0]};
    const double l1 = std::sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
    for (double &x : e1) x /= l1;
    const double e2[3] = {nv[1] * e1[2] - nv[2] * e1[1], nv[2] * e1[0] - nv[0] * e1[2], nv[0] * e1[1] - nv[1] * e1[0]};
    for (int k = 0; k < 3; ++k) {
        c.centre[k] = src->centre[k];
        c.e1[k] = e1[k];
        c.e2[k] = e2[k];
        c.nrm[k] = nv[k];
    }
    c.theta0 = std::acos(std::max(-1.0, std::min(1.0, nv[2])));
    c.phi0 = std::atan2(nv[1], nv[0]);
    c.expansion = src->expansion;
    {
        // ParticleDisplacer::displaceParticlesFromPointSources
        // (src/Particle/ParticleDisplacer.cpp:48-87, :20-35): one shift per
        // source, along its direction (theta, phi), scaled so that its largest
        // component is the displacement
        const double st = std::sin(c.theta0);
        const double dir[3] = {st * std::cos(c.phi0), st * std::sin(c.phi0), std::cos(c.theta0)};
        fan_shift(dir, src->displacement, c.fan_shift);
    }
    c.radius = src->radius;
    c.xlim[0] = src->xlim[0];
    c.xlim[1] = src->xlim[1];
    c.ylim[0] = src->ylim[0];
    c.ylim[1] = src->ylim[1];
    c.z = src->z;
    c.one_minus_cos = 1.0 - std::cos(src->half_angle);
    c.mass = h->prm.mass;
    c.speed_mono = std::sqrt(2.0 * src->energy_ev * eV / h->prm.mass);
    c.binding_j = src->binding_ev * eV;
    c.s_max = src->emax_ev / (src->emax_ev + src->binding_ev);
    c.displacement = src->displacement;
    c.seed_lo = uint32_t(src->seed);
    c.seed_hi = uint32_t(src->seed >> 32);
    c.id_base = id_base;
    cudaStream_t s = h->stream;
    double *dcells = nullptr;
    int64_t *dfirst = nullptr;
    if (src->shape == SPG_SRC_CELLS) {
        // per cell: centre and the polar / azimuthal angle of its normal; the
        // count splits evenly and the remainder goes one each to cells chosen
        // by a shuffle seeded from the source seed and the first id
        const int k = src->n_cells;
        std::vector<double> cells(8 * size_t(k));
        for (int q = 0; q < k; ++q) {
            const double *cc = src->cells + 6 * size_t(q);
            const double m = std::sqrt(cc[3] * cc[3] + cc[4] * cc[4] + cc[5] * cc[5]);
            if (!(m > 0.0)) return fail(h, SPG_E_INVALID, w + ": zero cell normal");
            double *o = cells.data() + 8 * size_t(q);
            o[0] = cc[0];
            o[1] = cc[1];
            o[2] = cc[2];
            o[3] = std::acos(std::max(-1.0, std::min(1.0, cc[5] / m)));
            o[4] = std::atan2(cc[4] / m, cc[3] / m);
            // displaceParticlesFromSurfaceSources (ParticleDisplacer.cpp:90-133):
            // the cell's normal as given, scaled to the displacement
            fan_shift(cc + 3, src->displacement, o + 5);
        }
        std::vector<int64_t> count(k, n / k);
        std::vector<int> order(k);
        for (int q = 0; q < k; ++q) order[q] = q;
        std::mt19937_64 gen(src->seed ^ (uint64_t(id_base) * 0x9E3779B97F4A7C15ull));
        std::shuffle(order.begin(), order.end(), gen);
        for (int64_t q = 0; q < n % k; ++q) count[order[q]]++;
        std::vector<int64_t> first(k + 1, 0);
        for (int q = 0; q < k; ++q) first[q + 1] = first[q] + count[q];
        CK(upload(&dcells, cells, s));
        CK(upload(&dfirst, first, s));
        c.n_cells = k;
        c.cells = dcells;
        c.cell_first = dfirst;
    }
    launch_generate(c, n, dpos, dvel, s);
    launch_locate(dpos, n, mesh_dev(h), h->vox_seed, h->vox_oi, h->vox_dims, h->prm.max_crossings, dtet, s);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s));
    cudaFree(dcells);
    cudaFree(dfirst);
    return SPG_OK;
}

int spg_generate_particles(spg_handle *h, int64_t n, const spg_source *src) {
    if (!h) return SPG_E_INVALID;
    if (n < 0 || n > kMaxParticles) return fail(h, SPG_E_INVALID, "generate_particles: n out of range");
    CK(cudaSetDevice(h->device));
    h->phi_hist = 0;  // a new state: the next run solve starts from phi itself
    free_tracks(h);   // a new particle set ends any tracking
    cudaStream_t s = h->stream;
    {
        const int rc = alloc_particles(h, n);
        if (rc) return rc;
    }
    h->cur = 0;
    h->np = n;
    h->n_active = n;
    h->init_lost = 0;
    h->occupied = 0;
    if (n > 0) {
        IoStage st;
        int rc = io_stage(h, n, st);
        if (!rc) rc = sample_particles(h, n, src, 0, st.pos, st.vel, st.tet, "generate_particles");
        if (rc) {
            h->np = h->n_active = 0;
            return rc;
        }
        double *dpos = st.pos, *dvel = st.vel;
        int32_t *dtet = st.tet;
        unsigned long long *dlost = st.counter;
        CK(cudaMemsetAsync(dlost, 0, sizeof(unsigned long long), s));
        launch_count_lost(dtet, n, dlost, s);
        if (h->mixed)
            launch_to_local(dpos, dvel, dtet, h->cen, n, h->Q[0], s);
        else
            launch_init_particles(dpos, dvel, dtet, n, h->P[0], s);
        CK(cudaGetLastError());
        unsigned long long lost = 0;
        CK(cudaMemcpyAsync(&lost, dlost, sizeof(lost), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        h->init_lost = int64_t(lost);
    }
    h->have_particles = true;
    h->fix_bits = fix_bits_for(n);
    return reset_run_state(h);
}

int spg_inject_particles(spg_handle *h, int64_t n, const spg_source *src) {
    if (!h) return SPG_E_INVALID;
    if (!h->have_particles) return fail(h, SPG_E_STATE, "inject_particles: no particles set");
    if (n < 0 || h->np + n > kMaxParticles) return fail(h, SPG_E_INVALID, "inject_particles: n out of range");
    if (n == 0) return SPG_OK;
    CK(cudaSetDevice(h->device));
    h->occ_fresh = false;  // the new particles' tets are not on the deposit's list
    cudaStream_t s = h->stream;
    IoStage st;
    int rc = io_stage(h, n, st);
    if (!rc) rc = sample_particles(h, n, src, h->np, st.pos, st.vel, st.tet, "inject_particles");
    if (!rc) rc = grow_particles(h, h->np + n);
    if (rc) return rc;
    double *dpos = st.pos, *dvel = st.vel;
    int32_t *dtet = st.tet;
    unsigned long long *dlost = st.counter;
    CK(cudaMemsetAsync(dlost, 0, sizeof(unsigned long long), s));
    launch_count_lost(dtet, n, dlost, s);
    if (h->mixed)
        launch_to_local(dpos, dvel, dtet, h->cen, n, h->Q[h->cur], s, h->np);
    else
        launch_init_particles(dpos, dvel, dtet, n, h->P[h->cur], s, h->np);
    CK(cudaGetLastError());
    unsigned long long lost = 0;
    CK(cudaMemcpyAsync(&lost, dlost, sizeof(lost), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    h->grad_ready = false;  // the recorded gradient forward no longer matches the particle set
    // the new particles come after the active range; every slot up to np is processed
    h->np += n;
    h->n_active = h->np;
    h->init_lost += int64_t(lost);
    h->fix_bits = fix_bits_for(h->np);
    // their tets get the current field (the lazy field computes occupied tets only)
    const FieldArgs f = field_args(h);
    if (h->mixed)
        launch_refresh32(h->Q[h->cur], h->np, f, s);
    else
        launch_refresh64(h->P[h->cur], h->np, f, s);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s));
    return SPG_OK;
}

int spg_track_particles(spg_handle *h, int32_t k, const int64_t *ids, int32_t capacity) {
    if (!h) return SPG_E_INVALID;
    if (!h->have_particles) return fail(h, SPG_E_STATE, "track_particles: no particles set");
    if (k < 0 || (k > 0 && (!ids || capacity < 1))) return fail(h, SPG_E_INVALID, "track_particles: bad arguments");
    for (int32_t t = 0; t < k; ++t)
        if (ids[t] < 0 || ids[t] >= h->np) return fail(h, SPG_E_INVALID, "track_particles: id out of range");
    CK(cudaSetDevice(h->device));
    free_tracks(h);
    if (k == 0) return SPG_OK;
    cudaStream_t s = h->stream;
    CK(dalloc(&h->track_ids, k));
    CK(dalloc(&h->track_of_id, std::max<int64_t>(h->np, 1)));
    h->track_table_n = std::max<int64_t>(h->np, 1);
    CK(dalloc(&h->track_slot, k));
    CK(dalloc(&h->track_count, k));
    CK(dalloc(&h->track_xyz, 3 * int64_t(k) * capacity));
    CK(dalloc(&h->track_cur, 3 * int64_t(k)));
    CK(dalloc(&h->track_flags, k));
    CK(cudaMemcpyAsync(h->track_ids, ids, sizeof(int64_t) * k, cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(h->track_of_id, 0xff, sizeof(int32_t) * std::max<int64_t>(h->np, 1), s));
    CK(cudaMemsetAsync(h->track_slot, 0xff, sizeof(int32_t) * k, s));
    CK(cudaMemsetAsync(h->track_count, 0, sizeof(int32_t) * k, s));
    launch_track_map(h->track_ids, k, h->track_of_id, s);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s));
    h->track_k = k;
    h->track_cap = capacity;
    return SPG_OK;
}

int spg_get_tracks(spg_handle *h, int32_t *counts, double *xyz, double *last_xyz, uint32_t *last_flags) {
    if (!h) return SPG_E_INVALID;
    if (h->track_k == 0) return fail(h, SPG_E_STATE, "get_tracks: no particles tracked");
    CK(cudaSetDevice(h->device));
    cudaStream_t s = h->stream;
    const int k = h->track_k;
    const uint32_t *idf = h->mixed ? h->Q[h->cur].idf : h->P[h->cur].idf;
    launch_track_find(idf, h->np, h->track_of_id, h->track_table_n, h->track_slot, s);
    if (h->mixed)
        launch_track_current32(h->Q[h->cur], h->cen, h->track_slot, k, h->track_cur, h->track_flags, s);
    else
        launch_track_current64(h->P[h->cur], h->track_slot, k, h->track_cur, h->track_flags, s);
    CK(cudaGetLastError());
    if (counts) CK(cudaMemcpyAsync(counts, h->track_count, sizeof(int32_t) * k, cudaMemcpyDeviceToHost, s));
    if (xyz)
        CK(cudaMemcpyAsync(xyz, h->track_xyz, sizeof(double) * 3 * int64_t(k) * h->track_cap, cudaMemcpyDeviceToHost,
                           s));
    if (last_xyz) CK(cudaMemcpyAsync(last_xyz, h->track_cur, sizeof(double) * 3 * k, cudaMemcpyDeviceToHost, s));
    if (last_flags) CK(cudaMemcpyAsync(last_flags, h->track_flags, sizeof(uint32_t) * k, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return SPG_OK;
}

int spg_get_particles(spg_handle *h, int64_t n, double *pos, double *vel, int32_t *tet, uint32_t *flags) {
    if (!h) return SPG_E_INVALID;
    if (!h->have_particles) return fail(h, SPG_E_STATE, "get_particles: no particles set");
    if (n != h->np) return fail(h, SPG_E_INVALID, "get_particles: n does not match the particle count");
    if (n == 0) return SPG_OK;
    CK(cudaSetDevice(h->device));
    cudaStream_t s = h->stream;
    {
        // pinned or managed caller arrays: the gather writes them directly
        void *wp = pos ? device_writable(pos) : nullptr, *wv = vel ? device_writable(vel) : nullptr;
        void *wt = tet ? device_writable(tet) : nullptr, *wf = flags ? device_writable(flags) : nullptr;
        if ((!pos || wp) && (!vel || wv) && (!tet || wt) && (!flags || wf)) {
            if (n > h->id_slot_cap) {
                cudaFree(h->id_slot);
                h->id_slot = nullptr;
                h->id_slot_cap = 0;
                CK(dalloc(&h->id_slot, n));
                h->id_slot_cap = n;
            }
            double *dp = static_cast<double *>(wp), *dv = static_cast<double *>(wv);
            int32_t *dt = static_cast<int32_t *>(wt);
            uint32_t *df = static_cast<uint32_t *>(wf);
            if (h->mixed)
                launch_gather32(h->Q[h->cur], n, h->id_slot, h->cen, dp, dv, dt, df, s);
            else
                launch_gather_by_id(h->P[h->cur], n, h->id_slot, dp, dv, dt, df, s);
            CK(cudaGetLastError());
            CK(cudaStreamSynchronize(s));
            return SPG_OK;
        }
    }
    IoStage st;
    {
        const int rc = io_stage(h, n, st);
        if (rc) return rc;
    }
    double *dpos = pos ? st.pos : nullptr, *dvel = vel ? st.vel : nullptr;
    int32_t *dtet = tet ? st.tet : nullptr;
    uint32_t *dfl = flags ? st.flags : nullptr;
    if (h->mixed)
        launch_gather32(h->Q[h->cur], n, st.slot, h->cen, dpos, dvel, dtet, dfl, s);
    else
        launch_gather_by_id(h->P[h->cur], n, st.slot, dpos, dvel, dtet, dfl, s);
    CK(cudaGetLastError());
    if (pos) CK(cudaMemcpyAsync(pos, dpos, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
    if (vel) CK(cudaMemcpyAsync(vel, dvel, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
    if (tet) CK(cudaMemcpyAsync(tet, dtet, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
    if (flags) CK(cudaMemcpyAsync(flags, dfl, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return SPG_OK;
}

namespace {
// The periodic re-sort by tet, at the steps that are multiples of
// resort_every, once per step, by whichever call comes first in that step
// (spg_run, spg_gather or spg_process). It changes only the memory order.
int maybe_resort(spg_handle *h) {
    if (h->prm.resort_every <= 0 || h->step % h->prm.resort_every != 0 || h->resorted_at == h->step) return SPG_OK;
    h->resorted_at = h->step;
    return do_resort(h);
}

// Solve of the deposit just made from this handle's particles: AMG starts
// from the extrapolation of the last such solves, and the field is computed
// for the occupied tets only (the walks compute the tets particles enter).
int solve_run_deposit(spg_handle *h) {
    if (h->amg || h->amg32) {
        launch_extrapolate(h->phi, h->phi_prev, h->phi_prev2, h->n_nodes, std::min(kExtrapOrder, h->phi_hist - 1),
                           h->stream);
        h->launches += 1;
        h->phi_hist++;
    }
    const bool prev = h->in_run;
    h->in_run = true;
    const int rc = do_solve(h);
    h->in_run = prev;
    return rc;
}
}  // namespace

int spg_gather(spg_handle *h, double *rho_out) {
    if (!h) return SPG_E_INVALID;
    CK(cudaSetDevice(h->device));
    int rc = h->have_particles ? maybe_resort(h) : SPG_OK;
    if (rc) return rc;
    rc = do_gather(h);
    if (rc) return rc;
    if (rho_out) {
        launch_node_rho(h->node_q, h->dual_vol, h->rho, h->n_nodes, h->stream);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(rho_out, h->rho, sizeof(double) * h->n_nodes, cudaMemcpyDeviceToHost, h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));
    return SPG_OK;
}

int spg_get_charge_density(spg_handle *h, double *rho_out) {
    if (!h || !rho_out) return SPG_E_INVALID;
    if (!h->charge_valid) return fail(h, SPG_E_STATE, "get_charge_density: no deposit or given density yet");
    CK(cudaSetDevice(h->device));
    launch_node_rho(h->node_q, h->dual_vol, h->rho, h->n_nodes, h->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(rho_out, h->rho, sizeof(double) * h->n_nodes, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return SPG_OK;
}

int spg_solve(spg_handle *h, const double *rho_or_null, double *phi_out, int32_t *iters, double *relres) {
    if (!h) return SPG_E_INVALID;
    CK(cudaSetDevice(h->device));
    int rc;
    if (!rho_or_null && h->occ_fresh) {
        // The solve of this handle's own deposit, with no particle moved since
        // (the gather -> solve of the reference's time loop): the same solve
        // spg_run makes, with the extrapolated initial guess and the field of
        // the occupied tets only.
        rc = solve_run_deposit(h);
    } else {
        h->phi_hist = 0;  // a new state: the next run solve starts from phi itself
        if (rho_or_null) {
            // the density goes up once; the node charges are formed on the device
            CK(cudaMemcpyAsync(h->rho, rho_or_null, sizeof(double) * h->n_nodes, cudaMemcpyHostToDevice,
                               h->stream));
            launch_node_q_from_rho(h->rho, h->dual_vol, h->node_q, h->n_nodes, h->stream);
            CK(cudaGetLastError());
            h->charge_valid = true;
        }
        // while the deposit's list of occupied tets still holds every
        // particle, the field of those tets is enough (the walks compute the
        // tets particles enter)
        const bool prev = h->in_run;
        h->in_run = h->occ_fresh;
        rc = do_solve(h);
        h->in_run = prev;
    }
    if (iters) *iters = h->cg_iters_last;
    if (relres) *relres = h->cg_relres_last;
    if (rc && rc != SPG_E_NOT_CONVERGED) return rc;
    if (phi_out) {
        CK(cudaMemcpyAsync(phi_out, h->phi, sizeof(double) * h->n_nodes, cudaMemcpyDeviceToHost, h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));
    return rc;
}

int spg_process(spg_handle *h, int32_t nsteps, spg_stats *stats) {
    if (!h) return SPG_E_INVALID;
    if (!h->have_particles) return fail(h, SPG_E_STATE, "process: no particles set");
    if (nsteps < 0) return fail(h, SPG_E_INVALID, "process: nsteps < 0");
    CK(cudaSetDevice(h->device));
    for (int32_t k = 0; k < nsteps;) {
        int rc = maybe_resort(h);
        if (rc) return rc;
        const int l = steps_to_event(h, nsteps - k, false);
        rc = do_steps(h, l);
        if (rc) return rc;
        k += l;
    }
    return fill_stats(h, stats);
}

int spg_run(spg_handle *h, int32_t nsteps, spg_stats *stats) {
    if (!h) return SPG_E_INVALID;
    if (!h->have_particles) return fail(h, SPG_E_STATE, "run: no particles set");
    if (nsteps < 0) return fail(h, SPG_E_INVALID, "run: nsteps < 0");
    CK(cudaSetDevice(h->device));
    struct InRun {  // solves of the run refresh the occupied tets only and do not wait for the host
        spg_handle *h;
        explicit InRun(spg_handle *hh) : h(hh) {
            h->in_run = true;
            h->defer_solves = true;
            h->deferred_capped = false;
        }
        ~InRun() {
            h->in_run = false;
            h->defer_solves = false;
            if (h->n_solve_rec) {  // an early (error) return: keep its message
                const std::string err = h->err;
                drain_solves(h);
                h->err = err;
            }
        }
    } in_run(h);
    int status = SPG_OK;
    for (int32_t k = 0; k < nsteps;) {
        int rc = maybe_resort(h);
        if (rc) return rc;
        if (h->step % h->prm.poisson_every == 0) {
            rc = do_gather(h);
            if (rc) return rc;
            rc = solve_run_deposit(h);
            if (rc == SPG_E_NOT_CONVERGED)
                status = rc;
            else if (rc)
                return rc;
        }
        const int l = steps_to_event(h, nsteps - k, true);
        rc = do_steps(h, l);
        if (rc) return rc;
        k += l;
    }
    int rc = drain_solves(h);
    if (rc) return rc;
    if (h->deferred_capped) status = SPG_E_NOT_CONVERGED;
    rc = fill_stats(h, stats);
    return rc ? rc : status;
}

int spg_resort(spg_handle *h) {
    if (!h) return SPG_E_INVALID;
    CK(cudaSetDevice(h->device));
    return do_resort(h);
}

int spg_get_stats(spg_handle *h, spg_stats *stats) {
    if (!h || !stats) return SPG_E_INVALID;
    CK(cudaSetDevice(h->device));
    return fill_stats(h, stats);
}

int spg_get_triangle_counts(spg_handle *h, uint64_t *counts) {
    if (!h || (!counts && h->n_tris > 0)) return SPG_E_INVALID;
    if (h->n_tris == 0) return SPG_OK;
    CK(cudaSetDevice(h->device));
    std::vector<unsigned int> c(h->n_tris);
    CK(cudaMemcpyAsync(c.data(), h->tri_count, sizeof(unsigned int) * h->n_tris, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (int64_t k = 0; k < h->n_tris; ++k) counts[k] = c[k];
    return SPG_OK;
}

int spg_get_potential(spg_handle *h, double *phi) {
    if (!h || !phi) return SPG_E_INVALID;
    CK(cudaSetDevice(h->device));
    CK(cudaMemcpyAsync(phi, h->phi, sizeof(double) * h->n_nodes, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return SPG_OK;
}

int spg_set_potential(spg_handle *h, const double *phi) {
    if (!h || !phi) return SPG_E_INVALID;
    CK(cudaSetDevice(h->device));
    h->phi_hist = 0;  // a new state: the next run solve starts from phi itself
    CK(cudaMemcpyAsync(h->phi, phi, sizeof(double) * h->n_nodes, cudaMemcpyHostToDevice, h->stream));
    {
        const int rc = update_field(h, false);
        if (rc) return rc;
    }
    CK(cudaStreamSynchronize(h->stream));
    return SPG_OK;
}

int spg_get_efield(spg_handle *h, double *E) {
    if (!h || !E) return SPG_E_INVALID;
    CK(cudaSetDevice(h->device));
    if (!h->field_full) {  // the last run solve computed the occupied tets only: complete the field
        const FieldArgs f = field_args(h);
        if (h->mixed)
            launch_field32_full(f, h->n_tets, h->stream);
        else
            launch_field64_full(f, h->n_tets, h->stream);
        CK(cudaGetLastError());
        h->field_full = true;
    }
    CK(cudaMemcpyAsync(E, h->efield, sizeof(double) * 3 * h->n_tets, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return SPG_OK;
}

int spg_get_matrix(spg_handle *h, int32_t *row_ptr, int32_t *col, double *val, double *lift, double *dual_vol) {
    if (!h) return SPG_E_INVALID;
    CK(cudaSetDevice(h->device));
    cudaStream_t s = h->stream;
    const int64_t n = h->n_nodes;
    int32_t nnz = 0;
    CK(cudaMemcpyAsync(&nnz, h->row_ptr + n, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (row_ptr) CK(cudaMemcpyAsync(row_ptr, h->row_ptr, sizeof(int32_t) * (n + 1), cudaMemcpyDeviceToHost, s));
    if (col) CK(cudaMemcpyAsync(col, h->col, sizeof(int32_t) * size_t(nnz), cudaMemcpyDeviceToHost, s));
    if (val) CK(cudaMemcpyAsync(val, h->val, sizeof(double) * size_t(nnz), cudaMemcpyDeviceToHost, s));
    if (lift) CK(cudaMemcpyAsync(lift, h->lift, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    if (dual_vol) CK(cudaMemcpyAsync(dual_vol, h->dual_vol, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return SPG_OK;
}

int spg_locate(spg_handle *h, int64_t n, const double *pos, int32_t *tet_out) {
    if (!h || n < 0 || (n > 0 && (!pos || !tet_out))) return SPG_E_INVALID;
    if (n == 0) return SPG_OK;
    CK(cudaSetDevice(h->device));
    IoStage st;
    {
        const int rc = io_stage(h, n, st);
        if (rc) return rc;
    }
    double *dpos = st.pos;
    int32_t *dtet = st.tet;
    CK(cudaMemcpyAsync(dpos, pos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, h->stream));
    launch_locate(dpos, n, mesh_dev(h), h->vox_seed, h->vox_oi, h->vox_dims, h->prm.max_crossings, dtet, h->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(tet_out, dtet, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return SPG_OK;
}

// Checkpoint layout: header, 8 particle arrays (current order; positions and
// velocities are 8 B in the FP64 form, 4 B in the mixed form), phi, triangle
// counters, device counters.
namespace {
struct CkptHeader {
    uint64_t magic, version;
    int64_t np, n_active, step, n_nodes, n_tris, init_lost, occupied;
    int64_t cg_iters_total;
    int32_t cg_iters_last, cg_solves;
    double cg_relres_last;
    int32_t precision, phi_hist;
};
constexpr uint64_t kMagic = 0x5350474B50543032ull;  // "SPGKPT02"
size_t particle_bytes(const spg_handle *h) { return h->mixed ? 32 : 56; }
size_t ckpt_bytes_for(const spg_handle *h, int64_t np) {
    return sizeof(CkptHeader) + size_t(np) * particle_bytes(h) + size_t(h->n_nodes) * 24 + size_t(h->n_tris) * 4 +
           sizeof(DevCounters);
}
size_t ckpt_bytes(const spg_handle *h) { return ckpt_bytes_for(h, h->np); }
// The 8 particle arrays of buffer `which` with their element sizes.
void particle_arrays(spg_handle *h, int which, void *ptr[8], size_t sz[8]) {
    if (h->mixed) {
        const DevParticles32 &Q = h->Q[which];
        void *a[8] = {Q.x, Q.y, Q.z, Q.vx, Q.vy, Q.vz, Q.tet, Q.idf};
        for (int k = 0; k < 8; ++k) ptr[k] = a[k];
    } else {
        const DevParticles &P = h->P[which];
        void *a[8] = {P.x, P.y, P.z, P.vx, P.vy, P.vz, P.tet, P.idf};
        for (int k = 0; k < 8; ++k) ptr[k] = a[k];
    }
    for (int k = 0; k < 6; ++k) sz[k] = h->mixed ? 4 : 8;
    sz[6] = sz[7] = 4;
}
}  // namespace

int spg_checkpoint_size(spg_handle *h, size_t *bytes) {
    if (!h || !bytes) return SPG_E_INVALID;
    *bytes = ckpt_bytes(h);
    return SPG_OK;
}

int spg_checkpoint(spg_handle *h, void *buf, size_t bytes) {
    if (!h || !buf) return SPG_E_INVALID;
    if (!h->have_particles) return fail(h, SPG_E_STATE, "checkpoint: no particles set");
    if (bytes < ckpt_bytes(h)) return fail(h, SPG_E_INVALID, "checkpoint: buffer too small");
    CK(cudaSetDevice(h->device));
    CkptHeader hd{};
    hd.magic = kMagic;
    hd.version = 3;
    hd.np = h->np;
    hd.n_active = h->n_active;
    hd.step = h->step;
    hd.n_nodes = h->n_nodes;
    hd.n_tris = h->n_tris;
    hd.init_lost = h->init_lost;
    hd.occupied = h->occupied;
    hd.cg_iters_total = h->cg_iters_total;
    hd.cg_iters_last = h->cg_iters_last;
    hd.cg_solves = h->cg_solves;
    hd.cg_relres_last = h->cg_relres_last;
    hd.precision = h->prm.precision;
    hd.phi_hist = h->phi_hist;
    char *o = static_cast<char *>(buf);
    std::memcpy(o, &hd, sizeof(hd));
    o += sizeof(hd);
    const int64_t n = h->np;
    cudaStream_t s = h->stream;
    void *arr[8];
    size_t sz[8];
    particle_arrays(h, h->cur, arr, sz);
    for (int k = 0; k < 8; ++k) {
        if (n) CK(cudaMemcpyAsync(o, arr[k], sz[k] * n, cudaMemcpyDeviceToHost, s));
        o += sz[k] * n;
    }
    CK(cudaMemcpyAsync(o, h->phi, 8 * h->n_nodes, cudaMemcpyDeviceToHost, s));
    o += 8 * h->n_nodes;
    CK(cudaMemcpyAsync(o, h->phi_prev, 8 * h->n_nodes, cudaMemcpyDeviceToHost, s));
    o += 8 * h->n_nodes;
    CK(cudaMemcpyAsync(o, h->phi_prev2, 8 * h->n_nodes, cudaMemcpyDeviceToHost, s));
    o += 8 * h->n_nodes;
    if (h->n_tris) CK(cudaMemcpyAsync(o, h->tri_count, 4 * h->n_tris, cudaMemcpyDeviceToHost, s));
    o += 4 * h->n_tris;
    CK(cudaMemcpyAsync(o, h->ctr, sizeof(DevCounters), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return SPG_OK;
}

int spg_restore(spg_handle *h, const void *buf, size_t bytes) {
    if (!h || !buf) return SPG_E_INVALID;
    if (bytes < sizeof(CkptHeader)) return fail(h, SPG_E_INVALID, "restore: buffer too small");
    CkptHeader hd;
    std::memcpy(&hd, buf, sizeof(hd));
    if (hd.magic != kMagic || hd.version != 3) return fail(h, SPG_E_INVALID, "restore: not a checkpoint");
    if (hd.n_nodes != h->n_nodes || hd.n_tris != h->n_tris)
        return fail(h, SPG_E_INVALID, "restore: checkpoint is for a different mesh");
    if (hd.precision != h->prm.precision)
        return fail(h, SPG_E_INVALID, "restore: checkpoint is for the other precision form");
    if (hd.np < 0 || hd.np > kMaxParticles || hd.n_active < 0 || hd.n_active > hd.np)
        return fail(h, SPG_E_INVALID, "restore: corrupt header");
    const int64_t n = hd.np;
    if (bytes < ckpt_bytes_for(h, n)) return fail(h, SPG_E_INVALID, "restore: buffer too small");
    {
        // The particle downloads address particles through the slot of their
        // id, so a blob whose ids are not a permutation of 0..np-1, or whose
        // tets are out of range, is refused before anything is copied.
        const size_t es = h->mixed ? 4 : 8;
        const char *tp = static_cast<const char *>(buf) + sizeof(hd) + 6 * es * size_t(n);
        const char *ip = tp + 4 * size_t(n);
        std::vector<uint8_t> seen(size_t(n), 0);
        for (int64_t i = 0; i < n; ++i) {
            int32_t t;
            uint32_t idf;
            std::memcpy(&t, tp + 4 * i, 4);
            std::memcpy(&idf, ip + 4 * i, 4);
            const uint32_t id = idf & kIdMask;
            if (t < -1 || t >= h->n_tets || int64_t(id) >= n || seen[id])
                return fail(h, SPG_E_INVALID, "restore: particle ids or tets are corrupt");
            seen[id] = 1;
        }
    }
    CK(cudaSetDevice(h->device));
    free_tracks(h);  // slots and particle count may change
    {
        const int rc = alloc_particles(h, n);
        if (rc) return rc;
    }
    h->cur = 0;
    const char *o = static_cast<const char *>(buf) + sizeof(hd);
    cudaStream_t s = h->stream;
    void *arr[8];
    size_t sz[8];
    particle_arrays(h, 0, arr, sz);
    for (int k = 0; k < 8; ++k) {
        if (n) CK(cudaMemcpyAsync(arr[k], o, sz[k] * n, cudaMemcpyHostToDevice, s));
        o += sz[k] * n;
    }
    CK(cudaMemcpyAsync(h->phi, o, 8 * h->n_nodes, cudaMemcpyHostToDevice, s));
    o += 8 * h->n_nodes;
    CK(cudaMemcpyAsync(h->phi_prev, o, 8 * h->n_nodes, cudaMemcpyHostToDevice, s));
    o += 8 * h->n_nodes;
    CK(cudaMemcpyAsync(h->phi_prev2, o, 8 * h->n_nodes, cudaMemcpyHostToDevice, s));
    o += 8 * h->n_nodes;
    h->phi_hist = hd.phi_hist;
    if (h->n_tris) CK(cudaMemcpyAsync(h->tri_count, o, 4 * h->n_tris, cudaMemcpyHostToDevice, s));
    o += 4 * h->n_tris;
    CK(cudaMemcpyAsync(h->ctr, o, sizeof(DevCounters), cudaMemcpyHostToDevice, s));
    h->np = n;
    h->n_active = hd.n_active;
    h->step = hd.step;
    h->init_lost = hd.init_lost;
    h->occupied = hd.occupied;
    h->cg_iters_total = hd.cg_iters_total;
    h->cg_iters_last = hd.cg_iters_last;
    h->cg_solves = hd.cg_solves;
    h->cg_relres_last = hd.cg_relres_last;
    h->have_particles = true;
    h->occ_fresh = false;
    h->resorted_at = -1;
    if (h->cg_solves == 0) {
        zero_field(h);
    } else {
        const int rc = update_field(h, false);
        if (rc) return rc;
    }
    h->fix_bits = fix_bits_for(h->np);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s));
    return SPG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- gradient
namespace {

template <class T>
int ensure(spg_handle *h, T **ptr, size_t count) {
    if (*ptr) return SPG_OK;
    CK(dalloc(ptr, count));
    return SPG_OK;
}

int copy_particles(spg_handle *h, const DevParticles &dst, const DevParticles &src, int64_t n) {
    if (n == 0) return SPG_OK;
    cudaStream_t s = h->stream;
    CK(cudaMemcpyAsync(dst.x, src.x, 8 * n, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(dst.y, src.y, 8 * n, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(dst.z, src.z, 8 * n, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(dst.vx, src.vx, 8 * n, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(dst.vy, src.vy, 8 * n, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(dst.vz, src.vz, 8 * n, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(dst.tet, src.tet, 4 * n, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(dst.idf, src.idf, 4 * n, cudaMemcpyDeviceToDevice, s));
    return SPG_OK;
}

void free_particle_set(std::vector<DevParticles> &v) {
    for (auto &P : v)
        for (void *q : {(void *)P.x, (void *)P.y, (void *)P.z, (void *)P.vx, (void *)P.vy, (void *)P.vz,
                        (void *)P.tet, (void *)P.idf})
            cudaFree(q);
    v.clear();
}

int alloc_dev_particles(spg_handle *h, DevParticles &P, int64_t n) {
    CK(dalloc(&P.x, n));
    CK(dalloc(&P.y, n));
    CK(dalloc(&P.z, n));
    CK(dalloc(&P.vx, n));
    CK(dalloc(&P.vy, n));
    CK(dalloc(&P.vz, n));
    CK(dalloc(&P.tet, n));
    CK(dalloc(&P.idf, n));
    return SPG_OK;
}

int copy_particles32(spg_handle *h, const DevParticles32 &dst, const DevParticles32 &src, int64_t n) {
    if (n == 0) return SPG_OK;
    cudaStream_t s = h->stream;
    for (int k = 0; k < 6; ++k) {
        float *d = k == 0 ? dst.x : k == 1 ? dst.y : k == 2 ? dst.z : k == 3 ? dst.vx : k == 4 ? dst.vy : dst.vz;
        const float *q = k == 0 ? src.x : k == 1 ? src.y : k == 2 ? src.z : k == 3 ? src.vx : k == 4 ? src.vy : src.vz;
        CK(cudaMemcpyAsync(d, q, 4 * n, cudaMemcpyDeviceToDevice, s));
    }
    CK(cudaMemcpyAsync(dst.tet, src.tet, 4 * n, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(dst.idf, src.idf, 4 * n, cudaMemcpyDeviceToDevice, s));
    return SPG_OK;
}

int alloc_dev_particles32(spg_handle *h, DevParticles32 &P, int64_t n) {
    CK(dalloc(&P.x, n));
    CK(dalloc(&P.y, n));
    CK(dalloc(&P.z, n));
    CK(dalloc(&P.vx, n));
    CK(dalloc(&P.vy, n));
    CK(dalloc(&P.vz, n));
    CK(dalloc(&P.tet, n));
    CK(dalloc(&P.idf, n));
    return SPG_OK;
}

void free_particle_set32(std::vector<DevParticles32> &v) {
    for (auto &P : v)
        for (void *q : {(void *)P.x, (void *)P.y, (void *)P.z, (void *)P.vx, (void *)P.vy, (void *)P.vz,
                        (void *)P.tet, (void *)P.idf})
            cudaFree(q);
    v.clear();
}

// Solves K x = b (b, x device vectors of n_nodes) with the FP64 PCG of spg_solve.
int solve_into(spg_handle *h, double *b, double *x, int32_t *iters) {
    PcgScalars init{};
    init.tol2 = h->prm.cg_rtol * h->prm.cg_rtol;
    init.max_iter = h->prm.cg_max_iter;
    CK(cudaMemcpyAsync(h->sc, &init, sizeof(init), cudaMemcpyHostToDevice, h->stream));
    PcgDev d = pcg_dev(h);
    d.x = x;
    pcg_setup_any(h, d, b);
    PcgScalars hs{};
    for (int chunk = 0;; ++chunk) {
        for (int k = 0; k < pcg_chunk(h); ++k) pcg_iteration_any(h, d);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(&hs, h->sc, sizeof(hs), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        if (hs.converged) break;
    }
    if (iters) *iters = hs.iters;
    if (hs.converged == 2) return fail(h, SPG_E_NOT_CONVERGED, "adjoint PCG did not converge");
    return SPG_OK;
}

}  // namespace

extern "C" {

int spg_set_dirichlet(spg_handle *h, const double *g) {
    if (!h || !g) return SPG_E_INVALID;
    CK(cudaSetDevice(h->device));
    h->phi_hist = 0;  // a new state: the next run solve starts from phi itself
    h->vac_valid = false;  // the electrode field changes: solved again at the next new particle set
    double *dg = nullptr;
    CK(dalloc(&dg, h->n_nodes));
    CK(cudaMemcpyAsync(dg, g, sizeof(double) * h->n_nodes, cudaMemcpyHostToDevice, h->stream));
    launch_set_dirichlet(h->is_dir, dg, h->dir_value, h->phi, h->n_nodes, h->stream);
    launch_lift(h->elim_rp, h->elim_col, h->elim_val, h->dir_value, h->lift, h->n_nodes, h->stream);
    CK(cudaGetLastError());
    std::vector<uint8_t> isd(h->n_nodes);
    CK(cudaMemcpyAsync(isd.data(), h->is_dir, h->n_nodes, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (int64_t i = 0; i < h->n_nodes; ++i)
        if (isd[i]) h->phi_init[i] = g[i];
    cudaFree(dg);
    return SPG_OK;
}

int spg_set_step_segments(spg_handle *h, int32_t max_steps) {
    if (!h) return SPG_E_INVALID;
    if (max_steps < 1 || max_steps > 64) return fail(h, SPG_E_INVALID, "set_step_segments: 1 <= max_steps <= 64");
    h->seg_max = max_steps;
    return SPG_OK;
}

int spg_grad_field_gradient(spg_handle *h, int32_t on) {
    if (!h) return SPG_E_INVALID;
    h->grad_fg = on != 0;
    return SPG_OK;
}

int spg_grad_forward(spg_handle *h, int32_t nsteps, int32_t checkpoint_every, const double target[3], double sigma,
                     double *J, int64_t *n_landed) {
    if (!h || !target || !(sigma > 0.0) || nsteps < 1 || checkpoint_every < 1)
        return fail(h, SPG_E_INVALID, "grad_forward: bad arguments");
    if (h->prm.collision_model == SPG_COLL_VSS)
        return fail(h, SPG_E_INVALID, "grad_forward: VSS scattering has no adjoint here (HS, VHS or none)");
    if (!h->have_particles) return fail(h, SPG_E_STATE, "grad_forward: no particles set");
    CK(cudaSetDevice(h->device));
    const int64_t n = h->np;
    int rc;
    const int nck = (nsteps + checkpoint_every - 1) / checkpoint_every;
    h->grad_ready = false;
    h->occ_fresh = false;
    const size_t have = h->mixed ? h->ckpt32.size() : h->ckpt.size();
    if (int(have) < nck || n > h->ckpt_cap) {
        free_particle_set(h->ckpt);
        free_particle_set32(h->ckpt32);
        h->ckpt_cap = 0;
        if (h->mixed) {
            h->ckpt32.assign(nck, DevParticles32{});
            for (auto &P : h->ckpt32)
                if ((rc = alloc_dev_particles32(h, P, std::max<int64_t>(n, 1)))) return rc;
        } else {
            h->ckpt.assign(nck, DevParticles{});
            for (auto &P : h->ckpt)
                if ((rc = alloc_dev_particles(h, P, std::max<int64_t>(n, 1)))) return rc;
        }
        h->ckpt_cap = std::max<int64_t>(n, 1);
    }
    if (n > h->land_cap) {
        for (void *q : {(void *)h->land, (void *)h->gr, (void *)h->adj_x, (void *)h->adj_v}) cudaFree(q);
        h->land = nullptr;
        h->gr = h->adj_x = h->adj_v = nullptr;
        h->land_cap = 0;
        const int64_t m = std::max<int64_t>(n, 1);
        CK(dalloc(&h->land, m));
        CK(dalloc(&h->gr, 3 * m));
        CK(dalloc(&h->adj_x, 3 * m));
        CK(dalloc(&h->adj_v, 3 * m));
        h->land_cap = m;
    }
    if ((rc = ensure(h, &h->sums, 2)) || (rc = ensure(h, &h->gE, 3 * size_t(h->n_tets))) ||
        (rc = ensure(h, &h->lam, h->n_nodes)) || (rc = ensure(h, &h->mu, h->n_nodes)) ||
        (rc = ensure(h, &h->dJdg, h->n_nodes)) || (rc = ensure(h, &h->tri_scratch, std::max<int64_t>(h->n_tris, 1))) ||
        (rc = ensure(h, &h->ctr_scratch, 1)))
        return rc;
    CK(cudaMemsetAsync(h->land, 0xff, sizeof(LandRec) * std::max<int64_t>(n, 1), h->stream));
    h->grad_steps = nsteps;
    h->grad_every = checkpoint_every;
    h->grad_step0 = h->step;
    for (int k = 0; k < nsteps; ++k) {
        if (k % checkpoint_every == 0) {
            const int w = k / checkpoint_every;
            rc = h->mixed ? copy_particles32(h, h->ckpt32[w], h->Q[h->cur], n)
                          : copy_particles(h, h->ckpt[w], h->P[h->cur], n);
            if (rc) return rc;
        }
        StepConst c = step_const(h);
        if (h->mixed)
            launch_step32(h->Q[h->cur], h->n_active, mesh_dev32(h), c, h->tri_count, h->walkq, h->walkq_n, h->ctr,
                          field_args(h), h->stream, h->land);
        else
            launch_step64(h->P[h->cur], h->n_active, mesh_dev(h), c, h->tri_count, h->walkq, h->walkq_n, h->ctr,
                          field_args(h), h->stream, h->land);
        CK(cudaGetLastError());
        h->step++;
    }
    CK(cudaMemsetAsync(h->sums, 0, 2 * sizeof(double), h->stream));
    if (h->mixed)
        launch_objective32(h->Q[h->cur], n, mesh_dev32(h), h->land, target, sigma, h->gr, h->sums, h->stream);
    else
        launch_objective(h->P[h->cur], n, h->land, target, sigma, h->gr, h->sums, h->stream);
    CK(cudaGetLastError());
    double sums[2];
    CK(cudaMemcpyAsync(sums, h->sums, sizeof(sums), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (J) *J = sums[1] > 0.0 ? sums[0] / sums[1] : 0.0;
    if (n_landed) *n_landed = int64_t(sums[1]);
    // J = sum g / N_landed with N_landed held fixed: dJ/dr = (dg/dr) / N
    h->grad_inv_n = sums[1] > 0.0 ? 1.0 / sums[1] : 0.0;
    h->grad_ready = sums[1] > 0.0;
    return SPG_OK;
}

int spg_grad_backward(spg_handle *h, double *dJ_dg, double *dJ_dx0, double *dJ_dv0, int32_t *adj_iters) {
    if (!h || !dJ_dg) return fail(h, SPG_E_INVALID, "grad_backward: dJ_dg is required");
    if (!h->grad_ready) return fail(h, SPG_E_STATE, "grad_backward: run spg_grad_forward first (with landings)");
    CK(cudaSetDevice(h->device));
    const int64_t n = h->np;
    const int W = h->grad_every;
    cudaStream_t s = h->stream;
    int rc;
    h->occ_fresh = false;
    const int64_t hneed = int64_t(W) * std::max<int64_t>(n, 1);
    if (hneed > h->hist_cap) {
        for (void *q : {(void *)h->hist.tet, (void *)h->hist.vx, (void *)h->hist.vy, (void *)h->hist.vz}) cudaFree(q);
        h->hist = AdjHist{};
        h->hist_cap = 0;
        CK(dalloc(&h->hist.tet, hneed));
        CK(dalloc(&h->hist.vx, hneed));
        CK(dalloc(&h->hist.vy, hneed));
        CK(dalloc(&h->hist.vz, hneed));
        h->hist_cap = hneed;
    }
    CK(cudaMemsetAsync(h->adj_x, 0, sizeof(double) * 3 * n, s));
    CK(cudaMemsetAsync(h->adj_v, 0, sizeof(double) * 3 * n, s));
    CK(cudaMemsetAsync(h->gE, 0, sizeof(double) * 3 * h->n_tets, s));
    const double *G = nullptr;
    if (h->grad_fg) {
        // the gradient of the recovered field, from the E every tet has now
        // (the forward's field; completed first where a run left it partial)
        if (!h->grad_G) {
            CK(dalloc(&h->grad_G, 9 * h->n_tets));
            CK(dalloc(&h->grad_En, 4 * h->n_nodes));
        }
        if (!h->field_full) {
            const FieldArgs f = field_args(h);
            if (h->mixed)
                launch_field32_full(f, h->n_tets, s);
            else
                launch_field64_full(f, h->n_tets, s);
            h->field_full = true;
        }
        launch_field_gradient(h->tet_nodes, h->rec, h->efield, h->n_tets, h->n_nodes, h->grad_En,
                              h->grad_En + 3 * h->n_nodes, h->grad_G, s);
        CK(cudaGetLastError());
        G = h->grad_G;
    }
    DevParticles &work = h->P[1 - h->cur];
    DevParticles32 &work32 = h->Q[1 - h->cur];
    const int nck = (h->grad_steps + W - 1) / W;
    for (int w = nck - 1; w >= 0; --w) {
        const int k0 = w * W, k1 = std::min(h->grad_steps, k0 + W);
        rc = h->mixed ? copy_particles32(h, work32, h->ckpt32[w], n) : copy_particles(h, work, h->ckpt[w], n);
        if (rc) return rc;
        CK(cudaMemsetAsync(h->ctr_scratch, 0, sizeof(DevCounters), s));
        for (int k = k0; k < k1; ++k) {
            StepConst c = step_const(h);
            c.step = h->grad_step0 + k;
            if (h->mixed) {
                launch_record32(work32, n, h->hist, k - k0, s);
                launch_step32(work32, n, mesh_dev32(h), c, h->tri_scratch, h->walkq, h->walkq_n, h->ctr_scratch,
                              field_args(h), s);
            } else {
                launch_record(work, n, h->hist, k - k0, s);
                launch_step64(work, n, mesh_dev(h), c, h->tri_scratch, h->walkq, h->walkq_n, h->ctr_scratch,
                              field_args(h), s);
            }
        }
        StepConst c = step_const(h);
        c.step = h->grad_step0;  // absolute step of k = 0 (landing steps and Philox counters are absolute)
        if (h->mixed)
            launch_backward32(work32, n, mesh_dev32(h), h->hist, k0, k1, h->land, h->gr, h->grad_inv_n, h->adj_x,
                              h->adj_v, h->gE, c, s, G);
        else
            launch_backward(work, n, h->hist, k0, k1, h->rec, h->land, h->gr, h->grad_inv_n, h->adj_x, h->adj_v,
                            h->gE, c, s, G);
        CK(cudaGetLastError());
    }
    CK(cudaMemsetAsync(h->lam, 0, sizeof(double) * h->n_nodes, s));
    launch_gE_to_nodes(h->tet_nodes, h->rec, h->gE, h->n_tets, h->lam, s);
    launch_adj_rhs(h->lam, h->is_dir, h->b, h->mu, h->n_nodes, s);
    CK(cudaGetLastError());
    int32_t it = 0;
    if ((rc = solve_into(h, h->b, h->mu, &it))) return rc;
    if (adj_iters) *adj_iters = it;
    launch_dirichlet_grad(h->lam, h->is_dir, h->elim_row, h->elim_col, h->elim_val, h->n_elim, h->mu, h->dJdg,
                          h->n_nodes, s);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(dJ_dg, h->dJdg, sizeof(double) * h->n_nodes, cudaMemcpyDeviceToHost, s));
    if (dJ_dx0 || dJ_dv0) {
        double *dx = nullptr, *dv = nullptr;
        if (dJ_dx0) CK(dalloc(&dx, 3 * n));
        if (dJ_dv0) CK(dalloc(&dv, 3 * n));
        if (h->mixed)
            launch_gather_adj32(h->Q[h->cur], n, h->adj_x, h->adj_v, dx, dv, s);
        else
            launch_gather_adj(h->P[h->cur], n, h->adj_x, h->adj_v, dx, dv, s);
        if (dJ_dx0) CK(cudaMemcpyAsync(dJ_dx0, dx, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
        if (dJ_dv0) CK(cudaMemcpyAsync(dJ_dv0, dv, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        cudaFree(dx);
        cudaFree(dv);
    }
    CK(cudaStreamSynchronize(s));
    return SPG_OK;
}

int spg_synchronize(spg_handle *h) {
    if (!h) return SPG_E_INVALID;
    CK(cudaStreamSynchronize(h->stream));
    return SPG_OK;
}

void *spg_stream(spg_handle *h) { return h ? static_cast<void *>(h->stream) : nullptr; }

int spg_profile_enable(spg_handle *h, int32_t on) {
    if (!h) return SPG_E_INVALID;
    if (on && !h->prof) {
        h->prof = true;
        return spg_profile_reset(h);
    }
    h->prof = on != 0;
    return SPG_OK;
}

int spg_profile_reset(spg_handle *h) {
    if (!h) return SPG_E_INVALID;
    CK(cudaStreamSynchronize(h->stream));
    for (EventSeries *s : {&h->ev_step, &h->ev_dep, &h->ev_pcg, &h->ev_ef, &h->ev_sort}) {
        s->used = 0;
        s->ms = 0.0;
        s->launches = 0;
    }
    h->step_bytes = h->dep_bytes = h->pcg_bytes = h->sort_bytes = 0.0;
    h->pcg_iters_prof = 0;
    h->launches = 0;
    DevCounters c{};
    int rc = read_counters(h, c);
    if (rc) return rc;
    h->processed_at_reset = c.processed;
    return SPG_OK;
}

int spg_get_profile(spg_handle *h, spg_profile *pr) {
    if (!h || !pr) return SPG_E_INVALID;
    CK(cudaStreamSynchronize(h->stream));
    for (EventSeries *s : {&h->ev_step, &h->ev_dep, &h->ev_pcg, &h->ev_ef, &h->ev_sort}) ev_resolve(*s);
    DevCounters c{};
    int rc = read_counters(h, c);
    if (rc) return rc;
    std::memset(pr, 0, sizeof(*pr));
    pr->step_ms = h->ev_step.ms;
    pr->step_launches = h->ev_step.launches;
    // 56 B (FP64) or 32 B (mixed) read and written per processed particle
    pr->step_bytes = h->step_bytes + 2.0 * h->pbytes * double(c.processed - h->processed_at_reset);
    pr->deposit_ms = h->ev_dep.ms;
    pr->deposit_launches = h->ev_dep.launches;
    pr->deposit_bytes = h->dep_bytes;
    pr->pcg_ms = h->ev_pcg.ms;
    pr->pcg_solves = h->ev_pcg.launches;
    pr->pcg_bytes = h->pcg_bytes;
    pr->pcg_iters = h->pcg_iters_prof;
    pr->efield_ms = h->ev_ef.ms;
    pr->efield_launches = h->ev_ef.launches;
    pr->sort_ms = h->ev_sort.ms;
    pr->sort_launches = h->ev_sort.launches;
    pr->sort_bytes = h->sort_bytes;
    pr->kernel_launches = h->launches;
    pr->occupied_tets = h->occupied;
    return SPG_OK;
}

}  // extern "C"
