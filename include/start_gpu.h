/*
 * start_gpu.h -- C ABI of the GB300 particle-in-cell / DSMC time step.
 *
 * The library (libstart_gpu.so) replaces the per-step calls that Start's
 * ModelingMainDriver makes into its ParticleInCellEngine
 * (src/ModelingMainDriver.cpp:146-184):
 *
 *   NodeChargeDensityProcessor::gather   -> spg_gather
 *     (include/ParticleInCellEngine/NodeChargeDensityProcessor.hpp:39-46)
 *   ChargeDensityEquationSolver::solve   -> spg_solve
 *     (include/ParticleInCellEngine/ChargeDensityEquationSolver.hpp:38-42,
 *      which calls MatrixEquationSolver::solve / calculateElectricField,
 *      src/FiniteElementMethod/Solvers/MatrixEquationSolver.cpp:359-427)
 *   ParticleDynamicsProcessor::process   -> spg_process
 *     (include/ParticleInCellEngine/ParticleDynamicsProcessor/ParticleDynamicsProcessor.hpp:154-170)
 *   the whole time loop                  -> spg_run
 *     (src/ModelingMainDriver.cpp:132-220)
 *   SurfaceMesh triangle counters        -> spg_get_triangle_counts
 *     (include/Geometry/Mesh/Surface/TriangleCell.hpp:17-23, read by
 *      src/DataHandling/TriangleMeshHdf5Manager.cpp:97-140)
 *
 * Conventions
 *   - Every function returns an int status: 0 (SPG_OK) or a negative
 *     spg_status code. No C++ exception crosses this boundary.
 *   - spg_last_error(h) returns a message for the last failure on h;
 *     spg_last_error(NULL) returns the last failure of spg_create on the
 *     calling thread.
 *   - The handle owns all device memory and one CUDA stream. Caller buffers
 *     are host memory; they are copied in and out inside the call.
 *   - One handle per host thread at a time.
 *   - Units are SI (metres, seconds, volts, coulombs, kilograms). The
 *     reference keeps mesh coordinates in millimetres; convert on load.
 *   - Particle identity: particle k of spg_set_particles keeps id k for the
 *     whole run; every getter returns particles in id order.
 */
#ifndef START_GPU_H
#define START_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPG_ABI_VERSION 1

typedef enum spg_status {
    SPG_OK = 0,
    SPG_E_INVALID = -1,        /* bad argument (null pointer, size mismatch, bad enum) */
    SPG_E_CUDA = -2,           /* a CUDA runtime call failed */
    SPG_E_BAD_MESH = -3,       /* degenerate tet, bad node index, non-manifold face */
    SPG_E_NOT_CONVERGED = -4,  /* PCG hit cg_max_iter; the iterate is kept */
    SPG_E_LOST_PARTICLES = -5, /* some particle left the mesh or hit max_crossings */
    SPG_E_NO_DEVICE = -6,      /* no CUDA device / wrong architecture */
    SPG_E_OOM = -7,            /* device allocation failed */
    SPG_E_STATE = -8           /* call order (e.g. process before set_particles) */
} spg_status;

typedef enum spg_collision_model {
    SPG_COLL_NONE = 0,
    SPG_COLL_HS = 1,  /* src/Particle/PhysicsCore/CollisionModel/HSModel.cpp:6-42 */
    SPG_COLL_VHS = 2, /* .../VHSModel.cpp:6-52 */
    SPG_COLL_VSS = 3  /* .../VSSModel.cpp:6-54 */
} spg_collision_model;

typedef enum spg_precision {
    SPG_FP64 = 0,  /* plain form: FP64 state, push, walk and PCG */
    SPG_MIXED = 1  /* FP32 tet-local state and push; FP32 V-cycle in FP64 PCG (AMG), FP32-SpMV PCG in FP64 refinement (Jacobi) */
} spg_precision;

/* Preconditioner of the Poisson PCG. The reference preconditions Belos CG
 * with MueLu (src/FiniteElementMethod/Solvers/MatrixEquationSolver.cpp:359-427),
 * whose default is smoothed aggregation with Chebyshev smoothing. */
typedef enum spg_preconditioner {
    SPG_PRECOND_JACOBI = 0,  /* diagonal scaling */
    SPG_PRECOND_AMG = 1,     /* smoothed-aggregation AMG V-cycle with damped-Jacobi smoothing; the
                                V-cycle runs in FP64 in the plain form, in FP32 in the mixed form */
    SPG_PRECOND_AMG_F32 = 2  /* the same V-cycle in FP32 in both forms. The PCG itself (SpMV, vectors,
                                dot products, stop test) stays FP64, so the solve reaches the same
                                FP64 residual target; only M^-1 is rounded to FP32 */
} spg_preconditioner;

/* Particle flag bits returned by spg_get_particles. */
#define SPG_FLAG_SETTLED 1u /* crossed a surface triangle; position = hit point */
#define SPG_FLAG_LOST 2u    /* left the mesh through a face with no triangle, or walk cap */

/* Tet mesh. Node index = gmsh node tag - 1 (GSMAssembler.cpp:10-72). */
typedef struct spg_mesh_desc {
    int64_t n_nodes;
    const double *node_xyz;        /* [3*n_nodes] */
    int64_t n_tets;
    const int32_t *tet_nodes;      /* [4*n_tets]; either orientation */
    int64_t n_triangles;
    const int32_t *tri_nodes;      /* [3*n_triangles]; surface triangles, id = row */
    int64_t n_dirichlet;
    const int32_t *dirichlet_nodes; /* [n_dirichlet] */
    const double *dirichlet_values; /* [n_dirichlet] volts */
} spg_mesh_desc;

typedef struct spg_params {
    double dt;                /* time step [s] */
    double charge;            /* charge of one physical particle [C] */
    double mass;              /* projectile mass [kg] */
    double weight;            /* physical particles per macro-particle */
    int32_t collision_model;  /* spg_collision_model */
    int32_t precision;        /* spg_precision */
    double gas_mass;          /* background gas molecule mass [kg] */
    double gas_concentration; /* n [m^-3]; P*N_A/(R*T) in the reference (Utilities.cpp:132-149) */
    double hs_diameter;       /* HS collision diameter d: sigma = pi*d^2 */
    double vhs_dref;          /* VHS/VSS reference diameter */
    double omega;             /* viscosity-temperature index */
    double alpha;             /* VSS deflection parameter */
    double kT_ref;            /* k*T_ref [J]; 297*1.380658e-23 in Constants.hpp:12 */
    double epsilon0;          /* vacuum permittivity [F/m] */
    double min_velocity;      /* particles slower than this are not moved (Constants.hpp:50) */
    double bbox_expansion;    /* surface bbox expansion factor (Constants.hpp, 1.01) */
    uint64_t seed;            /* Philox key for collisions */
    int32_t poisson_every;    /* spg_run: deposit + solve every N steps */
    int32_t resort_every;     /* spg_run: re-sort particles by tet every N steps (0 = never) */
    int32_t max_crossings;    /* tet-walk cap per particle per step */
    int32_t cg_max_iter;      /* PCG iteration cap */
    double cg_rtol;           /* PCG stop: ||r||_2 <= cg_rtol * ||b||_2 */
    int32_t device;           /* CUDA device ordinal */
    int32_t preconditioner;   /* spg_preconditioner: PCG preconditioner of the Poisson solve */
} spg_params;

typedef struct spg_stats {
    int64_t step;             /* steps taken so far */
    int64_t n_particles;
    int64_t n_alive;          /* neither settled nor lost */
    int64_t n_settled;
    int64_t n_lost;
    int64_t particle_steps;   /* cumulative alive-particle steps processed */
    int64_t collisions;       /* cumulative gas collisions */
    int64_t crossings;        /* cumulative tet-face crossings */
    int64_t cg_iters_total;
    int32_t cg_iters_last;
    int32_t cg_solves;
    double cg_relres_last;
} spg_stats;

/* Cumulative device timings (CUDA events on the handle's stream), enabled by
 * spg_profile_enable. Times in milliseconds, bytes are algorithmic bytes. */
typedef struct spg_profile {
    double step_ms;      int64_t step_launches;    double step_bytes;
    double deposit_ms;   int64_t deposit_launches; double deposit_bytes;
    double pcg_ms;       int64_t pcg_solves;       double pcg_bytes; int64_t pcg_iters;
    double efield_ms;    int64_t efield_launches;
    double sort_ms;      int64_t sort_launches;    double sort_bytes;
    int64_t kernel_launches; /* every kernel this library launched while profiling */
    int64_t occupied_tets;   /* tets holding alive particles at the last re-sort */
} spg_profile;

typedef struct spg_handle spg_handle;

const char *spg_version(void);
void spg_default_params(spg_params *p);
const char *spg_last_error(const spg_handle *h);

/* Builds the device mesh, P1 stiffness (closed form, GSMAssembler.cpp:10-118),
 * symmetric Dirichlet elimination and surface-triangle face map. */
int spg_create(const spg_mesh_desc *mesh, const spg_params *params, spg_handle **out);
int spg_destroy(spg_handle *h);

/* Wall times of spg_create in ms: [whole call, GPU element maps and orientation,
 * GPU node incidence + stiffness + Dirichlet elimination, host face matching +
 * surface triangles + location grid, AMG hierarchy (0 without AMG), uploads
 * and the rest]. (The reference's FEMInitializer + GSMAssembler set-up.) */
int spg_setup_times(const spg_handle *h, double ms[6]);

/* Mesh counters: [n_nodes, n_tets, n_triangles, n_boundary_faces, nnz, n_dirichlet]. */
int spg_mesh_info(const spg_handle *h, int64_t info[6]);

/* Uploads particles (SoA-free interleaved xyz). tet may be NULL: the library
 * then locates each particle with a tet walk from a voxel seed; particles
 * outside the mesh are flagged LOST. Resets step, counters and potential: with
 * an AMG preconditioner the potential restarts from the electrode field (the
 * potential of the Dirichlet values with no charge, solved in spg_create and
 * again at the first new particle set after spg_set_dirichlet), otherwise from
 * the Dirichlet values with zero elsewhere. */
int spg_set_particles(spg_handle *h, int64_t n, const double *pos, const double *vel,
                      const int32_t *tet_or_null);
/* Any output pointer may be NULL. Arrays are [3*n] / [n], in id order. */
int spg_get_particles(spg_handle *h, int64_t n, double *pos, double *vel, int32_t *tet,
                      uint32_t *flags);

/* Particle source sampled on the device, in place of ParticleGeneratorDevice
 * (src/Generators/CUDA/ParticleGeneratorDevice.cu:95-304) and the host sampling of
 * ParticleDynamicUtils.hpp:52-97: points uniform over a disk or a rectangle,
 * directions uniform in a cone or Lambert (cosine) about the normal, energies
 * monoenergetic or Thompson f(E) ~ E/(E+U)^3 truncated at E_max, then the
 * ParticleDisplacer shift (src/Particle/ParticleDisplacer.cpp:20-35), the
 * vector s / max|s_k| * displacement: with the fan law (the reference's point
 * and surface sources) s is the source's direction or the cell's normal, one
 * vector for all its particles (:48-133); with the cone and cosine laws s is
 * each particle's own direction. Particle i draws from Philox4x32-10 keyed
 * by (seed) and counted by (i, block), so a source is reproducible and does
 * not depend on the launch shape. */
typedef enum spg_source_shape {
    SPG_SRC_DISK = 0,
    SPG_SRC_RECT = 1,
    SPG_SRC_POINT = 2, /* every particle at centre (ParticleGenerator::fromPointSource) */
    SPG_SRC_CELLS = 3  /* surface cells: count split evenly over the cells, the remainder one each to
                          seed-chosen cells (ParticleGenerator::fromSurfaceSource) */
} spg_source_shape;
typedef enum spg_source_directions {
    SPG_DIR_CONE = 0,
    SPG_DIR_COSINE = 1,
    SPG_DIR_FAN = 2 /* the reference's law: polar angle theta0 + U(-1,1) expansion at the fixed azimuth
                       phi0 of the normal, theta0 = acos(n_z), phi0 = atan2(n_y, n_x)
                       (ParticleDynamicUtils::calculateVelocityFromEnergy_eV) */
} spg_source_directions;
typedef enum spg_source_energy { SPG_ENERGY_MONO = 0, SPG_ENERGY_THOMPSON = 1 } spg_source_energy;
typedef struct spg_source {
    int32_t shape;        /* spg_source_shape */
    int32_t directions;   /* spg_source_directions */
    int32_t energy;       /* spg_source_energy */
    int32_t reserved0;
    double centre[3];     /* disk centre [m] */
    double normal[3];     /* disk normal; directions are about it (rectangles: +z) */
    double radius;        /* disk radius [m] */
    double xlim[2], ylim[2], z; /* rectangle in the plane z = const [m] */
    double half_angle;    /* cone half-angle [rad] */
    double energy_ev;     /* monoenergetic energy [eV] */
    double binding_ev;    /* Thompson U [eV] */
    double emax_ev;       /* Thompson truncation [eV] */
    double displacement;  /* largest component of the shift [m]; 0.05 mm in the reference */
    uint64_t seed;
    /* SPG_SRC_CELLS: n_cells cells, cells[6 k .. 6 k + 5] = centre xyz [m], normal xyz (the
     * baseCoordinates of a surface source); host memory, read during the call */
    int32_t n_cells;
    int32_t reserved1;
    const double *cells;
    double expansion;     /* SPG_DIR_FAN: polar-angle spread [rad] (expansionAngle) */
} spg_source;
void spg_default_source(spg_source *src);

/* Trajectory sampling, in place of ParticleMovementTracker::recordMovement
 * (src/ParticleInCellEngine/ParticleDynamicsProcessor/ParticleMovementTracker.cpp:4-16):
 * the k particles ids[] (0 <= id < n) have their position appended before
 * every step in which they are alive, up to `capacity` positions each. A new
 * particle set, a restore, or k = 0 ends the tracking.
 * spg_get_tracks: counts [k], xyz [k * capacity * 3] (row t holds counts[t]
 * positions), and each tracked particle's current position and flags; a
 * settled particle's current position is its surface hit point, the last
 * point the reference's surface handler records. Any output may be NULL. */
int spg_track_particles(spg_handle *h, int32_t k, const int64_t *ids, int32_t capacity);
int spg_get_tracks(spg_handle *h, int32_t *counts, double *xyz, double *last_xyz, uint32_t *last_flags);
/* Samples n particles of mass params.mass on the device and installs them as
 * spg_set_particles does (location, LOST flags, reset of step, counters and
 * potential); nothing crosses the host link. */
int spg_generate_particles(spg_handle *h, int64_t n, const spg_source *src);
/* Continuous injection (the per-step _spawnParticles of ModelingMainDriver.cpp:37-68 with
 * sputtering on): samples n more particles from src on the device and appends them to the
 * current set, after the existing ones, with ids np .. np + n - 1. Step, counters, potential,
 * field and tracks are kept; the Philox counter of a particle is its id, so each injection
 * draws new numbers from the same seed. */
int spg_inject_particles(spg_handle *h, int64_t n, const spg_source *src);

/* (a) P1 charge deposit of all alive particles; rho_out [n_nodes] C/m^3 (nullable).
 * With rho_out NULL the density stays on the device, where the next
 * spg_solve(h, NULL, ...) uses it: the per-step gather -> solve of
 * ModelingMainDriver.cpp:146-184 then moves nothing through the host. */
int spg_gather(spg_handle *h, double *rho_out);
/* Nodal density [n_nodes] C/m^3 of the handle's current charge (the last
 * deposit, or the density last given to spg_solve), without depositing again:
 * the NodeChargeDensitiesMap that gather fills in the reference
 * (include/ParticleInCellEngine/NodeChargeDensityProcessor.hpp:39-46), read
 * only when the caller looks at it. SPG_E_STATE before any deposit. */
int spg_get_charge_density(spg_handle *h, double *rho_out);
/* (b) Poisson solve K phi = rho*Vdual/eps0 with Dirichlet lifting, warm started
 * from the previous phi; then E per tet. rho_or_null: use this nodal rho
 * (host memory, copied up once; the node charges rho*Vdual are formed on the
 * device) instead of the last deposit. Returns SPG_E_NOT_CONVERGED at the cap. */
int spg_solve(spg_handle *h, const double *rho_or_null, double *phi_out, int32_t *iters,
              double *relres);
/* (c)(d)(e) nsteps particle steps with the current E (no deposit, no solve). */
int spg_process(spg_handle *h, int32_t nsteps, spg_stats *stats);
/* The whole loop: per step, gather+solve when step % poisson_every == 0,
 * re-sort when step % resort_every == 0, then process. The host does not
 * wait for the solves: their iteration counts and residuals are read when
 * the call ends, and a solve that reached cg_max_iter makes the call return
 * SPG_E_NOT_CONVERGED then (the run goes on with its potential, as the
 * reference's loop does: src/FiniteElementMethod/Solvers/
 * MatrixEquationSolver.cpp:405-412 logs the failure and returns). */
int spg_run(spg_handle *h, int32_t nsteps, spg_stats *stats);
/* Re-sorts particles by tet now (settled/lost particles move to the end). */
int spg_resort(spg_handle *h);
/* No counterpart in the reference (an execution choice, not a result). In the
 * mixed form spg_run and spg_process run the steps between two events of the
 * loop (a solve, a re-sort, the end of the call) as segments of up to
 * max_steps steps: one pass keeps each particle in registers until a move
 * needs the exact tet walk, the walk runs batched, and the walked particles
 * resume from the next step. Results are bit-identical to one launch per
 * step (max_steps = 1). Default 32; SPG_E_INVALID outside 1..64. The FP64
 * form and runs with trajectory sampling always step one launch per step. */
int spg_set_step_segments(spg_handle *h, int32_t max_steps);

int spg_get_stats(spg_handle *h, spg_stats *stats);
int spg_get_triangle_counts(spg_handle *h, uint64_t *counts /* [n_triangles] */);
int spg_get_potential(spg_handle *h, double *phi /* [n_nodes] */);
/* Sets phi (Dirichlet values are kept as given) and recomputes E. */
int spg_set_potential(spg_handle *h, const double *phi);
int spg_get_efield(spg_handle *h, double *E /* [3*n_tets] */);
/* The assembled FEM system (the counterpart of GSMAssembler's global matrix after
 * MatrixBoundaryConditionsManager): CSR stiffness with Dirichlet rows as identity rows,
 * row_ptr [n_nodes + 1], col and val [nnz] (info[4] of spg_mesh_info), the lifting of the current
 * Dirichlet values [n_nodes] and the dual volumes [n_nodes]. Any output may be NULL. */
int spg_get_matrix(spg_handle *h, int32_t *row_ptr, int32_t *col, double *val, double *lift, double *dual_vol);
/* Point location through the same walk as spg_set_particles. */
int spg_locate(spg_handle *h, int64_t n, const double *pos, int32_t *tet_out);

/* Checkpoint: particles, step, phi, counters. The Philox streams are keyed by
 * (seed, particle id, step), so a restored run continues bit-identically. */
int spg_checkpoint_size(spg_handle *h, size_t *bytes);
int spg_checkpoint(spg_handle *h, void *buf, size_t bytes);
int spg_restore(spg_handle *h, const void *buf, size_t bytes);

/* Dirichlet values: g [n_nodes], read at the Dirichlet nodes of the mesh.
 * Updates the lifting of the right-hand side; the next spg_solve uses them.
 * (The reference sets them once from its config, MatrixBoundaryConditionsManager.) */
int spg_set_dirichlet(spg_handle *h, const double *g);

/* Gradient of a smoothed landing objective through the particle steps, of
 * the FP64 form or of the mixed form's FP32 step (collisions none/HS/VHS,
 * with their events and random numbers held fixed; the cell whose field
 * pushes each step also counts as fixed: the field is constant per tet).
 * spg_grad_forward runs nsteps particle steps in the current field
 * (no deposit or solve), keeping the particle state every checkpoint_every
 * steps and where each particle lands, and returns
 *   J = (1/N) sum over the N particles that landed of exp(-|r - target|^2 / (2 sigma^2)).
 * spg_grad_backward recomputes each checkpoint window, runs the adjoint of
 * push, move and frozen collisions, one adjoint CG on the stiffness matrix,
 * and returns dJ/dg at the Dirichlet nodes (0 elsewhere) and, if non-NULL,
 * dJ/d(initial position) and dJ/d(initial velocity) per particle [3n, id order].
 * N is held constant. Tet crossings are piecewise constant and carry no gradient. */
int spg_grad_forward(spg_handle *h, int32_t nsteps, int32_t checkpoint_every, const double target[3], double sigma,
                     double *J, int64_t *n_landed);
int spg_grad_backward(spg_handle *h, double *dJ_dg, double *dJ_dx0, double *dJ_dv0, int32_t *adj_cg_iters);
/* No counterpart in the reference. on != 0: spg_grad_backward also carries the
 * push's dependence on the particle's position, through the gradient of a
 * continuous field recovered from the per-tet E (nodal volume averages,
 * linear in each tet). The per-cell field has no gradient inside a cell, so
 * the plain pathwise gradient (on = 0, the default: the exact derivative of
 * the step with collision events, random numbers and pushing cells held
 * fixed) leaves out how a shifted trajectory feels a different field; with
 * this term the gradient follows central differences of the live step far
 * more closely. Costs 72 B per tet of device memory when first used. */
int spg_grad_field_gradient(spg_handle *h, int32_t on);

int spg_synchronize(spg_handle *h);
/* cudaStream_t of the handle, for callers that record their own events. */
void *spg_stream(spg_handle *h);
int spg_profile_enable(spg_handle *h, int32_t on);
int spg_get_profile(spg_handle *h, spg_profile *prof);
int spg_profile_reset(spg_handle *h);

/* Jacobi-preconditioned CG on a caller-provided CSR matrix that allocates
 * nothing. It has no counterpart in the reference: it exists for callers that
 * must not call cudaMalloc/cudaFree. That covers a program whose device memory
 * is all owned by its own pool (a PyTorch caching allocator, a fixed arena),
 * and a loop that must not take the device-wide synchronisation that
 * cudaMalloc/cudaFree can imply. The call itself still synchronises the
 * stream it is given: every 8 iterations it reads the CG scalars back to the
 * host to decide whether to go on.
 *
 * row_ptr [n+1], col [nnz], val [nnz], b [n] and x [n] are DEVICE pointers the
 * caller allocated; x holds the initial guess and receives the solution.
 * Stop rule: ||r_k||_2 <= rtol ||b||_2, where r_k is the CG residual updated
 * by the recurrence r_{k+1} = r_k - alpha A p_k (equal to b - A x_k up to
 * rounding), or max_iter iterations.
 * Results:
 *   SPG_OK               converged; *iters and *relres = ||r_k|| / ||b||.
 *                        b = 0 gives x = 0, 0 iterations, relres 0.
 *   SPG_E_NOT_CONVERGED  max_iter reached, or a CG breakdown (p.Ap <= 0: the
 *                        matrix is not SPD, or the data hold NaN); the
 *                        message says which; x keeps the last iterate.
 *   SPG_E_INVALID        bad sizes or null arrays, or a row with no stored
 *                        diagonal entry or a zero or non-finite one.
 * stream is a cudaStream_t, or NULL for the default stream.
 *
 * Limit: n <= 131072 rows. Larger n returns SPG_E_INVALID without touching
 * the GPU. The working vectors live in one static device array of about
 * 5.3 MB that every GPU loading the library keeps until the process exits.
 * All calls on a device share it. Calls that overlap on the GPU (several
 * streams, several host threads) race on it and must be serialised by the
 * caller. Each call resets the parts that must start at zero.
 *
 * The first call on each device looks up the array's device address with
 * that device current. Make that first call before any stream capture. Error
 * messages: spg_last_error(NULL) on the calling thread. */
int spg_pcg_solve_noalloc(int64_t n, const int32_t *row_ptr, const int32_t *col, const double *val,
                          const double *b, double *x, double rtol, int32_t max_iter, void *stream,
                          int32_t *iters, double *relres);

#ifdef __cplusplus
}
#endif

#endif /* START_GPU_H */
