/*
 * pic_oracle.h -- CPU oracle of the PIC/DSMC time step. TEST INFRASTRUCTURE:
 * only the tests, the smoke check and the benchmark's CPU-baseline leg use it,
 * as the checker of libstart_gpu.so; the product never links it.
 *
 * An FP64 C++17 + OpenMP restatement of the reference's step
 * (src/ParticleInCellEngine/ParticleDynamicsProcessor/ParticleDynamicsProcessor.cpp:161-200)
 * with the intended physics (push applied with the containing tet's E,
 * E = -grad(phi), P1 deposit, Poisson with eps0, symmetric Dirichlet
 * elimination). It takes the same mesh and parameter structs as the GPU ABI.
 * Parity is pinned by the reference's own known-answer tests for the
 * primitives (tests/Particle/ParticleTests.cpp, tests/Geometry/
 * SegmentTriangleIntersectionTests.cpp, boundary-condition tests); the
 * reference has no golden vectors for the PIC loop itself.
 */
#ifndef PIC_ORACLE_H
#define PIC_ORACLE_H

#include "../include/start_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct spo_handle spo_handle;

const char *spo_last_error(void);
int spo_set_threads(int n);
int spo_get_threads(void);

int spo_create(const spg_mesh_desc *mesh, const spg_params *params, spo_handle **out);
void spo_destroy(spo_handle *h);
int spo_mesh_info(const spo_handle *h, int64_t info[6]);
int spo_set_particles(spo_handle *h, int64_t n, const double *pos, const double *vel, const int32_t *tet_or_null);
int spo_get_particles(spo_handle *h, int64_t n, double *pos, double *vel, int32_t *tet, uint32_t *flags);
int spo_gather(spo_handle *h, double *rho_out);
int spo_solve(spo_handle *h, const double *rho_or_null, double *phi_out, int32_t *iters, double *relres);
int spo_process(spo_handle *h, int32_t nsteps);
/* Processes only particles [first, first+count) for one step without
 * advancing the step counter (bounded CPU-baseline samples). */
int spo_process_range(spo_handle *h, int64_t first, int64_t count);
int spo_run(spo_handle *h, int32_t nsteps);
int spo_get_stats(spo_handle *h, spg_stats *st);
int spo_get_triangle_counts(spo_handle *h, uint64_t *counts);
int spo_get_potential(spo_handle *h, double *phi);
int spo_set_potential(spo_handle *h, const double *phi);
int spo_get_efield(spo_handle *h, double *E);
int spo_locate(spo_handle *h, int64_t n, const double *pos, int32_t *tet_out);
/* Stiffness in CSR after Dirichlet elimination, and the lifting vector. */
int spo_get_matrix(spo_handle *h, int32_t *row_ptr, int32_t *col, double *val, double *lift);
int spo_get_dual_volumes(spo_handle *h, double *dv);

/* Dirichlet values (g [n_nodes] read at the Dirichlet nodes). */
int spo_set_dirichlet(spo_handle *h, const double *g);
/* FP64 reference gradient of J = (1/N) sum over landed particles of
 * exp(-|r - target|^2 / (2 sigma^2)) after nsteps steps in the current field:
 * full histories, particle adjoint, one adjoint PCG, lifting transpose.
 * dJ_dg [n_nodes]; dJ_dx0, dJ_dv0 [3n] nullable. */
int spo_grad(spo_handle *h, int32_t nsteps, const double *target, double sigma, double *J, int64_t *n_landed,
             double *dJ_dg, double *dJ_dx0, double *dJ_dv0);

/* Field-cell freezing for spo_grad, for finite differences of the map the
 * pathwise adjoint differentiates: mode 1 records the cell whose E pushes each
 * particle at each step of the next spo_grad, mode 2 pushes with the recorded
 * cells in later calls (the walk, landing and collisions stay live), 0 off. */
int spo_grad_freeze(spo_handle *h, int mode);

/* With on != 0, spo_grad also carries the sensitivity of the push to the
 * particle's position, through the gradient of a continuous field recovered
 * from the per-tet E (nodal volume averages, linear in each tet). */
int spo_grad_field_gradient(spo_handle *h, int on);

/* Reference-behaviour switches: each reproduces one behaviour of the
 * reference's own loop that the build changes on purpose. All off by default.
 *   PUSH_NEVER        no electromagnetic push: the pushing tet is looked up by
 *                     particle id among tracker copies that carry new ids
 *                     (src/Particle/Particle.cpp:113-155,
 *                     src/Geometry/Mesh/Cubic/CubicGrid.cpp:149-158)
 *   E_SIGN_SCALE      E = + sum phi_i grad(N_i) |det J| w0 per tet, w0 the
 *                     weight of cubature point 0
 *                     (src/Geometry/Mesh/Volumetric/VolumetricMesh.cpp:371-375,398)
 *   RHS_RAW_RHO       right-hand side = nodal density itself (no eps0, no
 *                     volume), solve from x = 0 every call
 *                     (src/ParticleInCellEngine/ChargeDensityEquationSolver.cpp:17-29,
 *                     src/FiniteElementMethod/Solvers/MatrixEquationSolver.cpp:5-11)
 *   DEPOSIT_VOLAVG    per-tet density, then the volume average over each
 *                     node's occupied tets into a map kept across steps
 *                     (src/ParticleInCellEngine/NodeChargeDensityProcessor.cpp:25-113,
 *                     one chunk: the single-thread semantics)
 *   CLOSED_TETS       with DEPOSIT_VOLAVG, a particle on a shared face, edge or
 *                     vertex counts in every tet holding it
 *                     (VolumetricMesh.cpp:23-33, NodeChargeDensityProcessor.cpp:52-55)
 *   SOLVE_EVERY_STEP  gather + solve at every step (src/ModelingMainDriver.cpp:146-161)
 *   MIXED_UNITS       displacement v dt / 1000: metres added to millimetre
 *                     coordinates (src/Particle/Particle.cpp:157-165) */
enum {
    SPO_COMPAT_PUSH_NEVER = 1,
    SPO_COMPAT_E_SIGN_SCALE = 2,
    SPO_COMPAT_RHS_RAW_RHO = 4,
    SPO_COMPAT_DEPOSIT_VOLAVG = 8,
    SPO_COMPAT_CLOSED_TETS = 16,
    SPO_COMPAT_SOLVE_EVERY_STEP = 32,
    SPO_COMPAT_MIXED_UNITS = 64,
    SPO_COMPAT_ALL = 127
};
/* Sets the switches (and the cubature weight for E_SIGN_SCALE, 1/6 for the
 * one-point rule); clears the volume-average density map. */
int spo_set_ref_compat(spo_handle *h, uint32_t flags, double cubature_w0);

/* Primitives pinned by the reference's unit tests. */
void spo_update_position(double *pos3, const double *vel3, double dt);
/* Segment-triangle intersection: 1 and the point when they meet (a segment
 * lying in the triangle returns its source), else 0. */
int spo_segment_triangle(const double *s0, const double *s1, const double *a, const double *b, const double *c,
                         double *point);
double spo_gas_concentration(double pressure, double temperature);
/* Collision law with given uniforms u0 (decision), u1, u2: returns 1 and the
 * new velocity when u0 < P. model: spg_collision_model. */
int spo_collide_with(const spg_params *p, double *vel3, double u0, double u1, double u2);
double spo_collision_probability(const spg_params *p, const double *vel3);
/* Barycentric map; returns det(J). */
double spo_tet_map(const double *x0, const double *x1, const double *x2, const double *x3, double *M9);
/* Philox4x32-10 block. */
void spo_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* The collision decisions of n (step, particle id) pairs at probability P
 * each (the candidate-byte rule of the step), 1 = a collision. */
void spo_collides(const uint64_t *steps, const uint32_t *ids, int64_t n, uint64_t seed, double P, uint8_t *out);

#ifdef __cplusplus
}
#endif

#endif
