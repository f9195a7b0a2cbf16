// Adjoint of the particle step for the gradient of a smoothed landing-point
// objective with respect to the field (and through it the electrode
// potentials) and to each particle's initial state.
//
// The field is P1, constant per tet, so within a step the velocity does not
// depend on the position: the step is
//     v_a = v_k + c E(t_k)            (Boris push with B = 0, c = q dt / m)
//     x_{k+1} = x_k + v_a dt
//     v_{k+1} = C_k(v_a)              (gas collision when one happened, with
//                                      the collision event and its random
//                                      numbers held fixed)
// and a particle that lands in step N does so at r = x_N + s v_a dt on the
// plane n.r = const of the exit face, s = (const - n.x_N)/(n.v_a dt). With
// P = I - v_a n^T / (n.v_a) and g = dJ/dr the backward recursion is
//     at step N:   abar_x = P^T g,  abar_va = s dt P^T g
//     at step k<N: abar_va = J_Ck^T abar_v(k+1) + dt abar_x
//     each step:   dJ/dE(t_k) += c abar_va,  abar_v(k) = abar_va
// The tet sequence t_k and v_k come from recomputing each checkpoint window
// forward (k_record + the production step kernels); the discrete tet
// crossings and collision decisions are piecewise constant and carry no
// gradient.
#include <cmath>

#include "philox.h"
#include "spg_internal.h"

namespace spg {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr double kPi = 3.14159265358979323846;

__global__ void k_record(const DevParticles p, int64_t n, AdjHist h, int k) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t o = int64_t(k) * n + i;
    h.tet[o] = (p.idf[i] & kDead) ? -1 : p.tet[i];
    h.vx[o] = p.vx[i];
    h.vy[o] = p.vy[i];
    h.vz[o] = p.vz[i];
}

// dg/dr for each landed particle, g = exp(-|r - r_t|^2 / (2 sigma^2)), and the
// sums of g and of the landed count (J = sum g / N_landed; the backward scales
// dg/dr by 1/N_landed).
__global__ void k_objective(const DevParticles p, int64_t n, const LandRec *__restrict__ land, double tx, double ty,
                            double tz, double inv_2s2, double *__restrict__ gr, double *__restrict__ sums) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    double g = 0.0, cnt = 0.0;
    if (i < n) {
        gr[3 * i] = gr[3 * i + 1] = gr[3 * i + 2] = 0.0;
        if ((p.idf[i] & kSettled) && land[i].step >= 0) {
            const double dx = p.x[i] - tx, dy = p.y[i] - ty, dz = p.z[i] - tz;
            g = exp(-(dx * dx + dy * dy + dz * dz) * inv_2s2);
            const double f = -2.0 * inv_2s2 * g;  // d g / d r = -g (r - r_t) / sigma^2
            gr[3 * i] = f * dx;
            gr[3 * i + 1] = f * dy;
            gr[3 * i + 2] = f * dz;
            cnt = 1.0;
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        g += __shfl_down_sync(kFull, g, off);
        cnt += __shfl_down_sync(kFull, cnt, off);
    }
    if ((threadIdx.x & 31) == 0 && cnt > 0.0) {
        atomicAdd(sums, g);
        atomicAdd(sums + 1, cnt);
    }
}

__device__ __forceinline__ void face_normal(const TetRec &r, int f, double n[3]) {
    if (f == 0) {
        for (int k = 0; k < 3; ++k) n[k] = -(r.M[k] + r.M[3 + k] + r.M[6 + k]);
    } else {
        for (int k = 0; k < 3; ++k) n[k] = r.M[3 * (f - 1) + k];
    }
}

// Collision decision of step k for velocity va, exactly as the forward took
// it (u0 < P with the reference's P), and the scattering direction.
__device__ bool collided(const StepConst &c, uint32_t id, int64_t k, double vx, double vy, double vz, double nh[3]) {
    const uint32_t byte = candidate_byte(candidate_block(uint64_t(k), id, c.seed_lo, c.seed_hi), uint64_t(k));
    const double vmod = sqrt(vx * vx + vy * vy + vz * vz);
    double sigma;
    if (c.model == SPG_COLL_HS) {
        sigma = c.sigma_hs;
    } else {
        const double base = c.two_kT / ((c.mr * vmod) * vmod);
        sigma = kPi * (c.vhs_c1 * pow(base, c.expo));
    }
    const double P = ((sigma * vmod) * c.gas_n) * c.dt;
    bool hit;
    if (P <= kCandQ) {
        hit = byte == 0u && u01_from_block(collision_draw(uint64_t(k), 3u, id, c.seed_lo, c.seed_hi)) < P * 256.0;
    } else {
        hit = byte == 0u ||
              u01_from_block(collision_draw(uint64_t(k), 4u, id, c.seed_lo, c.seed_hi)) < (P - kCandQ) / (1.0 - kCandQ);
    }
    if (!hit) return false;
    const Philox4 r = collision_draw(uint64_t(k), 1u, id, c.seed_lo, c.seed_hi);
    const double u1 = u01_from(r.v[0], r.v[1]);
    const double u2 = u01_from(r.v[2], r.v[3]);
    const double xc = c.model == SPG_COLL_HS ? -1.0 + 2.0 * u1 : u1;
    const double xs = sqrt(1.0 - xc * xc);
    double sph, cph;  // the forward's azimuth, cospi / sinpi (2 u2)
    sincospi(2.0 * u2, &sph, &cph);
    nh[0] = xs * cph;
    nh[1] = xs * sph;
    nh[2] = xc;
    return true;
}

// Backward recursion over steps [k0, k1) of one checkpoint window, one
// particle per thread; the adjoint state (abar_x, abar_v) carries between
// windows in ax/av. Contributions to dJ/dE of consecutive steps in one tet
// are summed in registers and added once.
__global__ void __launch_bounds__(128) k_backward(const DevParticles p, int64_t n, const AdjHist h, int k0, int k1,
                                                  const TetRec *__restrict__ rec, const LandRec *__restrict__ land,
                                                  const double *__restrict__ gr, double gscale, double *__restrict__ ax,
                                                  double *__restrict__ av, double *__restrict__ gE, StepConst c,
                                                  double cq, const double *__restrict__ G) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const LandRec L = land[i];
    // c.step is the absolute step of k = 0; landing steps are absolute
    const int N = L.step < 0 ? -1 : int(int64_t(L.step) - c.step);
    if (N < k0) return;
    const uint32_t id = p.idf[i] & kIdMask;
    double Ax = ax[3 * i], Ay = ax[3 * i + 1], Az = ax[3 * i + 2];
    double Vx = av[3 * i], Vy = av[3 * i + 1], Vz = av[3 * i + 2];
    int run = -1;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int k = min(k1 - 1, N); k >= k0; --k) {
        const int64_t o = int64_t(k - k0) * n + i;
        const int t = h.tet[o];
        if (t < 0) continue;
        const double vx = h.vx[o], vy = h.vy[o], vz = h.vz[o];
        if (sqrt(vx * vx + vy * vy + vz * vz) < c.vmin) continue;  // the step did not move it
        const TetRec &R = rec[t];
        double ax_ = vx, ay_ = vy, az_ = vz;
        if (!R.ezero) {
            ax_ = (vx + R.H[0]) + R.H[0];
            ay_ = (vy + R.H[1]) + R.H[1];
            az_ = (vz + R.H[2]) + R.H[2];
        }
        double bx, by, bz;  // abar_va
        if (k == N) {
            const TetRec &RL = rec[L.tet];
            double nn[3];
            face_normal(RL, L.face, nn);
            const double gx = gr[3 * i] * gscale, gy = gr[3 * i + 1] * gscale, gz = gr[3 * i + 2] * gscale;
            const double nv = nn[0] * ax_ + nn[1] * ay_ + nn[2] * az_;
            const double vg = (ax_ * gx + ay_ * gy + az_ * gz) / nv;
            Ax = gx - nn[0] * vg;  // P^T g
            Ay = gy - nn[1] * vg;
            Az = gz - nn[2] * vg;
            const double sdt = L.s * c.dt;
            bx = sdt * Ax;
            by = sdt * Ay;
            bz = sdt * Az;
        } else {
            double nh[3];
            if (c.model != SPG_COLL_NONE && collided(c, id, c.step + k, ax_, ay_, az_, nh)) {
                // v' = m_cp v + m_ct |v| n:  J^T a = m_cp a + m_ct v/|v| (n . a)
                const double vm = sqrt(ax_ * ax_ + ay_ * ay_ + az_ * az_);
                const double na = (nh[0] * Vx + nh[1] * Vy + nh[2] * Vz) * c.mass_ct / vm;
                Vx = c.mass_cp * Vx + na * ax_;
                Vy = c.mass_cp * Vy + na * ay_;
                Vz = c.mass_cp * Vz + na * az_;
            }
            bx = Vx + c.dt * Ax;
            by = Vy + c.dt * Ay;
            bz = Vz + c.dt * Az;
        }
        // v_a = v + c E is continuous in E, also where E = 0 skipped the push
        if (t != run) {
            if (run >= 0) {
                atomicAdd(gE + 3 * run, cq * sx);
                atomicAdd(gE + 3 * run + 1, cq * sy);
                atomicAdd(gE + 3 * run + 2, cq * sz);
            }
            run = t;
            sx = sy = sz = 0.0;
        }
        sx += bx;
        sy += by;
        sz += bz;
        Vx = bx;
        Vy = by;
        Vz = bz;
        if (G && !R.ezero) {
            // the pushed velocity depends on the position through the recovered
            // field: abar_x += cq G^T abar_va, G[3 d + c] = dE_d / dx_c
            const double *g = G + 9 * int64_t(t);
            Ax += cq * (g[0] * bx + g[3] * by + g[6] * bz);
            Ay += cq * (g[1] * bx + g[4] * by + g[7] * bz);
            Az += cq * (g[2] * bx + g[5] * by + g[8] * bz);
        }
    }
    if (run >= 0) {
        atomicAdd(gE + 3 * run, cq * sx);
        atomicAdd(gE + 3 * run + 1, cq * sy);
        atomicAdd(gE + 3 * run + 2, cq * sz);
    }
    ax[3 * i] = Ax;
    ax[3 * i + 1] = Ay;
    ax[3 * i + 2] = Az;
    av[3 * i] = Vx;
    av[3 * i + 1] = Vy;
    av[3 * i + 2] = Vz;
}

// Gradient of a continuous field recovered from the per-tet E: the nodal
// field is the volume average of the incident tets' E, interpolated linearly
// in each tet, so its gradient is constant per tet:
// G_t[3 d + c] = sum_i E_node(i)[d] dlambda_i / dx_c. The volume of a tet is
// 1 / (6 |det M|) with M its barycentric map.
__global__ void k_node_field(const int4 *__restrict__ tet_nodes, const TetRec *__restrict__ rec,
                             const double *__restrict__ E, int64_t nt, double *__restrict__ En, double *__restrict__ Wn) {
    const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const double *M = rec[t].M;
    const double det = M[0] * (M[4] * M[8] - M[5] * M[7]) - M[1] * (M[3] * M[8] - M[5] * M[6]) +
                       M[2] * (M[3] * M[7] - M[4] * M[6]);
    const double vol = 1.0 / (6.0 * fabs(det));
    const int4 tn = tet_nodes[t];
    const int nd[4] = {tn.x, tn.y, tn.z, tn.w};
    for (int k = 0; k < 4; ++k) {
        for (int c = 0; c < 3; ++c) atomicAdd(En + 3 * int64_t(nd[k]) + c, vol * E[3 * t + c]);
        atomicAdd(Wn + nd[k], vol);
    }
}

__global__ void k_tet_field_gradient(const int4 *__restrict__ tet_nodes, const TetRec *__restrict__ rec,
                                     const double *__restrict__ En, const double *__restrict__ Wn, int64_t nt,
                                     double *__restrict__ G) {
    const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const double *M = rec[t].M;
    double gl[4][3];
    for (int c = 0; c < 3; ++c) {
        gl[1][c] = M[c];
        gl[2][c] = M[3 + c];
        gl[3][c] = M[6 + c];
        gl[0][c] = -(gl[1][c] + gl[2][c] + gl[3][c]);
    }
    const int4 tn = tet_nodes[t];
    const int nd[4] = {tn.x, tn.y, tn.z, tn.w};
    double g[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int k = 0; k < 4; ++k) {
        const double w = 1.0 / Wn[nd[k]];
        for (int d = 0; d < 3; ++d) {
            const double e = En[3 * int64_t(nd[k]) + d] * w;
            for (int c = 0; c < 3; ++c) g[3 * d + c] += e * gl[k][c];
        }
    }
    for (int q = 0; q < 9; ++q) G[9 * t + q] = g[q];
}

// dJ/dphi from dJ/dE: E = -sum_r (phi_{r+1} - phi_0) M_r.
__global__ void k_gE_to_nodes(const int4 *__restrict__ tet_nodes, const TetRec *__restrict__ rec,
                              const double *__restrict__ gE, int64_t nt, double *__restrict__ lam) {
    const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const double a0 = gE[3 * t], a1 = gE[3 * t + 1], a2 = gE[3 * t + 2];
    if (a0 == 0.0 && a1 == 0.0 && a2 == 0.0) return;
    const int4 tn = tet_nodes[t];
    const TetRec &r = rec[t];
    const double m0 = r.M[0] * a0 + r.M[1] * a1 + r.M[2] * a2;
    const double m1 = r.M[3] * a0 + r.M[4] * a1 + r.M[5] * a2;
    const double m2 = r.M[6] * a0 + r.M[7] * a1 + r.M[8] * a2;
    atomicAdd(lam + tn.x, m0 + m1 + m2);
    atomicAdd(lam + tn.y, -m0);
    atomicAdd(lam + tn.z, -m1);
    atomicAdd(lam + tn.w, -m2);
}

// b = lam on free nodes, 0 on Dirichlet nodes (adjoint right-hand side).
__global__ void k_adj_rhs(const double *__restrict__ lam, const uint8_t *__restrict__ is_dir, double *__restrict__ b,
                          double *__restrict__ x, int64_t nn) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    b[i] = is_dir[i] ? 0.0 : lam[i];
    x[i] = 0.0;
}

// dJ/dg_d = lam_d - sum_f K_fd mu_f on Dirichlet nodes (0 elsewhere).
__global__ void k_dirichlet_grad_init(const double *__restrict__ lam, const uint8_t *__restrict__ is_dir,
                                      double *__restrict__ out, int64_t nn) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    out[i] = is_dir[i] ? lam[i] : 0.0;
}

__global__ void k_dirichlet_grad_elim(const int32_t *__restrict__ er, const int32_t *__restrict__ ec,
                                      const double *__restrict__ ev, int64_t ne, const double *__restrict__ mu,
                                      double *__restrict__ out) {
    const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    atomicAdd(out + ec[e], -ev[e] * mu[er[e]]);
}

// lift_f = sum_d K_fd g_d (eliminated couplings in row order, CSR by free row).
__global__ void k_lift(const int64_t *__restrict__ erp, const int32_t *__restrict__ ec, const double *__restrict__ ev,
                       const double *__restrict__ g, double *__restrict__ lift, int64_t nn) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    double s = 0.0;
    for (int64_t e = erp[i]; e < erp[i + 1]; ++e) s += ev[e] * g[ec[e]];
    lift[i] = s;
}

__global__ void k_set_dirichlet(const uint8_t *__restrict__ is_dir, const double *__restrict__ g,
                                double *__restrict__ dir_value, double *__restrict__ phi, int64_t nn) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= nn || !is_dir[i]) return;
    dir_value[i] = g[i];
    phi[i] = g[i];
}

__global__ void k_gather_adj(const DevParticles p, int64_t n, const double *__restrict__ ax,
                             const double *__restrict__ av, double *dx, double *dv) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t id = p.idf[i] & kIdMask;
    for (int k = 0; k < 3; ++k) {
        if (dx) dx[3 * id + k] = ax[3 * i + k];
        if (dv) dv[3 * id + k] = av[3 * i + k];
    }
}

inline unsigned grid_for(int64_t n, int b) { return unsigned((n + b - 1) / b); }

}  // namespace

void launch_record(const DevParticles &p, int64_t n, const AdjHist &h, int k, cudaStream_t s) {
    if (n > 0) k_record<<<grid_for(n, 256), 256, 0, s>>>(p, n, h, k);
}
void launch_objective(const DevParticles &p, int64_t n, const LandRec *land, const double *target, double sigma,
                      double *gr, double *sums, cudaStream_t s) {
    if (n > 0)
        k_objective<<<grid_for(n, 256), 256, 0, s>>>(p, n, land, target[0], target[1], target[2],
                                                      1.0 / (2.0 * sigma * sigma), gr, sums);
}
void launch_backward(const DevParticles &p, int64_t n, const AdjHist &h, int k0, int k1, const TetRec *rec,
                     const LandRec *land, const double *gr, double gscale, double *ax, double *av, double *gE,
                     const StepConst &c, cudaStream_t s, const double *G) {
    if (n > 0)
        k_backward<<<grid_for(n, 128), 128, 0, s>>>(p, n, h, k0, k1, rec, land, gr, gscale, ax, av, gE, c,
                                                     c.charge / c.mass * c.dt, G);
}
void launch_gE_to_nodes(const int4 *tet_nodes, const TetRec *rec, const double *gE, int64_t nt, double *lam,
                        cudaStream_t s) {
    k_gE_to_nodes<<<grid_for(nt, 256), 256, 0, s>>>(tet_nodes, rec, gE, nt, lam);
}
void launch_adj_rhs(const double *lam, const uint8_t *is_dir, double *b, double *x, int64_t nn, cudaStream_t s) {
    k_adj_rhs<<<grid_for(nn, 256), 256, 0, s>>>(lam, is_dir, b, x, nn);
}
void launch_dirichlet_grad(const double *lam, const uint8_t *is_dir, const int32_t *er, const int32_t *ec,
                           const double *ev, int64_t ne, const double *mu, double *out, int64_t nn, cudaStream_t s) {
    k_dirichlet_grad_init<<<grid_for(nn, 256), 256, 0, s>>>(lam, is_dir, out, nn);
    if (ne > 0) k_dirichlet_grad_elim<<<grid_for(ne, 256), 256, 0, s>>>(er, ec, ev, ne, mu, out);
}
void launch_lift(const int64_t *erp, const int32_t *ec, const double *ev, const double *g, double *lift, int64_t nn,
                 cudaStream_t s) {
    k_lift<<<grid_for(nn, 256), 256, 0, s>>>(erp, ec, ev, g, lift, nn);
}
void launch_set_dirichlet(const uint8_t *is_dir, const double *g, double *dir_value, double *phi, int64_t nn,
                          cudaStream_t s) {
    k_set_dirichlet<<<grid_for(nn, 256), 256, 0, s>>>(is_dir, g, dir_value, phi, nn);
}
void launch_gather_adj(const DevParticles &p, int64_t n, const double *ax, const double *av, double *dx, double *dv,
                       cudaStream_t s) {
    if (n > 0) k_gather_adj<<<grid_for(n, 256), 256, 0, s>>>(p, n, ax, av, dx, dv);
}

void launch_field_gradient(const int4 *tet_nodes, const TetRec *rec, const double *E, int64_t nt, int64_t nn,
                           double *En, double *Wn, double *G, cudaStream_t s) {
    cudaMemsetAsync(En, 0, sizeof(double) * 3 * nn, s);
    cudaMemsetAsync(Wn, 0, sizeof(double) * nn, s);
    if (nt <= 0) return;
    const unsigned grid = unsigned((nt + 255) / 256);
    k_node_field<<<grid, 256, 0, s>>>(tet_nodes, rec, E, nt, En, Wn);
    k_tet_field_gradient<<<grid, 256, 0, s>>>(tet_nodes, rec, En, Wn, nt, G);
}

}  // namespace spg

