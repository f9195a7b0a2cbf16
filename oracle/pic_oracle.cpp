// CPU oracle of the PIC/DSMC time step -- TEST INFRASTRUCTURE ONLY.
//
// Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as
// the checker of libstart_gpu.so. Written independently of the GPU library; it
// shares only the public ABI structs (include/start_gpu.h).
//
// Build: g++ -O2 -std=c++17 -fopenmp -ffp-contract=off (oracle/build.py).
// -ffp-contract=off keeps every a*b+c unfused so that the collisionless push
// and walk evaluate the same IEEE operations as the GPU kernels (built with
// --fmad=false).
//
// Reference files restated here (paths within ViNN280801/Start):
//   step order         src/ParticleInCellEngine/ParticleDynamicsProcessor/ParticleDynamicsProcessor.cpp:161-200
//   push               src/Particle/Particle.cpp:196-234 (Boris, B = 0)
//   move               src/Particle/Particle.cpp:157-165
//   HS / VHS / VSS     src/Particle/PhysicsCore/CollisionModel/{HS,VHS,VSS}Model.cpp
//   VSS rotation       include/Geometry/Basics/GeometryVector.hpp:66-90,448-471
//   bbox test          src/Geometry/Mesh/Surface/SurfaceMesh.cpp:104-134
//   surface settle     ParticleSurfaceCollisionHandler.cpp:6-142, ParticleSettler.cpp:7-26
//   assembly           src/FiniteElementMethod/Assemblers/GSMAssembler.cpp:10-118
//   Dirichlet          src/FiniteElementMethod/BoundaryConditions/*.cpp (symmetric form here)
//   E field            src/Geometry/Mesh/Volumetric/VolumetricMesh.cpp:382-411 (E = -grad phi here)
//   concentration      src/Utilities/Utilities.cpp:132-149
//   seg/tri hit        src/Geometry/Utils/Intersections/SegmentTriangleIntersection.cpp:12-40
#include "pic_oracle.h"

#include <omp.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

namespace {

thread_local std::string g_err;
int g_threads = 0;

constexpr double PI = 3.14159265358979323846;
constexpr uint32_t FLAG_SETTLED = 1u, FLAG_LOST = 2u;

int fail(int code, const std::string &m) {
    g_err = m;
    return code;
}

// ---------------------------------------------------------------- Philox4x32-10
// Salmon et al., SC'11. Streams keyed by (particle id, seed low word), counter
// (step low, draw, step high, seed high word).
void philox(const uint32_t in[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = in[0], c1 = in[1], c2 = in[2], c3 = in[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = uint64_t(0xD2511F53u) * c0;
        const uint64_t p1 = uint64_t(0xCD9E8D57u) * c2;
        const uint32_t hi0 = uint32_t(p0 >> 32), lo0 = uint32_t(p0);
        const uint32_t hi1 = uint32_t(p1 >> 32), lo1 = uint32_t(p1);
        const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

double u01(uint32_t a, uint32_t b) {
    return (double(a >> 5) * 67108864.0 + double(b >> 6)) * (1.0 / 9007199254740992.0);
}

void draws(uint64_t step, uint32_t draw, uint32_t id, uint64_t seed, uint32_t out[4]) {
    const uint32_t c[4] = {uint32_t(step), draw, uint32_t(step >> 32), uint32_t(seed >> 32)};
    const uint32_t k[2] = {id, uint32_t(seed)};
    philox(c, k, out);
}

// Collision test of a step with probability P (q = 1/256): the step is a
// candidate when its byte (step & 15) of block (step >> 4, draw 2) is zero;
// P <= q: a collision iff a candidate and u_acc < 256 P (block (step, draw
// 3)); P > q: iff a candidate or else u_f < (P - q) / (1 - q) (block (step,
// draw 4)). Each step collides with probability P, independently. A
// collision's angle draws: block (step, draw 1), u1 from words 0-1, u2 from
// words 2-3.
bool collides(uint64_t step, uint32_t id, uint64_t seed, double P) {
    uint32_t b[4];
    draws(step >> 4, 2u, id, seed, b);
    const uint32_t k = uint32_t(step & 15u);
    const uint32_t byte = (b[k >> 2] >> (8u * (k & 3u))) & 0xffu;
    const double q = 1.0 / 256.0;
    uint32_t r[4];
    if (P <= q) {
        if (byte != 0u) return false;
        draws(step, 3u, id, seed, r);
        return u01(r[0], r[1]) < P * 256.0;
    }
    if (byte == 0u) return true;
    draws(step, 4u, id, seed, r);
    return u01(r[0], r[1]) < (P - q) / (1.0 - q);
}

// ---------------------------------------------------------------- geometry
// Barycentric map of a tet: lambda_{1..3} = M (p - x0); rows of M are
// (b x c)/det, (c x a)/det, (a x b)/det with a,b,c the edge vectors from x0.
double tet_map(const double *x0, const double *x1, const double *x2, const double *x3, double M[9]) {
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

struct Tet {
    double M[9];
    double x0[3];
    double E[3];
};

inline void bary(const Tet &T, const double p[3], double l[4]) {
    const double d0 = p[0] - T.x0[0], d1 = p[1] - T.x0[1], d2 = p[2] - T.x0[2];
    l[1] = T.M[0] * d0 + T.M[1] * d1 + T.M[2] * d2;
    l[2] = T.M[3] * d0 + T.M[4] * d1 + T.M[5] * d2;
    l[3] = T.M[6] * d0 + T.M[7] * d1 + T.M[8] * d2;
    l[0] = 1.0 - l[1] - l[2] - l[3];
}

}  // namespace

struct spo_handle {
    spg_params prm{};
    int64_t Nn = 0, Nt = 0, Ntri = 0, nbf = 0;
    std::vector<double> xyz;
    std::vector<int32_t> tn;  // 4*Nt oriented
    std::vector<Tet> tet;
    std::vector<double> vol, dual;
    std::vector<int32_t> nbr_t, nbr_f;  // neighbour tet / its face, -1
    std::vector<int32_t> ftri;
    // stiffness after symmetric Dirichlet elimination
    std::vector<int32_t> rp, ci;
    std::vector<double> av, diag, lift, gval;
    std::vector<std::map<int32_t, double>> elim;  // free row -> (Dirichlet col -> K_fd)
    std::vector<uint8_t> isd;
    double lo[3], hi[3];
    // location grid (tet bounding boxes)
    double go[3], gh[3];
    int gd[3];
    std::vector<int64_t> gstart;
    std::vector<int32_t> glist;
    // fields
    std::vector<double> phi, node_q;
    // particles
    int64_t np = 0;
    std::vector<double> x, v;
    std::vector<int32_t> pt;
    std::vector<uint32_t> fl;
    std::vector<uint64_t> tri_count;
    int64_t step = 0;
    int64_t processed = 0, collisions = 0, crossings = 0, settled = 0, lost = 0;
    int64_t cg_iters_total = 0;
    int32_t cg_iters_last = 0, cg_solves = 0;
    double cg_relres_last = 0.0;
    bool have_E = false;
    // field-cell freezing for spo_grad (0 off, 1 record, 2 replay)
    int freeze = 0;
    // spo_grad adds the gradient of the recovered continuous field (see spo_grad_field_gradient)
    bool field_gradient = false;
    std::vector<int32_t> frozen;
    // reference-behaviour switches (SPO_COMPAT_*), off by default
    uint32_t compat = 0;
    double cubature_w0 = 1.0 / 6.0;
    std::vector<int64_t> nt_start;   // node -> incident tets, CSR, ascending tet id
    std::vector<int32_t> nt_tets;
    std::vector<double> rho_map;     // NodeChargeDensitiesMap of the volume-average deposit
    std::vector<uint8_t> rho_has;    // node has an entry in that map
};

namespace {

// ---------------------------------------------------------------- walk
enum { W_IN = 0, W_SURF = 1, W_EXIT = 2, W_CAP = 3 };

struct Walk {
    int32_t tet;
    int status;
    int32_t tri;
    int crossings;
    double s;
    int face;  // exit face of the final tet when the walk stops on a surface
};

// The segment p0 -> p1 from tet t: stop when lambda(p1) >= 0 in all four
// coordinates; else leave through the face (not the entry face) with
// lambda(p1) < 0 and the smallest crossing parameter l0/(l0 - l1), the
// lowest face index winning ties.
Walk walk(const spo_handle &h, int32_t t, const double p0[3], const double p1[3], int max_cross, bool stop_surface) {
    Walk w{t, W_IN, -1, 0, 1.0, -1};
    int enter = -1;
    for (;;) {
        const Tet &T = h.tet[t];
        double l1[4];
        bary(T, p1, l1);
        if (l1[0] >= 0.0 && l1[1] >= 0.0 && l1[2] >= 0.0 && l1[3] >= 0.0) {
            w.tet = t;
            w.status = W_IN;
            return w;
        }
        double l0[4];
        bary(T, p0, l0);
        int best = -1;
        double sb = 0.0;
        for (int f = 0; f < 4; ++f) {
            if (f == enter || !(l1[f] < 0.0)) continue;
            const double s = l0[f] / (l0[f] - l1[f]);
            if (best < 0 || s < sb) {
                best = f;
                sb = s;
            }
        }
        if (best < 0) {
            w.tet = t;
            w.status = W_IN;
            return w;
        }
        const int32_t tri = h.ftri[4 * int64_t(t) + best];
        if (stop_surface && tri >= 0) {
            w.tet = t;
            w.status = W_SURF;
            w.tri = tri;
            w.s = sb;
            w.face = best;
            return w;
        }
        const int32_t nb = h.nbr_t[4 * int64_t(t) + best];
        if (nb < 0) {
            w.tet = t;
            w.status = W_EXIT;
            w.s = sb;
            return w;
        }
        if (w.crossings == max_cross) {
            w.tet = t;
            w.status = W_CAP;
            return w;
        }
        w.crossings++;
        enter = h.nbr_f[4 * int64_t(t) + best];
        t = nb;
    }
}

// ---------------------------------------------------------------- collisions
struct CollConst {
    double sigma_hs, c1, two_kT, mr, expo, inv_alpha, mass_cp, mass_ct;
};

CollConst coll_const(const spg_params &p) {
    CollConst c;
    c.sigma_hs = PI * std::pow(p.hs_diameter, 2);
    c.c1 = (p.vhs_dref * p.vhs_dref) / std::tgamma(5.0 / 2.0 - p.omega);
    c.two_kT = 2.0 * p.kT_ref;
    c.mr = p.mass * p.gas_mass / (p.mass + p.gas_mass);
    c.expo = p.omega - 1.0 / 2.0;
    c.inv_alpha = 1.0 / p.alpha;
    c.mass_cp = p.mass / (p.gas_mass + p.mass);
    c.mass_ct = p.gas_mass / (p.gas_mass + p.mass);
    return c;
}

double probability(const spg_params &p, const CollConst &c, const double v[3]) {
    const double vmod = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    double sigma;
    if (p.collision_model == SPG_COLL_HS) {
        sigma = c.sigma_hs;  // HSModel.cpp:12
    } else {
        // VHSModel.cpp:19-22: d^2 = dref^2/Gamma(5/2-w) (2 kT/(m_r v^2))^(w-1/2)
        const double base = c.two_kT / ((c.mr * vmod) * vmod);
        sigma = PI * (c.c1 * std::pow(base, c.expo));
    }
    return ((sigma * vmod) * p.gas_concentration) * p.dt;
}

// Post-collision velocity for the reference's laws given the two angle draws.
void scatter(const spg_params &p, const CollConst &c, double v[3], double u1, double u2) {
    double xi_cos;
    if (p.collision_model == SPG_COLL_HS)
        xi_cos = -1.0 + 2.0 * u1;  // HSModel.cpp:22, rng(-1, 1)
    else if (p.collision_model == SPG_COLL_VHS)
        xi_cos = u1;  // VHSModel.cpp:31, rng() in [0, 1)
    else
        xi_cos = 2.0 * std::pow(u1, c.inv_alpha) - 1.0;  // VSSModel.cpp:32
    const double xi_sin = std::sqrt(1.0 - xi_cos * xi_cos);
    const double ph = (2.0 * PI) * u2;
    const double nx = xi_sin * std::cos(ph), ny = xi_sin * std::sin(ph), nz = xi_cos;
    const double cm[3] = {v[0] * c.mass_cp, v[1] * c.mass_cp, v[2] * c.mass_cp};
    const double pv[3] = {c.mass_ct * v[0], c.mass_ct * v[1], c.mass_ct * v[2]};
    const double mp = std::sqrt(pv[0] * pv[0] + pv[1] * pv[1] + pv[2] * pv[2]);
    double e[3] = {nx * mp, ny * mp, nz * mp};
    if (p.collision_model == SPG_COLL_VSS) {
        const double beta = std::acos(pv[2] / mp), gamma = std::atan2(pv[1], pv[0]);
        const double cb = std::cos(beta), sb = std::sin(beta);
        const double tx = cb * e[0] + sb * e[2], tz = -sb * e[0] + cb * e[2];  // _rotate_y
        e[0] = tx;
        e[2] = tz;
        const double cg = std::cos(gamma), sg = std::sin(gamma);
        const double ux = cg * e[0] - sg * e[1], uy = sg * e[0] + cg * e[1];  // _rotate_z
        e[0] = ux;
        e[1] = uy;
    }
    v[0] = e[0] + cm[0];
    v[1] = e[1] + cm[1];
    v[2] = e[2] + cm[2];
}

// ---------------------------------------------------------------- one particle
struct StepOut {
    int processed, coll, cross, settled, lost;
};

StepOut step_particle(spo_handle &h, const CollConst &cc, int64_t i, int32_t ecell = -1) {
    StepOut o{0, 0, 0, 0, 0};
    if (h.fl[i] & (FLAG_SETTLED | FLAG_LOST)) return o;  // 1. settled
    o.processed = 1;
    const spg_params &p = h.prm;
    double *x = &h.x[3 * i], *v = &h.v[3 * i];
    const double vmod = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (vmod < p.min_velocity) return o;  // 2. slow
    const bool inside = x[0] >= h.lo[0] && x[0] <= h.hi[0] && x[1] >= h.lo[1] && x[1] <= h.hi[1] &&
                        x[2] >= h.lo[2] && x[2] <= h.hi[2];
    if (!inside) return o;  // 3. outside the modelling space
    const int32_t t = h.pt[i];
    const Tet &T = h.tet[ecell >= 0 ? ecell : t];
    // 4. push: a = qE/m; v- = v + a dt/2; (rotation = identity for B = 0); v = v+ + a dt/2
    // SPO_COMPAT_PUSH_NEVER: the reference finds the pushing tet by particle id
    // in the tracker filled by gather, whose entries are copies with new ids
    // (Particle.cpp:113-155, CubicGrid.cpp:149-158), so it never pushes.
    if (!(h.compat & SPO_COMPAT_PUSH_NEVER) && !(T.E[0] == 0.0 && T.E[1] == 0.0 && T.E[2] == 0.0)) {
        for (int k = 0; k < 3; ++k) {
            const double a = (p.charge * T.E[k]) / p.mass;
            const double half = (a * p.dt) / 2.0;
            v[k] = (v[k] + half) + half;
        }
    }
    // 6. move. SPO_COMPAT_MIXED_UNITS: the reference adds v dt in metres to
    // coordinates in millimetres (Particle.cpp:157-165), a displacement of
    // v dt / 1000 in SI.
    const double p0[3] = {x[0], x[1], x[2]};
    const double dtm = (h.compat & SPO_COMPAT_MIXED_UNITS) ? p.dt * 1e-3 : p.dt;
    const double p1[3] = {x[0] + v[0] * dtm, x[1] + v[1] * dtm, x[2] + v[2] * dtm};
    if (p1[0] == p0[0] && p1[1] == p0[1] && p1[2] == p0[2]) return o;  // degenerate segment
    // 7. gas collision
    if (p.collision_model != SPG_COLL_NONE) {
        const double P = probability(p, cc, v);
        if (collides(uint64_t(h.step), uint32_t(i), p.seed, P)) {
            uint32_t r[4];
            draws(uint64_t(h.step), 1u, uint32_t(i), p.seed, r);
            scatter(p, cc, v, u01(r[0], r[1]), u01(r[2], r[3]));
            o.coll = 1;
        }
    }
    if (!(std::isfinite(p1[0]) && std::isfinite(p1[1]) && std::isfinite(p1[2]))) {
        h.fl[i] |= FLAG_LOST;
        o.lost = 1;
        return o;
    }
    // 8. surface: first triangle crossed along the segment settles the particle
    const Walk w = walk(h, t, p0, p1, p.max_crossings, true);
    o.cross = w.crossings;
    if (w.status == W_IN) {
        x[0] = p1[0];
        x[1] = p1[1];
        x[2] = p1[2];
    } else if (w.status == W_SURF) {
        x[0] = p0[0] + w.s * (p1[0] - p0[0]);
        x[1] = p0[1] + w.s * (p1[1] - p0[1]);
        x[2] = p0[2] + w.s * (p1[2] - p0[2]);
#pragma omp atomic
        h.tri_count[w.tri]++;
        h.fl[i] |= FLAG_SETTLED;
        o.settled = 1;
    } else {
        x[0] = p1[0];
        x[1] = p1[1];
        x[2] = p1[2];
        h.fl[i] |= FLAG_LOST;
        o.lost = 1;
    }
    h.pt[i] = w.tet;
    return o;
}

void process_range(spo_handle &h, int64_t first, int64_t count) {
    const CollConst cc = coll_const(h.prm);
    int64_t pr = 0, co = 0, cr = 0, se = 0, lo = 0;
    const int nth = g_threads > 0 ? g_threads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 256) num_threads(nth) reduction(+ : pr, co, cr, se, lo)
    for (int64_t i = first; i < first + count; ++i) {
        const StepOut o = step_particle(h, cc, i);
        pr += o.processed;
        co += o.coll;
        cr += o.cross;
        se += o.settled;
        lo += o.lost;
    }
    h.processed += pr;
    h.collisions += co;
    h.crossings += cr;
    h.settled += se;
    h.lost += lo;
}

// ---------------------------------------------------------------- linear algebra
// Dot product with fixed 4096-element blocks, partials summed in order: the
// result does not depend on the thread count.
double dot(const std::vector<double> &a, const std::vector<double> &b) {
    const int64_t n = int64_t(a.size());
    const int64_t nb = (n + 4095) / 4096;
    std::vector<double> part(nb, 0.0);
    const int nth = g_threads > 0 ? g_threads : omp_get_max_threads();
#pragma omp parallel for num_threads(nth)
    for (int64_t k = 0; k < nb; ++k) {
        double s = 0.0;
        const int64_t e = std::min(n, (k + 1) * 4096);
        for (int64_t i = k * 4096; i < e; ++i) s += a[i] * b[i];
        part[k] = s;
    }
    double s = 0.0;
    for (double x : part) s += x;
    return s;
}

void spmv(const spo_handle &h, const std::vector<double> &x, std::vector<double> &y) {
    const int nth = g_threads > 0 ? g_threads : omp_get_max_threads();
#pragma omp parallel for schedule(static, 4096) num_threads(nth)
    for (int64_t i = 0; i < h.Nn; ++i) {
        double s = 0.0;
        for (int32_t k = h.rp[i]; k < h.rp[i + 1]; ++k) s += h.av[k] * x[h.ci[k]];
        y[i] = s;
    }
}

// Jacobi-preconditioned CG, warm started from phi.
int pcg(spo_handle &h, const std::vector<double> &b, int32_t *iters, double *relres) {
    const int64_t n = h.Nn;
    std::vector<double> r(n), z(n), pv(n), q(n);
    spmv(h, h.phi, q);
    for (int64_t i = 0; i < n; ++i) {
        r[i] = b[i] - q[i];
        z[i] = r[i] / h.diag[i];
        pv[i] = z[i];
    }
    double rz = dot(r, z);
    const double bb = dot(b, b);
    double rr = dot(r, r);
    const double tol2 = h.prm.cg_rtol * h.prm.cg_rtol * bb;
    int it = 0;
    bool ok = rr <= tol2 || bb == 0.0;
    while (!ok && it < h.prm.cg_max_iter) {
        spmv(h, pv, q);
        const double pq = dot(pv, q);
        if (!(pq > 0.0)) break;
        const double alpha = rz / pq;
        for (int64_t i = 0; i < n; ++i) {
            h.phi[i] += alpha * pv[i];
            r[i] -= alpha * q[i];
            z[i] = r[i] / h.diag[i];
        }
        ++it;
        rr = dot(r, r);
        if (rr <= tol2) {
            ok = true;
            break;
        }
        const double rz2 = dot(r, z);
        const double beta = rz2 / rz;
        rz = rz2;
        for (int64_t i = 0; i < n; ++i) pv[i] = z[i] + beta * pv[i];
    }
    *iters = it;
    *relres = bb > 0.0 ? std::sqrt(rr / bb) : 0.0;
    return ok ? SPG_OK : SPG_E_NOT_CONVERGED;
}

void compute_E(spo_handle &h) {
    const bool ref = h.compat & SPO_COMPAT_E_SIGN_SCALE;
    for (int64_t t = 0; t < h.Nt; ++t) {
        const int32_t *n = &h.tn[4 * t];
        const double d1 = h.phi[n[1]] - h.phi[n[0]], d2 = h.phi[n[2]] - h.phi[n[0]], d3 = h.phi[n[3]] - h.phi[n[0]];
        Tet &T = h.tet[t];
        if (ref) {
            // VolumetricMesh.cpp:371-375,398: E = + sum phi_i grad(N_i) |det J| w0,
            // the basis gradients weighted by the measure of cubature point 0
            const double meas = (6.0 * h.vol[t]) * h.cubature_w0;
            for (int k = 0; k < 3; ++k) T.E[k] = ((d1 * T.M[k] + d2 * T.M[3 + k]) + d3 * T.M[6 + k]) * meas;
        } else {
            for (int k = 0; k < 3; ++k) T.E[k] = -((d1 * T.M[k] + d2 * T.M[3 + k]) + d3 * T.M[6 + k]);
        }
    }
    h.have_E = true;
}

// All tets whose closed cell holds p (a point on a face, edge or vertex lies
// in every tet sharing it), from the location grid.
void tets_containing(const spo_handle &h, const double p[3], std::vector<int32_t> &out) {
    out.clear();
    int c[3];
    for (int k = 0; k < 3; ++k) {
        const double u = (p[k] - h.go[k]) / h.gh[k];
        if (!(u >= 0.0) || u >= double(h.gd[k]) + 1e-9) return;
        c[k] = std::min(h.gd[k] - 1, int(u));
    }
    const int64_t cell = c[0] + int64_t(h.gd[0]) * (c[1] + int64_t(h.gd[1]) * c[2]);
    for (int64_t k = h.gstart[cell]; k < h.gstart[cell + 1]; ++k) {
        const int32_t t = h.glist[k];
        double l[4];
        bary(h.tet[t], p, l);
        if (l[0] >= 0.0 && l[1] >= 0.0 && l[2] >= 0.0 && l[3] >= 0.0) out.push_back(t);
    }
    std::sort(out.begin(), out.end());
}

// SPO_COMPAT_DEPOSIT_VOLAVG: NodeChargeDensityProcessor.cpp:25-113 with one
// chunk (the single-thread std path). The charge of each tet's particles over
// its volume, rho_t = sum q / V_t; then per node the volume average over its
// occupied tets, rho_n = sum rho_t V_t / sum V_t, written into a map that
// lives as long as the run (ModelingMainDriver.cpp:122): a node with no
// occupied tet keeps its last density. The particle's tet is its walk tet, or
// with SPO_COMPAT_CLOSED_TETS every tet whose closed cell holds it
// (VolumetricMesh.cpp:23-33; no break at NodeChargeDensityProcessor.cpp:52-55).
void deposit_volavg(spo_handle &h) {
    const double wq = h.prm.weight * h.prm.charge;
    std::vector<double> tq(h.Nt, 0.0);
    std::vector<uint8_t> occ(h.Nt, 0);
    std::vector<int32_t> hold;
    for (int64_t i = 0; i < h.np; ++i) {
        if (h.fl[i] & (FLAG_SETTLED | FLAG_LOST)) continue;
        if (h.compat & SPO_COMPAT_CLOSED_TETS) {
            tets_containing(h, &h.x[3 * i], hold);
        } else {
            hold.assign(1, h.pt[i]);
        }
        for (int32_t t : hold) {
            tq[t] += wq;
            occ[t] = 1;
        }
    }
    for (int64_t n = 0; n < h.Nn; ++n) {
        double charge = 0.0, volume = 0.0;
        for (int64_t k = h.nt_start[n]; k < h.nt_start[n + 1]; ++k) {
            const int32_t t = h.nt_tets[k];
            if (!occ[t]) continue;
            const double rho_t = tq[t] / h.vol[t];
            charge += rho_t * h.vol[t];
            volume += h.vol[t];
        }
        if (volume > 0.0) {
            h.rho_map[n] = charge / volume;
            h.rho_has[n] = 1;
        }
    }
    for (int64_t n = 0; n < h.Nn; ++n) h.node_q[n] = h.rho_has[n] ? h.rho_map[n] * h.dual[n] : 0.0;
}

void deposit(spo_handle &h) {
    if (h.compat & SPO_COMPAT_DEPOSIT_VOLAVG) {
        deposit_volavg(h);
        return;
    }
    std::fill(h.node_q.begin(), h.node_q.end(), 0.0);
    const double wq = h.prm.weight * h.prm.charge;
    for (int64_t i = 0; i < h.np; ++i) {
        if (h.fl[i] & (FLAG_SETTLED | FLAG_LOST)) continue;
        const int32_t t = h.pt[i];
        double l[4];
        bary(h.tet[t], &h.x[3 * i], l);
        for (int k = 0; k < 4; ++k) h.node_q[h.tn[4 * int64_t(t) + k]] += wq * l[k];
    }
}

int solve_current(spo_handle &h) {
    std::vector<double> b(h.Nn);
    const double inv_eps0 = 1.0 / h.prm.epsilon0;
    if (h.compat & SPO_COMPAT_RHS_RAW_RHO) {
        // ChargeDensityEquationSolver.cpp:17-29 and VectorBoundaryConditionsManager.cpp:29-43:
        // b_i = rho_i (no eps0, no volume) at the free nodes, b_i = V at the
        // Dirichlet nodes, whose rows are identity rows with their columns kept
        // (MatrixBoundaryConditionsManager.cpp): the same solution as moving
        // K_FD g to the right-hand side. A new solver per call starts from
        // x = 0 (MatrixEquationSolver.cpp:5-11).
        for (int64_t i = 0; i < h.Nn; ++i) b[i] = h.isd[i] ? h.gval[i] : h.node_q[i] / h.dual[i] - h.lift[i];
        std::fill(h.phi.begin(), h.phi.end(), 0.0);
    } else {
        for (int64_t i = 0; i < h.Nn; ++i) b[i] = h.isd[i] ? h.gval[i] : h.node_q[i] * inv_eps0 - h.lift[i];
    }
    int32_t it = 0;
    double rr = 0.0;
    const int rc = pcg(h, b, &it, &rr);
    compute_E(h);
    h.cg_iters_last = it;
    h.cg_iters_total += it;
    h.cg_solves++;
    h.cg_relres_last = rr;
    return rc;
}

int32_t locate_one(const spo_handle &h, const double p[3]) {
    int c[3];
    for (int k = 0; k < 3; ++k) {
        const double u = (p[k] - h.go[k]) / h.gh[k];
        if (!(u >= 0.0) || u >= double(h.gd[k]) + 1e-9) return -1;
        c[k] = std::min(h.gd[k] - 1, int(u));
    }
    const int64_t cell = c[0] + int64_t(h.gd[0]) * (c[1] + int64_t(h.gd[1]) * c[2]);
    int32_t best = -1;
    for (int64_t k = h.gstart[cell]; k < h.gstart[cell + 1]; ++k) {
        const int32_t t = h.glist[k];
        double l[4];
        bary(h.tet[t], p, l);
        if (l[0] >= 0.0 && l[1] >= 0.0 && l[2] >= 0.0 && l[3] >= 0.0 && (best < 0 || t < best)) best = t;
    }
    return best;
}

}  // namespace

extern "C" {

const char *spo_last_error(void) { return g_err.c_str(); }
int spo_set_threads(int n) {
    g_threads = n;
    return 0;
}
int spo_get_threads(void) { return g_threads > 0 ? g_threads : omp_get_max_threads(); }

int spo_create(const spg_mesh_desc *d, const spg_params *prm, spo_handle **out) {
    if (!d || !prm || !out) return fail(SPG_E_INVALID, "null argument");
    *out = nullptr;
    if (d->n_nodes <= 0 || d->n_tets <= 0) return fail(SPG_E_INVALID, "empty mesh");
    auto *h = new spo_handle();
    h->prm = *prm;
    h->Nn = d->n_nodes;
    h->Nt = d->n_tets;
    h->Ntri = d->n_triangles;
    h->xyz.assign(d->node_xyz, d->node_xyz + 3 * h->Nn);
    h->tn.assign(d->tet_nodes, d->tet_nodes + 4 * h->Nt);
    h->tet.resize(h->Nt);
    h->vol.resize(h->Nt);
    for (int64_t t = 0; t < h->Nt; ++t) {
        int32_t *n = &h->tn[4 * t];
        for (int k = 0; k < 4; ++k)
            if (n[k] < 0 || n[k] >= h->Nn) {
                delete h;
                return fail(SPG_E_BAD_MESH, "bad node index");
            }
        double M[9];
        double det = tet_map(&h->xyz[3 * n[0]], &h->xyz[3 * n[1]], &h->xyz[3 * n[2]], &h->xyz[3 * n[3]], M);
        if (det < 0.0) {
            std::swap(n[2], n[3]);
            det = tet_map(&h->xyz[3 * n[0]], &h->xyz[3 * n[1]], &h->xyz[3 * n[2]], &h->xyz[3 * n[3]], M);
        }
        if (!(det > 0.0)) {
            delete h;
            return fail(SPG_E_BAD_MESH, "zero-volume tet");
        }
        std::memcpy(h->tet[t].M, M, sizeof(M));
        for (int k = 0; k < 3; ++k) {
            h->tet[t].x0[k] = h->xyz[3 * n[0] + k];
            h->tet[t].E[k] = 0.0;
        }
        h->vol[t] = det / 6.0;
    }
    // faces: sorted node triple -> (tet, local face)
    std::vector<std::tuple<int32_t, int32_t, int32_t, int32_t>> faces;
    faces.reserve(4 * h->Nt);
    for (int64_t t = 0; t < h->Nt; ++t)
        for (int f = 0; f < 4; ++f) {
            std::array<int32_t, 3> v;
            int k = 0;
            for (int j = 0; j < 4; ++j)
                if (j != f) v[k++] = h->tn[4 * t + j];
            std::sort(v.begin(), v.end());
            faces.emplace_back(v[0], v[1], v[2], int32_t(4 * t + f));
        }
    std::sort(faces.begin(), faces.end());
    h->nbr_t.assign(4 * h->Nt, -1);
    h->nbr_f.assign(4 * h->Nt, -1);
    for (size_t a = 0; a < faces.size();) {
        size_t b = a + 1;
        while (b < faces.size() && std::get<0>(faces[b]) == std::get<0>(faces[a]) &&
               std::get<1>(faces[b]) == std::get<1>(faces[a]) && std::get<2>(faces[b]) == std::get<2>(faces[a]))
            ++b;
        if (b - a == 2) {
            const int32_t f0 = std::get<3>(faces[a]), f1 = std::get<3>(faces[a + 1]);
            h->nbr_t[f0] = f1 >> 2;
            h->nbr_f[f0] = f1 & 3;
            h->nbr_t[f1] = f0 >> 2;
            h->nbr_f[f1] = f0 & 3;
        } else if (b - a == 1) {
            h->nbf++;
        } else {
            delete h;
            return fail(SPG_E_BAD_MESH, "non-manifold face");
        }
        a = b;
    }
    h->ftri.assign(4 * h->Nt, -1);
    for (int64_t k = 0; k < h->Ntri; ++k) {
        std::array<int32_t, 3> v = {d->tri_nodes[3 * k], d->tri_nodes[3 * k + 1], d->tri_nodes[3 * k + 2]};
        std::sort(v.begin(), v.end());
        auto it = std::lower_bound(faces.begin(), faces.end(), std::make_tuple(v[0], v[1], v[2], int32_t(-1)));
        int hits = 0;
        for (; it != faces.end() && std::get<0>(*it) == v[0] && std::get<1>(*it) == v[1] && std::get<2>(*it) == v[2];
             ++it) {
            h->ftri[std::get<3>(*it)] = int32_t(k);
            hits++;
        }
        if (!hits) {
            delete h;
            return fail(SPG_E_BAD_MESH, "triangle is not a tet face");
        }
    }
    faces.clear();
    faces.shrink_to_fit();
    // Dirichlet values
    h->isd.assign(h->Nn, 0);
    h->gval.assign(h->Nn, 0.0);
    for (int64_t k = 0; k < d->n_dirichlet; ++k) {
        const int32_t n = d->dirichlet_nodes[k];
        if (n < 0 || n >= h->Nn) {
            delete h;
            return fail(SPG_E_INVALID, "Dirichlet node out of range");
        }
        h->isd[n] = 1;
        h->gval[n] = d->dirichlet_values[k];
    }
    // dual volumes and stiffness via node -> incident tets
    std::vector<std::vector<int32_t>> inc(h->Nn);
    for (int64_t t = 0; t < h->Nt; ++t)
        for (int k = 0; k < 4; ++k) inc[h->tn[4 * t + k]].push_back(int32_t(4 * t + k));
    h->dual.assign(h->Nn, 0.0);
    h->nt_start.assign(h->Nn + 1, 0);
    for (int64_t n = 0; n < h->Nn; ++n) {
        double s = 0.0;
        for (int32_t e : inc[n]) s += h->vol[e >> 2];
        h->dual[n] = 0.25 * s;
        h->nt_start[n + 1] = h->nt_start[n] + int64_t(inc[n].size());
    }
    h->nt_tets.resize(size_t(h->nt_start[h->Nn]));
    for (int64_t n = 0; n < h->Nn; ++n)
        for (size_t k = 0; k < inc[n].size(); ++k) h->nt_tets[size_t(h->nt_start[n]) + k] = inc[n][k] >> 2;
    h->rp.assign(h->Nn + 1, 0);
    std::vector<std::map<int32_t, double>> rows(h->Nn);
    h->lift.assign(h->Nn, 0.0);
    h->elim.assign(h->Nn, {});
    h->diag.assign(h->Nn, 1.0);
#pragma omp parallel for schedule(dynamic, 512)
    for (int64_t i = 0; i < h->Nn; ++i) {
        if (h->isd[i]) {
            rows[i][int32_t(i)] = 1.0;
            continue;
        }
        double lift = 0.0;
        for (int32_t e : inc[i]) {
            const int64_t t = e >> 2;
            const int a = e & 3;
            const Tet &T = h->tet[t];
            double G[4][3];
            for (int c = 0; c < 3; ++c) {
                G[1][c] = T.M[c];
                G[2][c] = T.M[3 + c];
                G[3][c] = T.M[6 + c];
                G[0][c] = -(G[1][c] + G[2][c] + G[3][c]);
            }
            for (int b = 0; b < 4; ++b) {
                const double kab = h->vol[t] * (G[a][0] * G[b][0] + G[a][1] * G[b][1] + G[a][2] * G[b][2]);
                const int32_t j = h->tn[4 * t + b];
                if (h->isd[j]) {
                    lift += kab * h->gval[j];
                    h->elim[i][j] += kab;
                } else {
                    rows[i][j] += kab;
                }
            }
        }
        h->lift[i] = lift;
    }
    for (int64_t i = 0; i < h->Nn; ++i) h->rp[i + 1] = h->rp[i] + int32_t(rows[i].size());
    h->ci.resize(h->rp[h->Nn]);
    h->av.resize(h->rp[h->Nn]);
    for (int64_t i = 0; i < h->Nn; ++i) {
        int32_t k = h->rp[i];
        for (auto &kv : rows[i]) {
            h->ci[k] = kv.first;
            h->av[k] = kv.second;
            if (kv.first == i) h->diag[i] = kv.second;
            ++k;
        }
        std::map<int32_t, double>().swap(rows[i]);
    }
    // modelling-space box from the surface triangles (SurfaceMesh.cpp:92-134)
    double blo[3] = {HUGE_VAL, HUGE_VAL, HUGE_VAL}, bhi[3] = {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL};
    const int64_t nb = h->Ntri > 0 ? 3 * h->Ntri : h->Nn;
    for (int64_t k = 0; k < nb; ++k) {
        const int64_t n = h->Ntri > 0 ? d->tri_nodes[k] : k;
        for (int c = 0; c < 3; ++c) {
            blo[c] = std::min(blo[c], h->xyz[3 * n + c]);
            bhi[c] = std::max(bhi[c], h->xyz[3 * n + c]);
        }
    }
    for (int c = 0; c < 3; ++c) {
        const double centre = (blo[c] + bhi[c]) / 2.0;
        const double half = ((bhi[c] - blo[c]) / 2.0) * prm->bbox_expansion;
        h->lo[c] = centre - half;
        h->hi[c] = centre + half;
    }
    // location grid over the node box, tets listed in every cell their bbox touches
    double nlo[3] = {HUGE_VAL, HUGE_VAL, HUGE_VAL}, nhi[3] = {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL};
    for (int64_t n = 0; n < h->Nn; ++n)
        for (int c = 0; c < 3; ++c) {
            nlo[c] = std::min(nlo[c], h->xyz[3 * n + c]);
            nhi[c] = std::max(nhi[c], h->xyz[3 * n + c]);
        }
    const double g = std::cbrt(2.0 * (nhi[0] - nlo[0]) * (nhi[1] - nlo[1]) * (nhi[2] - nlo[2]) / double(h->Nt) * 6.0);
    int64_t ncell = 1;
    for (int c = 0; c < 3; ++c) {
        const double ext = std::max(nhi[c] - nlo[c], 1e-30);
        h->gd[c] = int(std::max(1.0, std::min(512.0, std::floor(ext / g))));
        h->gh[c] = ext / h->gd[c];
        h->go[c] = nlo[c];
        ncell *= h->gd[c];
    }
    std::vector<std::vector<int32_t>> cells(ncell);
    for (int64_t t = 0; t < h->Nt; ++t) {
        int c0[3], c1[3];
        for (int c = 0; c < 3; ++c) {
            double mn = HUGE_VAL, mx = -HUGE_VAL;
            for (int k = 0; k < 4; ++k) {
                mn = std::min(mn, h->xyz[3 * h->tn[4 * t + k] + c]);
                mx = std::max(mx, h->xyz[3 * h->tn[4 * t + k] + c]);
            }
            c0[c] = std::max(0, std::min(h->gd[c] - 1, int(std::floor((mn - h->go[c]) / h->gh[c] - 1e-9))));
            c1[c] = std::max(0, std::min(h->gd[c] - 1, int(std::floor((mx - h->go[c]) / h->gh[c] + 1e-9))));
        }
        for (int k = c0[2]; k <= c1[2]; ++k)
            for (int j = c0[1]; j <= c1[1]; ++j)
                for (int i = c0[0]; i <= c1[0]; ++i)
                    cells[i + int64_t(h->gd[0]) * (j + int64_t(h->gd[1]) * k)].push_back(int32_t(t));
    }
    h->gstart.assign(ncell + 1, 0);
    for (int64_t c = 0; c < ncell; ++c) h->gstart[c + 1] = h->gstart[c] + int64_t(cells[c].size());
    h->glist.resize(h->gstart[ncell]);
    for (int64_t c = 0; c < ncell; ++c) std::copy(cells[c].begin(), cells[c].end(), h->glist.begin() + h->gstart[c]);
    h->phi = h->gval;
    h->node_q.assign(h->Nn, 0.0);
    h->tri_count.assign(h->Ntri, 0);
    *out = h;
    return SPG_OK;
}

void spo_destroy(spo_handle *h) { delete h; }

int spo_mesh_info(const spo_handle *h, int64_t info[6]) {
    info[0] = h->Nn;
    info[1] = h->Nt;
    info[2] = h->Ntri;
    info[3] = h->nbf;
    info[4] = int64_t(h->ci.size());
    int64_t nd = 0;
    for (uint8_t b : h->isd) nd += b;
    info[5] = nd;
    return SPG_OK;
}

int spo_locate(spo_handle *h, int64_t n, const double *pos, int32_t *tet_out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) tet_out[i] = locate_one(*h, &pos[3 * i]);
    return SPG_OK;
}

int spo_set_particles(spo_handle *h, int64_t n, const double *pos, const double *vel, const int32_t *tet) {
    if (n < 0 || n > (int64_t(1) << 28)) return fail(SPG_E_INVALID, "n out of range");
    h->np = n;
    h->x.assign(pos, pos + 3 * n);
    h->v.assign(vel, vel + 3 * n);
    h->pt.assign(n, -1);
    if (tet)
        for (int64_t i = 0; i < n; ++i) h->pt[i] = tet[i] < h->Nt ? tet[i] : -1;
    else
        spo_locate(h, n, pos, h->pt.data());
    h->fl.assign(n, 0);
    int64_t lost = 0;
    for (int64_t i = 0; i < n; ++i)
        if (h->pt[i] < 0) {
            h->fl[i] = FLAG_LOST;
            lost++;
        }
    h->step = 0;
    h->processed = h->collisions = h->crossings = h->settled = 0;
    h->lost = lost;
    h->cg_iters_total = 0;
    h->cg_iters_last = h->cg_solves = 0;
    h->cg_relres_last = 0.0;
    std::fill(h->tri_count.begin(), h->tri_count.end(), 0);
    h->phi = h->gval;
    std::fill(h->node_q.begin(), h->node_q.end(), 0.0);
    for (auto &T : h->tet) T.E[0] = T.E[1] = T.E[2] = 0.0;
    h->have_E = false;
    return SPG_OK;
}

int spo_get_particles(spo_handle *h, int64_t n, double *pos, double *vel, int32_t *tet, uint32_t *flags) {
    if (n != h->np) return fail(SPG_E_INVALID, "count mismatch");
    if (pos) std::copy(h->x.begin(), h->x.end(), pos);
    if (vel) std::copy(h->v.begin(), h->v.end(), vel);
    if (tet) std::copy(h->pt.begin(), h->pt.end(), tet);
    if (flags) std::copy(h->fl.begin(), h->fl.end(), flags);
    return SPG_OK;
}

int spo_gather(spo_handle *h, double *rho_out) {
    deposit(*h);
    if (rho_out)
        for (int64_t i = 0; i < h->Nn; ++i) rho_out[i] = h->node_q[i] / h->dual[i];
    return SPG_OK;
}

int spo_solve(spo_handle *h, const double *rho, double *phi_out, int32_t *iters, double *relres) {
    if (rho)
        for (int64_t i = 0; i < h->Nn; ++i) h->node_q[i] = rho[i] * h->dual[i];
    const int rc = solve_current(*h);
    if (iters) *iters = h->cg_iters_last;
    if (relres) *relres = h->cg_relres_last;
    if (phi_out) std::copy(h->phi.begin(), h->phi.end(), phi_out);
    if (rc) g_err = "PCG did not converge";
    return rc;
}

int spo_process(spo_handle *h, int32_t nsteps) {
    for (int32_t s = 0; s < nsteps; ++s) {
        process_range(*h, 0, h->np);
        h->step++;
    }
    return SPG_OK;
}

int spo_process_range(spo_handle *h, int64_t first, int64_t count) {
    if (first < 0 || count < 0 || first + count > h->np) return fail(SPG_E_INVALID, "range");
    process_range(*h, first, count);
    return SPG_OK;
}

int spo_run(spo_handle *h, int32_t nsteps) {
    int status = SPG_OK;
    for (int32_t s = 0; s < nsteps; ++s) {
        // SPO_COMPAT_SOLVE_EVERY_STEP: gather and solve at every time moment
        // (ModelingMainDriver.cpp:146-161)
        if (h->step % h->prm.poisson_every == 0 || (h->compat & SPO_COMPAT_SOLVE_EVERY_STEP)) {
            deposit(*h);
            const int rc = solve_current(*h);
            if (rc) status = rc;
        }
        process_range(*h, 0, h->np);
        h->step++;
    }
    return status;
}

int spo_get_stats(spo_handle *h, spg_stats *st) {
    st->step = h->step;
    st->n_particles = h->np;
    st->n_settled = h->settled;
    st->n_lost = h->lost;
    st->n_alive = h->np - h->settled - h->lost;
    st->particle_steps = h->processed;
    st->collisions = h->collisions;
    st->crossings = h->crossings;
    st->cg_iters_total = h->cg_iters_total;
    st->cg_iters_last = h->cg_iters_last;
    st->cg_solves = h->cg_solves;
    st->cg_relres_last = h->cg_relres_last;
    return SPG_OK;
}

int spo_get_triangle_counts(spo_handle *h, uint64_t *c) {
    std::copy(h->tri_count.begin(), h->tri_count.end(), c);
    return SPG_OK;
}

int spo_get_potential(spo_handle *h, double *phi) {
    std::copy(h->phi.begin(), h->phi.end(), phi);
    return SPG_OK;
}

int spo_set_potential(spo_handle *h, const double *phi) {
    h->phi.assign(phi, phi + h->Nn);
    compute_E(*h);
    return SPG_OK;
}

int spo_get_efield(spo_handle *h, double *E) {
    for (int64_t t = 0; t < h->Nt; ++t)
        for (int k = 0; k < 3; ++k) E[3 * t + k] = h->tet[t].E[k];
    return SPG_OK;
}

int spo_get_matrix(spo_handle *h, int32_t *row_ptr, int32_t *col, double *val, double *lift) {
    if (row_ptr) std::copy(h->rp.begin(), h->rp.end(), row_ptr);
    if (col) std::copy(h->ci.begin(), h->ci.end(), col);
    if (val) std::copy(h->av.begin(), h->av.end(), val);
    if (lift) std::copy(h->lift.begin(), h->lift.end(), lift);
    return SPG_OK;
}

int spo_get_dual_volumes(spo_handle *h, double *dv) {
    std::copy(h->dual.begin(), h->dual.end(), dv);
    return SPG_OK;
}

int spo_set_dirichlet(spo_handle *h, const double *g) {
    for (int64_t i = 0; i < h->Nn; ++i)
        if (h->isd[i]) {
            h->gval[i] = g[i];
            h->phi[i] = g[i];
        }
    for (int64_t i = 0; i < h->Nn; ++i) {
        double s = 0.0;
        for (const auto &e : h->elim[i]) s += e.second * h->gval[e.first];
        h->lift[i] = s;
    }
    return SPG_OK;
}

// FP64 reference gradient of J = (1/N) sum_landed exp(-|r - t|^2/(2 s^2)):
// the forward keeps every particle's full history (tet and velocity at the
// start of each step), then the backward recursion of the particle adjoint,
// dJ/dE -> dJ/dphi, one adjoint PCG and the transpose of the lifting.
int spo_grad(spo_handle *h, int32_t nsteps, const double *target, double sigma, double *J, int64_t *n_landed,
             double *dJ_dg, double *dJ_dx0, double *dJ_dv0) {
    const spg_params &p = h->prm;
    if (p.collision_model == SPG_COLL_VSS) return fail(SPG_E_INVALID, "VSS has no adjoint");
    const int64_t n = h->np;
    std::vector<int32_t> htet(size_t(nsteps) * n);
    std::vector<double> hv(size_t(nsteps) * n * 3);
    std::vector<int32_t> land_step(n, -1), land_tet(n, -1), land_face(n, -1);
    std::vector<double> land_s(n, 0.0);
    const CollConst cc = coll_const(p);
    const int64_t step0 = h->step;
    const bool replay = h->freeze == 2 && h->frozen.size() == htet.size();
    for (int32_t k = 0; k < nsteps; ++k) {
        for (int64_t i = 0; i < n; ++i) {
            const size_t o = size_t(k) * n + i;
            const int32_t ec = replay && h->frozen[o] >= 0 ? h->frozen[o] : h->pt[i];
            htet[o] = (h->fl[i] & (FLAG_SETTLED | FLAG_LOST)) ? -1 : ec;
            for (int c = 0; c < 3; ++c) hv[3 * o + c] = h->v[3 * i + c];
        }
        // one step, remembering where a settle happened
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t i = 0; i < n; ++i) {
            const uint32_t before = h->fl[i];
            const int32_t t0 = h->pt[i];
            double x0[3] = {h->x[3 * i], h->x[3 * i + 1], h->x[3 * i + 2]};
            const int32_t ec = htet[size_t(k) * n + i];
            step_particle(*h, cc, i, ec);
            if (!(before & FLAG_SETTLED) && (h->fl[i] & FLAG_SETTLED)) {
                // recompute the hit fraction and face of the settling walk
                const Tet &T = h->tet[ec];
                double vp[3];
                for (int c = 0; c < 3; ++c) {
                    const double a = (p.charge * T.E[c]) / p.mass;
                    const double half = (a * p.dt) / 2.0;
                    vp[c] = (T.E[0] == 0.0 && T.E[1] == 0.0 && T.E[2] == 0.0) ? hv[3 * (size_t(k) * n + i) + c]
                                                                              : (hv[3 * (size_t(k) * n + i) + c] + half) + half;
                }
                const double p1[3] = {x0[0] + vp[0] * p.dt, x0[1] + vp[1] * p.dt, x0[2] + vp[2] * p.dt};
                const Walk w = walk(*h, t0, x0, p1, p.max_crossings, true);
                land_step[i] = k;
                land_tet[i] = w.tet;
                land_face[i] = w.face;
                land_s[i] = w.s;
            }
        }
        h->step++;
    }
    if (h->freeze == 1) h->frozen = htet;
    // objective
    const double inv2 = 1.0 / (2.0 * sigma * sigma);
    double sum = 0.0;
    int64_t cnt = 0;
    std::vector<double> gr(3 * n, 0.0);
    for (int64_t i = 0; i < n; ++i)
        if (land_step[i] >= 0) {
            const double dx = h->x[3 * i] - target[0], dy = h->x[3 * i + 1] - target[1], dz = h->x[3 * i + 2] - target[2];
            const double g = std::exp(-(dx * dx + dy * dy + dz * dz) * inv2);
            sum += g;
            cnt++;
            gr[3 * i] = -2.0 * inv2 * g * dx;
            gr[3 * i + 1] = -2.0 * inv2 * g * dy;
            gr[3 * i + 2] = -2.0 * inv2 * g * dz;
        }
    if (J) *J = cnt ? sum / double(cnt) : 0.0;
    if (n_landed) *n_landed = cnt;
    if (!cnt) return SPG_OK;
    for (double &v : gr) v /= double(cnt);
    // particle adjoint
    std::vector<double> gE(3 * h->Nt, 0.0), ax(3 * n, 0.0), av(3 * n, 0.0);
    const double cq = p.charge / p.mass * p.dt;
    // gradient of the recovered field per tet: nodal E as the volume average of
    // the incident tets' E, interpolated linearly: G_t[d][c] = sum_i E_i[d] dlambda_i/dx_c
    std::vector<double> G;
    if (h->field_gradient) {
        std::vector<double> En(3 * h->Nn, 0.0), Wn(h->Nn, 0.0);
        for (int64_t t = 0; t < h->Nt; ++t)
            for (int k = 0; k < 4; ++k) {
                const int32_t nd = h->tn[4 * t + k];
                for (int c = 0; c < 3; ++c) En[3 * nd + c] += h->vol[t] * h->tet[t].E[c];
                Wn[nd] += h->vol[t];
            }
        for (int64_t nd = 0; nd < h->Nn; ++nd)
            for (int c = 0; c < 3; ++c) En[3 * nd + c] /= Wn[nd];
        G.assign(9 * h->Nt, 0.0);
        for (int64_t t = 0; t < h->Nt; ++t) {
            const Tet &T = h->tet[t];
            double gl[4][3];
            for (int c = 0; c < 3; ++c) {
                gl[1][c] = T.M[c];
                gl[2][c] = T.M[3 + c];
                gl[3][c] = T.M[6 + c];
                gl[0][c] = -(gl[1][c] + gl[2][c] + gl[3][c]);
            }
            for (int k = 0; k < 4; ++k) {
                const double *e = &En[3 * h->tn[4 * t + k]];
                for (int d = 0; d < 3; ++d)
                    for (int c = 0; c < 3; ++c) G[9 * t + 3 * d + c] += e[d] * gl[k][c];
            }
        }
    }
    for (int64_t i = 0; i < n; ++i) {
        const int N = land_step[i];
        if (N < 0) continue;
        double A[3] = {0, 0, 0}, V[3] = {0, 0, 0};
        for (int k = N; k >= 0; --k) {
            const size_t o = size_t(k) * n + i;
            const int t = htet[o];
            if (t < 0) continue;
            const double *v = &hv[3 * o];
            if (std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) < p.min_velocity) continue;
            const Tet &T = h->tet[t];
            double va[3];
            const bool ez = T.E[0] == 0.0 && T.E[1] == 0.0 && T.E[2] == 0.0;
            for (int c = 0; c < 3; ++c) {
                const double a = (p.charge * T.E[c]) / p.mass;
                const double half = (a * p.dt) / 2.0;
                va[c] = ez ? v[c] : (v[c] + half) + half;
            }
            double b[3];
            if (k == N) {
                const Tet &TL = h->tet[land_tet[i]];
                double nn[3];
                const int f = land_face[i];
                for (int c = 0; c < 3; ++c)
                    nn[c] = f == 0 ? -(TL.M[c] + TL.M[3 + c] + TL.M[6 + c]) : TL.M[3 * (f - 1) + c];
                const double nv = nn[0] * va[0] + nn[1] * va[1] + nn[2] * va[2];
                const double *g = &gr[3 * i];
                const double vg = (va[0] * g[0] + va[1] * g[1] + va[2] * g[2]) / nv;
                for (int c = 0; c < 3; ++c) {
                    A[c] = g[c] - nn[c] * vg;
                    b[c] = land_s[i] * p.dt * A[c];
                }
            } else {
                if (p.collision_model != SPG_COLL_NONE) {
                    if (collides(uint64_t(step0 + k), uint32_t(i), p.seed, probability(p, cc, va))) {
                        uint32_t r[4];
                        draws(uint64_t(step0 + k), 1u, uint32_t(i), p.seed, r);
                        const double u1 = u01(r[0], r[1]);
                        const double u2 = u01(r[2], r[3]);
                        const double xc = p.collision_model == SPG_COLL_HS ? -1.0 + 2.0 * u1 : u1;
                        const double xs = std::sqrt(1.0 - xc * xc), ph = (2.0 * PI) * u2;
                        const double nh[3] = {xs * std::cos(ph), xs * std::sin(ph), xc};
                        const double vm = std::sqrt(va[0] * va[0] + va[1] * va[1] + va[2] * va[2]);
                        const double na = (nh[0] * V[0] + nh[1] * V[1] + nh[2] * V[2]) * cc.mass_ct / vm;
                        for (int c = 0; c < 3; ++c) V[c] = cc.mass_cp * V[c] + na * va[c];
                    }
                }
                for (int c = 0; c < 3; ++c) b[c] = V[c] + p.dt * A[c];
            }
            for (int c = 0; c < 3; ++c) {
                gE[3 * t + c] += cq * b[c];
                V[c] = b[c];
            }
            if (!G.empty() && !ez) {
                // the pushed velocity depends on the position through the field
                const double *g = &G[9 * size_t(t)];
                for (int c = 0; c < 3; ++c) A[c] += cq * (g[c] * b[0] + g[3 + c] * b[1] + g[6 + c] * b[2]);
            }
        }
        for (int c = 0; c < 3; ++c) {
            ax[3 * i + c] = A[c];
            av[3 * i + c] = V[c];
        }
    }
    // dJ/dphi
    std::vector<double> lam(h->Nn, 0.0);
    for (int64_t t = 0; t < h->Nt; ++t) {
        const double *a = &gE[3 * t];
        const Tet &T = h->tet[t];
        const double m0 = T.M[0] * a[0] + T.M[1] * a[1] + T.M[2] * a[2];
        const double m1 = T.M[3] * a[0] + T.M[4] * a[1] + T.M[5] * a[2];
        const double m2 = T.M[6] * a[0] + T.M[7] * a[1] + T.M[8] * a[2];
        const int32_t *nd = &h->tn[4 * t];
        lam[nd[0]] += m0 + m1 + m2;
        lam[nd[1]] -= m0;
        lam[nd[2]] -= m1;
        lam[nd[3]] -= m2;
    }
    // adjoint CG: K mu = lam on free nodes (the Dirichlet rows are identity, rhs 0)
    std::vector<double> b(h->Nn), saved_phi = h->phi;
    for (int64_t i = 0; i < h->Nn; ++i) b[i] = h->isd[i] ? 0.0 : lam[i];
    std::fill(h->phi.begin(), h->phi.end(), 0.0);
    int32_t it = 0;
    double rr = 0.0;
    const int rc = pcg(*h, b, &it, &rr);
    std::vector<double> mu = h->phi;
    h->phi = saved_phi;
    if (rc) return fail(rc, "adjoint PCG did not converge");
    for (int64_t i = 0; i < h->Nn; ++i) dJ_dg[i] = h->isd[i] ? lam[i] : 0.0;
    for (int64_t f = 0; f < h->Nn; ++f)
        for (const auto &e : h->elim[f]) dJ_dg[e.first] -= e.second * mu[f];
    if (dJ_dx0) std::copy(ax.begin(), ax.end(), dJ_dx0);
    if (dJ_dv0) std::copy(av.begin(), av.end(), dJ_dv0);
    return SPG_OK;
}

int spo_grad_field_gradient(spo_handle *h, int on) {
    h->field_gradient = on != 0;
    return SPG_OK;
}

int spo_grad_freeze(spo_handle *h, int mode) {
    h->freeze = mode;
    if (mode == 0) h->frozen.clear();
    return SPG_OK;
}

void spo_update_position(double *x, const double *v, double dt) {
    // Particle::updatePosition: x = x + v dt
    const double nx = x[0] + v[0] * dt, ny = x[1] + v[1] * dt, nz = x[2] + v[2] * dt;
    x[0] = nx;
    x[1] = ny;
    x[2] = nz;
}

int spo_segment_triangle(const double *s0, const double *s1, const double *a, const double *b, const double *c,
                         double *pt) {
    auto sub = [](const double *u, const double *v, double *o) {
        o[0] = u[0] - v[0];
        o[1] = u[1] - v[1];
        o[2] = u[2] - v[2];
    };
    auto cross = [](const double *u, const double *v, double *o) {
        o[0] = u[1] * v[2] - u[2] * v[1];
        o[1] = u[2] * v[0] - u[0] * v[2];
        o[2] = u[0] * v[1] - u[1] * v[0];
    };
    auto dotp = [](const double *u, const double *v) { return u[0] * v[0] + u[1] * v[1] + u[2] * v[2]; };
    double e1[3], e2[3], n[3], d[3], w[3];
    sub(b, a, e1);
    sub(c, a, e2);
    cross(e1, e2, n);
    sub(s1, s0, d);
    sub(a, s0, w);
    const double den = dotp(n, d);
    const double num = dotp(n, w);
    // inside test of a point q in the triangle's plane (closed)
    auto inside = [&](const double *q) {
        const double *P[3] = {a, b, c};
        for (int k = 0; k < 3; ++k) {
            double ed[3], qp[3], cr[3];
            sub(P[(k + 1) % 3], P[k], ed);
            sub(q, P[k], qp);
            cross(ed, qp, cr);
            if (dotp(cr, n) < 0.0) return false;
        }
        return true;
    };
    if (den == 0.0) {
        if (num != 0.0) return 0;  // parallel, off-plane
        // coplanar: first point of the segment (from s0) inside the triangle
        const int N = 1 << 12;
        for (int k = 0; k <= N; ++k) {
            const double t = double(k) / N;
            const double q[3] = {s0[0] + t * d[0], s0[1] + t * d[1], s0[2] + t * d[2]};
            if (inside(q)) {
                pt[0] = q[0];
                pt[1] = q[1];
                pt[2] = q[2];
                return 1;
            }
        }
        return 0;
    }
    const double t = num / den;
    if (t < 0.0 || t > 1.0) return 0;
    const double q[3] = {s0[0] + t * d[0], s0[1] + t * d[1], s0[2] + t * d[2]};
    if (!inside(q)) return 0;
    pt[0] = q[0];
    pt[1] = q[1];
    pt[2] = q[2];
    return 1;
}

double spo_gas_concentration(double pressure, double temperature) {
    return (pressure / (8.314 * temperature)) * 6.02214076e23;
}

double spo_collision_probability(const spg_params *p, const double *v) {
    const CollConst c = coll_const(*p);
    return probability(*p, c, v);
}

int spo_collide_with(const spg_params *p, double *v, double u0, double u1, double u2) {
    const CollConst c = coll_const(*p);
    if (!(u0 < probability(*p, c, v))) return 0;
    scatter(*p, c, v, u1, u2);
    return 1;
}

double spo_tet_map(const double *x0, const double *x1, const double *x2, const double *x3, double *M9) {
    return tet_map(x0, x1, x2, x3, M9);
}

void spo_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) { philox(ctr, key, out); }

void spo_collides(const uint64_t *steps, const uint32_t *ids, int64_t n, uint64_t seed, double P, uint8_t *out) {
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n; ++k) out[k] = collides(steps[k], ids[k], seed, P) ? 1 : 0;
}

int spo_set_ref_compat(spo_handle *h, uint32_t flags, double cubature_w0) {
    if (!h) return fail(SPG_E_INVALID, "null handle");
    if (flags & ~uint32_t(SPO_COMPAT_ALL)) return fail(SPG_E_INVALID, "unknown compat flag");
    if (!(cubature_w0 > 0.0)) return fail(SPG_E_INVALID, "cubature_w0 must be > 0");
    h->compat = flags;
    h->cubature_w0 = cubature_w0;
    h->rho_map.assign(h->Nn, 0.0);
    h->rho_has.assign(h->Nn, 0);
    if (h->have_E) compute_E(*h);
    return SPG_OK;
}

}  // extern "C"
