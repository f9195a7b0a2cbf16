// Particle kernels of the FP64 form: fused push + move + gas collision +
// tet walk + surface settle, P1 deposit, per-tet E, point location, re-sort.
//
// Compiled with --fmad=false: every a*b+c stays a separate multiply and add,
// matching the CPU oracle (built with -ffp-contract=off) bit for bit on the
// collisionless path. Division and sqrt are IEEE (CUDA defaults for double).
//
// FP64 on GB300 issues at about 2 instructions per clock per SM (FP32: ~128),
// and double<->float conversions share that pipe. The step kernel therefore
// keeps FP64 semantics exactly while spending FP64 instructions only where the
// result is stored: push, move and the offset from the tet origin. Every
// yes/no decision of the reference algorithm (slow particle, inside the
// modelling box, degenerate segment, inside the tet, collision) is taken by an
// integer or FP32 screen with a proven error bound; when a screen cannot
// decide, the exact FP64 expression (the oracle's) decides. The state written
// is therefore identical to an all-FP64 evaluation.
#include <cmath>
#include <cstdio>

#include "philox.h"
#include "deposit.cuh"
#include "field.cuh"
#include "exact_div.h"
#include "screen.h"
#include "sort_block.cuh"
#include "spg_internal.h"

namespace spg {

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr unsigned kFull = 0xffffffffu;

enum WalkStatus { W_INSIDE = 0, W_SURFACE = 1, W_EXIT = 2, W_CAP = 3 };

struct TetGeo {
    double M[9];
    double x0[3];
};

__device__ __forceinline__ void load_geo(const TetRec *__restrict__ rec, int t, TetGeo &g) {
    const double2 *rp = reinterpret_cast<const double2 *>(rec + t);
    double2 a = __ldg(rp + 0), b = __ldg(rp + 1), c = __ldg(rp + 2), d = __ldg(rp + 3);
    double2 e = __ldg(rp + 4), f = __ldg(rp + 5);
    g.M[0] = a.x; g.M[1] = a.y; g.M[2] = b.x; g.M[3] = b.y; g.M[4] = c.x; g.M[5] = c.y;
    g.M[6] = d.x; g.M[7] = d.y; g.M[8] = e.x;
    g.x0[0] = e.y; g.x0[1] = f.x; g.x0[2] = f.y;
}

// Barycentric coordinates from the tet's record in memory (L1-resident
// during a walk), so a walk holds no FP64 map in registers; same values as
// the oracle's evaluation order.
__device__ __forceinline__ void bary_rec(const TetRec *__restrict__ r, double px, double py, double pz,
                                         double l[4]) {
    const double2 *rp = reinterpret_cast<const double2 *>(r);
    const double2 e = __ldg(rp + 4), f = __ldg(rp + 5);
    const double d0 = px - e.y, d1 = py - f.x, d2 = pz - f.y;
    const double2 a = __ldg(rp + 0), b = __ldg(rp + 1);
    l[1] = a.x * d0 + a.y * d1 + b.x * d2;
    const double2 c = __ldg(rp + 2), d = __ldg(rp + 3);
    l[2] = b.y * d0 + c.x * d1 + c.y * d2;
    l[3] = d.x * d0 + d.y * d1 + e.x * d2;
    l[0] = 1.0 - l[1] - l[2] - l[3];
}

__device__ __forceinline__ int comp(const int4 &v, int f) {
    return f == 0 ? v.x : (f == 1 ? v.y : (f == 2 ? v.z : v.w));
}

// ---------------------------------------------------------------- screens
// Order-preserving integer key of a double (see order_key_host).
__device__ __forceinline__ long long order_key(double x) {
    long long b = __double_as_longlong(x);
    if (b == (long long)0x8000000000000000ULL) b = 0;
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}

// IEEE equality of two finite doubles from their bit patterns.
__device__ __forceinline__ bool same_value(double a, double b) {
    const long long x = __double_as_longlong(a), y = __double_as_longlong(b);
    return x == y || ((x | y) << 1) == 0;
}

// Screened inside test from the tet's TetScreen record: true = lambda(p) >= 0
// in all four coordinates for certain; false = undecided (the caller
// evaluates the exact FP64 walk). No FP64 instruction runs: M is truncated to
// 20 mantissa bits (hi_float, once per tet on the host) and
// d = p - x0 is formed in FP32 from p and x0 truncated the same way (integer
// ops). With S_i = sum_j |M_ij d_j|, the truncation of M and the FP32
// products put lambda_i within 2.2e-6 S_i of its value for the exact d; the
// margin takes 4e-6 S_i + 1e-30 (for terms flushed to zero).
// |p - pf| < 2^-20 |p| <= 9.6e-7 |pf| (pf truncates toward zero) and the FP32
// difference rounds by at most 2^-24 |d_f|, so each d_k is within
// delta_k = 9.6e-7 (|pf_k| + |x0f_k|) + 6e-8 |d_fk| + 1e-30 of p_k - x0_k.
// That adds sum_k |M_ik| delta_k (times 1.01 for the truncation of M) to the
// margin of lambda_i; lambda_0 = 1 - sum gets the sum of the three margins
// plus 1e-6 for its own FP32 rounding.
__device__ __forceinline__ bool inside_sure_scr(const TetScreen *__restrict__ scr, double px, double py, double pz) {
    const float4 *sp = reinterpret_cast<const float4 *>(scr);
    const float4 q0 = __ldg(sp), q1 = __ldg(sp + 1), q2 = __ldg(sp + 2);
    const float M[9] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w, q2.x};
    const float X0[3] = {q2.y, q2.z, q2.w};
    const float pf[3] = {hi_float(px), hi_float(py), hi_float(pz)};
    float e[3], dl[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float x0 = X0[k];
        e[k] = pf[k] - x0;
        dl[k] = fmaf(9.6e-7f, fabsf(pf[k]) + fabsf(x0), fmaf(6e-8f, fabsf(e[k]), 1e-30f));
    }
    float l[3], b[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const float m0 = M[3 * r], m1 = M[3 * r + 1], m2 = M[3 * r + 2];
        l[r] = fmaf(m2, e[2], fmaf(m1, e[1], m0 * e[0]));
        const float s = fmaf(fabsf(m2), fabsf(e[2]), fmaf(fabsf(m1), fabsf(e[1]), fabsf(m0) * fabsf(e[0])));
        const float pd = fmaf(fabsf(m2), dl[2], fmaf(fabsf(m1), dl[1], fabsf(m0) * dl[0]));
        b[r] = fmaf(4e-6f, s, fmaf(1.01f, pd, 1e-30f));
    }
    const float l0 = 1.0f - l[0] - l[1] - l[2];
    const float b0 = b[0] + b[1] + b[2] + 1e-6f;
    return l[0] > b[0] && l[1] > b[1] && l[2] > b[2] && l0 > b0;
}

struct WalkOut {
    int tet, status, tri, crossings, face;
    double s;
};

// Straight walk of the segment p0 -> p1 starting in tet t (geometry g).
// In each tet: if p1 is inside (all lambda >= 0) stop. Otherwise leave through
// the face, other than the entry face, with lambda(p1) < 0 whose crossing
// parameter s = l0/(l0 - l1) along the segment is smallest (lowest local face
// index on ties). A face carrying a surface triangle stops the walk there
// (when stop_surface); a boundary face without one is an exit.
// FP64 is spent only where the decision needs it: in a tet entered by a
// crossing the FP32 inside screen usually decides; lambda(p0) and the
// divisions are formed only when two or more faces compete or s is returned
// (the same expressions as the full evaluation, so the same values).
__device__ __noinline__ WalkOut walk64(const MeshDev m, int t, double p0x, double p0y, double p0z, double p1x,
                                       double p1y, double p1z, int max_cross, bool stop_surface) {
    WalkOut o;
    o.crossings = 0;
    o.tri = -1;
    o.face = -1;
    o.s = 1.0;
    int enter = -1;
    for (;;) {
        if (enter >= 0 && inside_sure_scr(m.screen + t, p1x, p1y, p1z)) {
            o.tet = t;
            o.status = W_INSIDE;
            return o;
        }
        const TetRec *rt = m.rec + t;
        double l1[4];
        bary_rec(rt, p1x, p1y, p1z, l1);
        if (l1[0] >= 0.0 && l1[1] >= 0.0 && l1[2] >= 0.0 && l1[3] >= 0.0) {
            o.tet = t;
            o.status = W_INSIDE;
            return o;
        }
        int ncand = 0, best = -1;
#pragma unroll
        for (int f = 0; f < 4; ++f)
            if (f != enter && l1[f] < 0.0) {
                ++ncand;
                best = f;
            }
        if (ncand == 0) {
            o.tet = t;
            o.status = W_INSIDE;
            return o;
        }
        double l0[4];
        double sb = 0.0;
        bool have_s = false;
        if (ncand > 1) {
            bary_rec(rt, p0x, p0y, p0z, l0);
            best = -1;
#pragma unroll
            for (int f = 0; f < 4; ++f) {
                if (f == enter || !(l1[f] < 0.0)) continue;
                const double s = l0[f] / (l0[f] - l1[f]);
                if (best < 0 || s < sb) {
                    best = f;
                    sb = s;
                }
            }
            have_s = true;
        }
        const int tri = comp(__ldg(m.ftri + t), best);
        const int nb = comp(__ldg(m.nbr + t), best);
        const bool surface = stop_surface && tri >= 0;
        if ((surface || nb < 0) && !have_s) {
            bary_rec(rt, p0x, p0y, p0z, l0);
            sb = l0[best] / (l0[best] - l1[best]);
        }
        if (surface) {
            o.tet = t;
            o.status = W_SURFACE;
            o.tri = tri;
            o.face = best;
            o.s = sb;
            return o;
        }
        if (nb < 0) {
            o.tet = t;
            o.status = W_EXIT;
            o.s = sb;
            return o;
        }
        if (o.crossings == max_cross) {
            o.tet = t;
            o.status = W_CAP;
            return o;
        }
        o.crossings++;
        t = nb >> 2;
        enter = nb & 3;
    }
}

// Collision probability exactly as the reference evaluates it:
// HSModel.cpp:12-15, VHSModel.cpp:14-25 (and VSSModel.cpp, same formula).
__device__ __noinline__ double probability64(const StepConst c, double vx, double vy, double vz) {
    const double vmod = sqrt(vx * vx + vy * vy + vz * vz);
    double sigma;
    if (c.model == SPG_COLL_HS) {
        sigma = c.sigma_hs;
    } else {
        const double base = c.two_kT / ((c.mr * vmod) * vmod);
        const double d2 = c.vhs_c1 * pow(base, c.expo);
        sigma = kPi * d2;
    }
    return ((sigma * vmod) * c.gas_n) * c.dt;
}

// Post-collision velocity (HSModel.cpp:24-39, VHSModel.cpp:31-46,
// VSSModel.cpp:32-48): stationary target; v' = m_p/(m_p+m_t) v + |m_t/(m_p+m_t) v| n.
// The azimuth phi = 2 pi u2 enters as cospi(2 u2), sinpi(2 u2) (no argument
// reduction), and the VSS frame angles beta = acos(pz/|p|), gamma =
// atan2(py, px) as their cosines and sines formed algebraically: the same
// quantities, rounded differently, at a fraction of the FP64 instructions
// (collisional runs are compared with the reference statistically).
__device__ __noinline__ void scatter64(const StepConst c, double u1, double u2, double &vx, double &vy, double &vz) {
    double xi_cos;
    if (c.model == SPG_COLL_HS)
        xi_cos = -1.0 + 2.0 * u1;
    else if (c.model == SPG_COLL_VHS)
        xi_cos = u1;
    else
        xi_cos = 2.0 * pow(u1, c.inv_alpha) - 1.0;
    const double xi_sin = sqrt(1.0 - xi_cos * xi_cos);
    double sphi, cphi;
    sincospi(2.0 * u2, &sphi, &cphi);
    const double nx = xi_sin * cphi, ny = xi_sin * sphi, nz = xi_cos;
    const double cmx = vx * c.mass_cp, cmy = vy * c.mass_cp, cmz = vz * c.mass_cp;
    const double pvx = c.mass_ct * vx, pvy = c.mass_ct * vy, pvz = c.mass_ct * vz;
    const double mp = sqrt(pvx * pvx + pvy * pvy + pvz * pvz);
    double ex = nx * mp, ey = ny * mp, ez = nz * mp;
    if (c.model == SPG_COLL_VSS) {
        // GeometryVector::calcBetaGamma + rotation (GeometryVector.hpp:448-471, 66-90)
        const double cb = fmin(1.0, fmax(-1.0, pvz / mp)), sb = sqrt(1.0 - cb * cb);
        const double tx = cb * ex + sb * ez, tz = -sb * ex + cb * ez;
        ex = tx;
        ez = tz;
        const double rxy = sqrt(pvx * pvx + pvy * pvy);
        const double cg = rxy > 0.0 ? pvx / rxy : 1.0, sg = rxy > 0.0 ? pvy / rxy : 0.0;
        const double ux = cg * ex - sg * ey, uy = sg * ex + cg * ey;
        ex = ux;
        ey = uy;
    }
    vx = ex + cmx;
    vy = ey + cmy;
    vz = ez + cmz;
}

// Gas collision decision (the candidate-byte test of philox.h) and
// scattering, bit-exact with the FP64 test and decided mostly in FP32:
//  * a step that is no candidate (255 of 256) with v^2 at most c.v2_cand_f,
//    computed from the 20-bit components (below the true v^2), has P below
//    q: no collision, no FP64 instruction;
//  * otherwise P_f = kp (v^2)^pexp from the 20-bit components (relative
//    error below 2e-5) decides P against q outside the band q (1 -+ 1e-4),
//    a candidate's u_acc against 256 P outside 256 P_f (1 -+ 1e-4), and
//    u_f against (P - q) / (1 - q) outside a band of 3e-5 P_f + 2e-7;
//  * P is computed in FP64 only inside a band.
// The test where the common case cannot decide it: a candidate, or P that
// may exceed q (out of line, so the step loop carries none of it).
__device__ __noinline__ bool collision_test64(const StepConst c, uint32_t id, uint64_t step, uint32_t byte, float v2,
                                              double vx, double vy, double vz) {
    constexpr float qf = float(kCandQ);
    const float pf = c.kp_f * exp2f(c.pexp_f * log2f(v2));
    if (byte == 0u) {
        // a candidate: P > q collides; P <= q collides iff u_acc < 256 P
        if (pf > qf * (1.0f + 1e-4f)) return true;
        const Philox4 r = collision_draw(step, 3u, id, c.seed_lo, c.seed_hi);
        if (pf < qf * (1.0f - 1e-4f)) {
            const float ulo = float(r.v[0] >> 8) * 5.9604644775390625e-8f;  // 2^-24
            const float uhi = ulo + 5.9604644775390625e-8f;
            const float a = pf * 256.0f;
            if (uhi < a * (1.0f - 1e-4f)) return true;
            if (ulo > a * (1.0f + 1e-4f)) return false;
        }
        const double P = probability64(c, vx, vy, vz);
        return P > kCandQ || u01_from(r.v[0], r.v[1]) < P * 256.0;
    }
    if (pf < qf * (1.0f - 1e-4f)) return false;
    const Philox4 r = collision_draw(step, 4u, id, c.seed_lo, c.seed_hi);
    const float ulo = float(r.v[0] >> 8) * 5.9604644775390625e-8f;  // 2^-24
    const float uhi = ulo + 5.9604644775390625e-8f;
    const float tf = (pf - qf) / (1.0f - qf), band = 3e-5f * pf + 2e-7f;
    if (pf > qf * (1.0f + 1e-4f) && uhi < tf - band) return true;
    if (pf > qf * (1.0f + 1e-4f) && ulo > tf + band) return false;
    const double P = probability64(c, vx, vy, vz);
    return P > kCandQ && u01_from(r.v[0], r.v[1]) < (P - kCandQ) / (1.0 - kCandQ);
}

__device__ __forceinline__ bool collide(const StepConst &c, uint32_t id, double &vx, double &vy, double &vz) {
    const uint64_t step = uint64_t(c.step);
    const uint32_t byte = candidate_byte(candidate_block(step, id, c.seed_lo, c.seed_hi), step);
    const float fx = hi_float(vx), fy = hi_float(vy), fz = hi_float(vz);
    const float v2 = fmaf(fz, fz, fmaf(fy, fy, fx * fx));
    if (byte != 0u && v2 <= c.v2_cand_f) return false;
    if (!collision_test64(c, id, step, byte, v2, vx, vy, vz)) return false;
    const Philox4 r = collision_draw(step, 1u, id, c.seed_lo, c.seed_hi);
    scatter64(c, u01_from(r.v[0], r.v[1]), u01_from(r.v[2], r.v[3]), vx, vy, vz);
    return true;
}

__device__ __forceinline__ unsigned long long warp_sum(unsigned v) { return __reduce_add_sync(kFull, v); }

// Finite test from the exponent bits (no FP64 compare).
__device__ __forceinline__ bool finite_bits(double x) {
    return ((__double2hiint(x) >> 20) & 0x7ff) != 0x7ff;
}

// Append of this lane's item to the walk queue, called where the lane decides
// to queue: the lanes converged there share one atomic (their slots follow
// their lane order; the order of the queue does not matter).
__device__ __forceinline__ void queue_walk(WalkItem *__restrict__ q, unsigned int *__restrict__ qn, int64_t i,
                                           double x, double y, double z) {
    const unsigned act = __activemask();
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(act) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(qn, unsigned(__popc(act)));
    base = __shfl_sync(act, base, leader);
    WalkItem &w = q[base + __popc(act & ((1u << lane) - 1u))];
    w.i = int32_t(i);
    w.x0 = x;
    w.y0 = y;
    w.z0 = z;
}

// E per tet: E = -sum_i phi_i grad(lambda_i) = -sum_r (phi_{r+1} - phi_0) M_r
// (VolumetricMesh::computeElectricFields, VolumetricMesh.cpp:382-411, with the
// sign and scale of E = -grad(phi)), plus the push increment
// H = ((q E / m) dt) / 2, the operations of Particle::electroMagneticPush.
__device__ __forceinline__ void field_of_tet64(const FieldArgs &f, int64_t t) {
    const int4 tn = __ldg(f.tet_nodes + t);
    const double f0 = f.phi[tn.x], f1 = f.phi[tn.y], f2 = f.phi[tn.z], f3 = f.phi[tn.w];
    const double d1 = f1 - f0, d2 = f2 - f0, d3 = f3 - f0;
    TetRec &r = f.rec[t];
    double E[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) E[k] = -((d1 * r.M[k] + d2 * r.M[3 + k]) + d3 * r.M[6 + k]);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        f.efield[3 * t + k] = E[k];
        const double a = div_by_known(f.charge * E[k], f.mass, f.inv_mass);  // (q E) / m
        r.H[k] = (a * f.dt) / 2.0;
    }
    r.ezero = (((__double_as_longlong(E[0]) | __double_as_longlong(E[1]) | __double_as_longlong(E[2])) << 1) == 0)
                  ? 1u : 0u;  // all three +-0
}

// One particle step (ParticleDynamicsProcessor.cpp:161-200 order):
// settled? -> |v| < vmin? -> outside bbox? -> E push (Boris, B = 0) -> move ->
// gas collision -> surface crossing along the move segment.
// The new position is written for every moving particle. A particle whose
// end point is not certainly inside its tet is appended to the walk queue
// with its start point; k_walk_queue64 then walks it in full warps (FP64
// instructions issue per warp on GB300, so a walk taken by a few lanes of
// every warp would cost the whole warp its FP64 throughput).
__global__ void __launch_bounds__(256, 6) k_step64(DevParticles p, int64_t n, MeshDev m, StepConst c,
                                                WalkItem *__restrict__ wq, unsigned int *__restrict__ wq_n,
                                                DevCounters *ctr) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    unsigned processed = 0, coll = 0, lost = 0;
    if (i < n) {
        // all of the particle's words in one round trip (the flags gate their use)
        uint32_t idf = p.idf[i];
        const int t = p.tet[i];
        const double x = p.x[i], y = p.y[i], z = p.z[i];
        double vx = p.vx[i], vy = p.vy[i], vz = p.vz[i];
        if (!(idf & kDead)) {
            processed = 1;
            // |v| < vmin: certainly false when some |v_k| >= 2 vmin (bit compare of
            // non-negative doubles); otherwise the exact FP64 test.
            const long long ax = __double_as_longlong(vx) & 0x7fffffffffffffffLL;
            const long long ay = __double_as_longlong(vy) & 0x7fffffffffffffffLL;
            const long long az = __double_as_longlong(vz) & 0x7fffffffffffffffLL;
            bool slow = false;
            if (ax < c.two_vmin_bits && ay < c.two_vmin_bits && az < c.two_vmin_bits)
                slow = sqrt(vx * vx + vy * vy + vz * vz) < c.vmin;
            const long long kx = order_key(x), ky = order_key(y), kz = order_key(z);
            const bool inside_box = kx >= c.lo_key[0] && kx <= c.hi_key[0] && ky >= c.lo_key[1] &&
                                    ky <= c.hi_key[1] && kz >= c.lo_key[2] && kz <= c.hi_key[2];
            if (!slow && inside_box) {
                const TetRec *rp = m.rec + t;
                if (!__ldg(&rp->ezero)) {
                    // Particle::electroMagneticPush (Particle.cpp:196-234) with B = 0:
                    // v- = v + a dt/2, the rotation is the identity, v = v- + a dt/2.
                    const double hx = __ldg(&rp->H[0]), hy = __ldg(&rp->H[1]), hz = __ldg(&rp->H[2]);
                    vx = (vx + hx) + hx;
                    vy = (vy + hy) + hy;
                    vz = (vz + hz) + hz;
                }
                // Particle::updatePosition (Particle.cpp:157-165)
                const double nx = x + vx * c.dt, ny = y + vy * c.dt, nz = z + vz * c.dt;
                if (!(same_value(nx, x) && same_value(ny, y) && same_value(nz, z))) {
                    const uint32_t id = idf & kIdMask;
                    if (c.model != SPG_COLL_NONE) coll = collide(c, id, vx, vy, vz) ? 1u : 0u;
                    if (!(finite_bits(nx) && finite_bits(ny) && finite_bits(nz))) {
                        idf |= kLost;
                        lost = 1;
                        p.idf[i] = idf;
                    } else {
                        if (!inside_sure_scr(m.screen + t, nx, ny, nz)) queue_walk(wq, wq_n, i, x, y, z);
                        p.x[i] = nx;
                        p.y[i] = ny;
                        p.z[i] = nz;
                    }
                }
                p.vx[i] = vx;
                p.vy[i] = vy;
                p.vz[i] = vz;
            }
        }
    }
    // Block-level counter reduction, one atomic per counter per block (the
    // walk kernel counts crossings, settled and capped particles).
    __shared__ unsigned long long sh[8][3];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const unsigned long long a0 = warp_sum(processed), a1 = warp_sum(coll), a2 = warp_sum(lost);
    if (lane == 0) {
        sh[wid][0] = a0;
        sh[wid][1] = a1;
        sh[wid][2] = a2;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        unsigned long long s = 0;
        const int nw = blockDim.x >> 5;
        for (int w = 0; w < nw; ++w) s += sh[w][threadIdx.x];
        if (s) {
            unsigned long long *dst = threadIdx.x == 0   ? &ctr->processed
                                      : threadIdx.x == 1 ? &ctr->collisions
                                                         : &ctr->lost;
            atomicAdd(dst, s);
        }
    }
}

// Exact FP64 walk of the queued particles (start point from the queue, end
// point already in the position arrays), one particle per lane.
// With land != nullptr, a particle that settles also records the step, the
// exit face of its final tet and the hit fraction of the segment (adjoint).
__global__ void __launch_bounds__(128) k_walk_queue64(DevParticles p, MeshDev m, int max_cross,
                                                      const WalkItem *__restrict__ wq,
                                                      const unsigned int *__restrict__ wq_n,
                                                      unsigned int *__restrict__ tri_count, DevCounters *ctr,
                                                      LandRec *__restrict__ land, int64_t step, const __grid_constant__ FieldArgs f) {
    const unsigned nq = *wq_n;
    unsigned cross = 0, settled = 0, lost = 0, capped = 0;
    for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x) {
        const WalkItem it = wq[q];
        const int64_t i = it.i;
        const int t = p.tet[i];
        const double nx = p.x[i], ny = p.y[i], nz = p.z[i];
        const WalkOut w = walk64(m, t, it.x0, it.y0, it.z0, nx, ny, nz, max_cross, true);
        cross += unsigned(w.crossings);
        uint32_t idf = p.idf[i];
        if (w.status == W_SURFACE) {
            p.x[i] = it.x0 + w.s * (nx - it.x0);
            p.y[i] = it.y0 + w.s * (ny - it.y0);
            p.z[i] = it.z0 + w.s * (nz - it.z0);
            atomicAdd(tri_count + w.tri, 1u);
            p.idf[i] = idf | kSettled;
            settled++;
            if (land) {
                land[i].step = int32_t(step);
                land[i].face = w.face;
                land[i].tet = w.tet;
                land[i].s = w.s;
            }
        } else if (w.status != W_INSIDE) {
            p.idf[i] = idf | kLost;
            lost++;
            if (w.status == W_CAP) capped++;
        }
        if (w.tet != t) {
            p.tet[i] = w.tet;
            if (w.status == W_INSIDE) refresh_tet(f.stamp, f.epoch, w.tet, [&f](int tt) { field_of_tet64(f, tt); });
        }
    }
    const unsigned long long a0 = __reduce_add_sync(kFull, cross), a1 = __reduce_add_sync(kFull, settled);
    const unsigned long long a2 = __reduce_add_sync(kFull, lost), a3 = __reduce_add_sync(kFull, capped);
    if ((threadIdx.x & 31) == 0) {
        if (a0) atomicAdd(&ctr->crossings, a0);
        if (a1) atomicAdd(&ctr->settled, a1);
        if (a2) atomicAdd(&ctr->lost, a2);
        if (a3) atomicAdd(&ctr->capped, a3);
    }
}

// round(x * 2^k) for |x| < 2 and k <= 52 with integer ops only (round half
// away from zero on the magnitude).
__device__ __forceinline__ long long fix_round(double x, int k) {
    const long long b = __double_as_longlong(x);
    const int e = int((b >> 52) & 0x7ff);
    if (e == 0) return 0;
    const long long mant = (b & 0xFFFFFFFFFFFFFLL) | (1LL << 52);
    const int sh = 1075 - e - k;
    long long r;
    if (sh <= 0)
        r = mant << (-sh);
    else if (sh > 62)
        r = 0;
    else
        r = (mant + (1LL << (sh - 1))) >> sh;
    return b < 0 ? -r : r;
}

// P1 deposit in fixed point: each alive particle adds round(lambda_i 2^k) for
// i = 1..3 and 2^k minus their sum for lambda_0, so its four node shares are
// exactly 2^k and charge is conserved exactly. Integer sums do not depend on
// summation order, so the result is the same for any particle order, grid
// or atomic interleaving. Lanes of a warp hold consecutive (tet-sorted)
// particles; runs of equal tet are summed per warp and merged in the
// block's node table over its range of tiles (deposit.cuh).
struct DepSrc64 {
    struct Raw {
        uint32_t idf;
        int32_t tet;
        double x, y, z;
    };
    DevParticles p;
    const TetRec *rec;
    int k;
    long long one;
    __device__ __forceinline__ Raw load(int64_t i, int64_t n) const {
        Raw r{kDead, -1, 0.0, 0.0, 0.0};
        if (i < n) {
            r.idf = __ldg(p.idf + i);
            r.tet = __ldg(p.tet + i);
            r.x = __ldg(p.x + i);
            r.y = __ldg(p.y + i);
            r.z = __ldg(p.z + i);
        }
        return r;
    }
    __device__ __forceinline__ int weights(const Raw &r, long long v[4]) const {
        v[0] = v[1] = v[2] = v[3] = 0;
        if (r.idf & kDead) return -1;
        TetGeo g;
        load_geo(rec, r.tet, g);
        const double d0 = r.x - g.x0[0], d1 = r.y - g.x0[1], d2 = r.z - g.x0[2];
        const double l1 = g.M[0] * d0 + g.M[1] * d1 + g.M[2] * d2;
        const double l2 = g.M[3] * d0 + g.M[4] * d1 + g.M[5] * d2;
        const double l3 = g.M[6] * d0 + g.M[7] * d1 + g.M[8] * d2;
        v[1] = fix_round(l1, k);
        v[2] = fix_round(l2, k);
        v[3] = fix_round(l3, k);
        v[0] = one - v[1] - v[2] - v[3];
        return r.tet;
    }
};

__global__ void __launch_bounds__(kDepThreads)
    k_deposit64(const DepSrc64 src, int64_t n, const int4 *__restrict__ tet_nodes,
                unsigned long long *__restrict__ node_fix, const OccList occ) {
    deposit_tiles(src, n, tet_nodes, node_fix, occ);
}

__global__ void k_fix_to_charge(const unsigned long long *__restrict__ node_fix, double scale,
                                double *__restrict__ node_q, int64_t n) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    node_q[i] = double((long long)node_fix[i]) * scale;
}

// The field of the tets listed by the deposit (each once).
__global__ void k_field64_list(const __grid_constant__ FieldArgs f, const int32_t *__restrict__ list,
                               const unsigned int *__restrict__ list_n) {
    const unsigned nl = *list_n;
    for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < nl; j += gridDim.x * blockDim.x) {
        const int t = list[j];
        field_of_tet64(f, t);
        f.stamp[t] = f.epoch;
    }
}

__global__ void k_field64_full(const __grid_constant__ FieldArgs f, int64_t n) {
    const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= n) return;
    field_of_tet64(f, t);
    f.stamp[t] = f.epoch;
}

// The field of every tet holding an alive particle. Particles are tet-sorted
// (up to the drift since the last re-sort), so only the first lane of each
// run of equal tets in a warp checks the stamp.
__global__ void k_refresh64(DevParticles p, int64_t n, const __grid_constant__ FieldArgs f) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int key = (i < n && !(p.idf[i] & kDead)) ? p.tet[i] : -1;
    const int prev = __shfl_up_sync(kFull, key, 1);
    if (key >= 0 && ((threadIdx.x & 31) == 0 || prev != key))
        refresh_tet(f.stamp, f.epoch, key, [&f](int t) { field_of_tet64(f, t); });
}

// E = 0 and H = 0 everywhere (before the first solve), stamped.
__global__ void k_zero_field(const __grid_constant__ FieldArgs f, int64_t n) {
    const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= n) return;
    f.rec[t].H[0] = 0.0;
    f.rec[t].H[1] = 0.0;
    f.rec[t].H[2] = 0.0;
    f.rec[t].ezero = 1u;
    if (f.rec32) {
        f.rec32[t].H[0] = 0.0f;
        f.rec32[t].H[1] = 0.0f;
        f.rec32[t].H[2] = 0.0f;
        f.rec32[t].ezero = (f.rec32[t].ezero & kRecInterior) | kRecEzero;
    }
    f.efield[3 * t] = 0.0;
    f.efield[3 * t + 1] = 0.0;
    f.efield[3 * t + 2] = 0.0;
    f.stamp[t] = f.epoch;
}

__global__ void k_count_lost(const int32_t *__restrict__ tet, int64_t n, unsigned long long *out) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const unsigned v = (i < n && tet[i] < 0) ? 1u : 0u;
    const unsigned s = __reduce_add_sync(kFull, v);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(out, (unsigned long long)s);
}

// Point location: walk from the centroid of the voxel's seed tet to p.
__global__ void k_locate(const double *__restrict__ pos, int64_t n, MeshDev m, const int32_t *__restrict__ vox_seed,
                         double ox, double oy, double oz, double ix, double iy, double iz, int dx, int dy, int dz,
                         int max_cross, int32_t *__restrict__ tet_out) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double px = pos[3 * i], py = pos[3 * i + 1], pz = pos[3 * i + 2];
    if (!(finite_bits(px) && finite_bits(py) && finite_bits(pz))) {
        tet_out[i] = -1;
        return;
    }
    const int vx = min(dx - 1, max(0, int(floor((px - ox) * ix))));
    const int vy = min(dy - 1, max(0, int(floor((py - oy) * iy))));
    const int vz = min(dz - 1, max(0, int(floor((pz - oz) * iz))));
    const int seed = vox_seed[vx + int64_t(dx) * (vy + int64_t(dy) * vz)];
    const int4 tn = __ldg(m.tet_nodes + seed);
    double c[3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
        c[k] = 0.25 * (((m.node_xyz[3 * tn.x + k] + m.node_xyz[3 * tn.y + k]) + m.node_xyz[3 * tn.z + k]) +
                       m.node_xyz[3 * tn.w + k]);
    const WalkOut w = walk64(m, seed, c[0], c[1], c[2], px, py, pz, max_cross, false);
    tet_out[i] = w.status == W_INSIDE ? w.tet : -1;
}

// Upload and location in one pass, reading the caller's position and
// velocity arrays where they lie (host memory the GPU reaches over the C2C
// link), so the copy overlaps the location walks: the same tet and state as
// k_locate followed by k_init_particles (FP64 form) or k_to_local (mixed form,
// cen != nullptr: FP32 position about the tet's centroid, FP32 velocity).
__global__ void __launch_bounds__(128) k_upload(const double *__restrict__ pos, const double *__restrict__ vel, int64_t n, MeshDev m,
                         const int32_t *__restrict__ vox_seed, double ox, double oy, double oz, double ix, double iy,
                         double iz, int dx, int dy, int dz, int max_cross, DevParticles p, DevParticles32 q,
                         const double *__restrict__ cen, unsigned long long *lost) {
    // the block's xyz triples come in as one contiguous run per array (whole
    // lines per warp load), then each thread takes its particle's
    __shared__ double sp[3 * 128], sv[3 * 128];
    const int64_t i0 = int64_t(blockIdx.x) * 128;
    const int64_t i = i0 + threadIdx.x;
    const int cnt = n - i0 < 128 ? int(n - i0) : 128;
    for (int k = threadIdx.x; k < 3 * cnt; k += 128) {
        sp[k] = pos[3 * i0 + k];
        sv[k] = vel[3 * i0 + k];
    }
    __syncthreads();
    unsigned is_lost = 0;
    if (i < n) {
        const double px = sp[3 * threadIdx.x], py = sp[3 * threadIdx.x + 1], pz = sp[3 * threadIdx.x + 2];
        const double vx = sv[3 * threadIdx.x], vy = sv[3 * threadIdx.x + 1], vz = sv[3 * threadIdx.x + 2];
        int32_t t = -1;
        if (finite_bits(px) && finite_bits(py) && finite_bits(pz)) {
            const int cx = min(dx - 1, max(0, int(floor((px - ox) * ix))));
            const int cy = min(dy - 1, max(0, int(floor((py - oy) * iy))));
            const int cz = min(dz - 1, max(0, int(floor((pz - oz) * iz))));
            const int seed = vox_seed[cx + int64_t(dx) * (cy + int64_t(dy) * cz)];
            const int4 tn = __ldg(m.tet_nodes + seed);
            double c[3];
#pragma unroll
            for (int k = 0; k < 3; ++k)
                c[k] = 0.25 * (((m.node_xyz[3 * tn.x + k] + m.node_xyz[3 * tn.y + k]) + m.node_xyz[3 * tn.z + k]) +
                               m.node_xyz[3 * tn.w + k]);
            const WalkOut w = walk64(m, seed, c[0], c[1], c[2], px, py, pz, max_cross, false);
            t = w.status == W_INSIDE ? w.tet : -1;
        }
        is_lost = t < 0 ? 1u : 0u;
        const uint32_t idf = uint32_t(i) | (t < 0 ? kLost : 0u);
        if (cen) {
            const int64_t tc = t < 0 ? 0 : t;
            q.x[i] = float(px - (t < 0 ? 0.0 : cen[3 * tc]));
            q.y[i] = float(py - (t < 0 ? 0.0 : cen[3 * tc + 1]));
            q.z[i] = float(pz - (t < 0 ? 0.0 : cen[3 * tc + 2]));
            q.vx[i] = float(vx);
            q.vy[i] = float(vy);
            q.vz[i] = float(vz);
            q.tet[i] = t;
            q.idf[i] = idf;
        } else {
            p.x[i] = px;
            p.y[i] = py;
            p.z[i] = pz;
            p.vx[i] = vx;
            p.vy[i] = vy;
            p.vz[i] = vz;
            p.tet[i] = t;
            p.idf[i] = idf;
        }
    }
    const unsigned s = __reduce_add_sync(kFull, is_lost);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(lost, (unsigned long long)s);
}

__global__ void k_init_particles(const double *__restrict__ pos, const double *__restrict__ vel,
                                 const int32_t *__restrict__ tet, int64_t n, DevParticles p, int64_t id_base) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t j = id_base + i;
    p.x[j] = pos[3 * i];
    p.y[j] = pos[3 * i + 1];
    p.z[j] = pos[3 * i + 2];
    p.vx[j] = vel[3 * i];
    p.vy[j] = vel[3 * i + 1];
    p.vz[j] = vel[3 * i + 2];
    const int32_t t = tet[i];
    p.tet[j] = t;
    p.idf[j] = uint32_t(j) | (t < 0 ? kLost : 0u);
}

// Slot of each particle id. The ids are a permutation of 0..n-1 (set, inject
// and restore keep it so); an id out of range is not written.
__global__ void k_slot_of_id(const uint32_t *__restrict__ idf, int64_t n, int32_t *__restrict__ slot) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t id = idf[i] & kIdMask;
    if (int64_t(id) < n) slot[id] = int32_t(i);
}

// One thread per id: scattered reads of its slot, writes in id order. The
// block's xyz triples go through shared memory and out as one contiguous run
// per array, so each warp store covers whole lines (the arrays may be the
// caller's pinned host memory, written over the C2C link).
__global__ void __launch_bounds__(256) k_gather_by_id(DevParticles p, int64_t n, const int32_t *__restrict__ slot,
                                                      double *pos, double *vel, int32_t *tet, uint32_t *flags) {
    __shared__ double sp[3 * 256], sv[3 * 256];
    const int64_t id0 = int64_t(blockIdx.x) * 256;
    const int64_t id = id0 + threadIdx.x;
    const int m = n - id0 < 256 ? int(n - id0) : 256;
    if (id < n) {
        const int64_t i = slot[id];
        const uint32_t idf = p.idf[i];
        if (pos) {
            sp[3 * threadIdx.x] = p.x[i];
            sp[3 * threadIdx.x + 1] = p.y[i];
            sp[3 * threadIdx.x + 2] = p.z[i];
        }
        if (vel) {
            sv[3 * threadIdx.x] = p.vx[i];
            sv[3 * threadIdx.x + 1] = p.vy[i];
            sv[3 * threadIdx.x + 2] = p.vz[i];
        }
        if (tet) tet[id] = p.tet[i];
        if (flags) flags[id] = ((idf & kSettled) ? SPG_FLAG_SETTLED : 0u) | ((idf & kLost) ? SPG_FLAG_LOST : 0u);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 3 * m; k += 256) {
        if (pos) pos[3 * id0 + k] = sp[k];
        if (vel) vel[3 * id0 + k] = sv[k];
    }
}

// ------------------------------------------------------------------ re-sort
// Counting sort by tet (dead particles get key n_tets and go last).

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void __launch_bounds__(kSortBlock) k_sort_hist(const int32_t *__restrict__ tet,
                                                          const uint32_t *__restrict__ idf, int64_t n, int n_tets,
                                                          int32_t *__restrict__ cnt) {
    __shared__ SortTable t;
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int key = i < n ? ((idf[i] & kDead) ? n_tets : tet[i]) : -1;
    sort_hist_block(t, key, cnt);
}

// Block-local exclusive scan of one tile; tile total to sums[blockIdx.x].
// Also counts non-empty tet bins (occupied tets).
__global__ void __launch_bounds__(kScanThreads) k_scan_tile(int32_t *__restrict__ a, int64_t len, int n_tets,
                                                            int32_t *__restrict__ sums,
                                                            unsigned long long *__restrict__ occupied) {
    __shared__ int32_t ws[kScanThreads / 32];
    const int64_t base = int64_t(blockIdx.x) * kScanTile + int64_t(threadIdx.x) * kScanItems;
    int32_t v[kScanItems];
    int32_t run = 0;
    unsigned occ = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t j = base + k;
        const int32_t x = j < len ? a[j] : 0;
        if (j < n_tets && x > 0) occ++;
        v[k] = run;
        run += x;
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int32_t incl = run;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int32_t up = __shfl_up_sync(kFull, incl, off);
        if (lane >= off) incl += up;
    }
    if (lane == 31) ws[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        int32_t w = lane < kScanThreads / 32 ? ws[lane] : 0;
        int32_t wi = w;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int32_t up = __shfl_up_sync(kFull, wi, off);
            if (lane >= off) wi += up;
        }
        if (lane < kScanThreads / 32) ws[lane] = wi - w;
    }
    __syncthreads();
    const int32_t offset = ws[wid] + (incl - run);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t j = base + k;
        if (j < len) a[j] = v[k] + offset;
    }
    if (threadIdx.x == kScanThreads - 1) sums[blockIdx.x] = offset + run;
    const unsigned long long occw = __reduce_add_sync(kFull, occ);
    if (lane == 0 && occw) atomicAdd(occupied, occw);
}

// Exclusive scan of the tile sums by one block, carrying across chunks.
__global__ void __launch_bounds__(1024) k_scan_sums(int32_t *__restrict__ sums, int64_t nb) {
    __shared__ int32_t ws[32];
    __shared__ int32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int64_t c0 = 0; c0 < nb; c0 += 1024) {
        const int64_t j = c0 + threadIdx.x;
        const int32_t x = j < nb ? sums[j] : 0;
        int32_t incl = x;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int32_t up = __shfl_up_sync(kFull, incl, off);
            if (lane >= off) incl += up;
        }
        if (lane == 31) ws[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            int32_t w = ws[lane];
            int32_t wi = w;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const int32_t up = __shfl_up_sync(kFull, wi, off);
                if (lane >= off) wi += up;
            }
            ws[lane] = wi - w;
        }
        __syncthreads();
        const int32_t excl = carry + ws[wid] + incl - x;
        if (j < nb) sums[j] = excl;
        __syncthreads();
        if (threadIdx.x == 1023) carry = excl + x;
        __syncthreads();
    }
}

__global__ void k_scan_add(int32_t *__restrict__ a, int64_t len, const int32_t *__restrict__ sums, int n_tets,
                           int64_t *__restrict__ n_alive) {
    const int64_t j = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= len) return;
    const int32_t v = a[j] + sums[j / kScanTile];
    a[j] = v;
    if (j == n_tets) *n_alive = v;
}

__global__ void __launch_bounds__(kSortBlock) k_sort_scatter(DevParticles src, DevParticles dst, int64_t n, int n_tets,
                                                             int32_t *__restrict__ offs) {
    __shared__ SortTable t;
    sort_scatter_block(t, src, dst, n, n_tets, kDead, offs);
}

inline unsigned grid_for(int64_t n, int block) { return unsigned((n + block - 1) / block); }

}  // namespace

void launch_step64(const DevParticles &p, int64_t n, const MeshDev &m, const StepConst &c, unsigned int *tri_count,
                   WalkItem *wq, unsigned int *wq_n, DevCounters *ctr, const FieldArgs &f, cudaStream_t s,
                   LandRec *land) {
    if (n <= 0) return;
    cudaMemsetAsync(wq_n, 0, sizeof(unsigned int), s);
    k_step64<<<grid_for(n, 256), 256, 0, s>>>(p, n, m, c, wq, wq_n, ctr);
    k_walk_queue64<<<152 * 8, 128, 0, s>>>(p, m, c.max_cross, wq, wq_n, tri_count, ctr, land, c.step, f);
}

void launch_deposit64(const DevParticles &p, int64_t n, const MeshDev &m, int k, unsigned long long *node_fix,
                      const OccList &occ, cudaStream_t s) {
    if (n <= 0) return;
    static int blocks = 0;  // one wave
    if (blocks == 0) blocks = resident_blocks(k_deposit64, kDepThreads);
    const DepSrc64 src{p, m.rec, k, 1LL << k};
    const unsigned grid = unsigned(std::min<int64_t>(grid_for(n, kDepThreads), blocks));
    k_deposit64<<<grid, kDepThreads, 0, s>>>(src, n, m.tet_nodes, node_fix, occ);
}

void launch_fix_to_charge(const unsigned long long *node_fix, double scale, double *node_q, int64_t n,
                          cudaStream_t s) {
    k_fix_to_charge<<<grid_for(n, 256), 256, 0, s>>>(node_fix, scale, node_q, n);
}

void launch_field64_full(const FieldArgs &f, int64_t n_tets, cudaStream_t s) {
    if (n_tets > 0) k_field64_full<<<grid_for(n_tets, 256), 256, 0, s>>>(f, n_tets);
}

void launch_field64_list(const FieldArgs &f, const int32_t *list, const unsigned int *list_n, cudaStream_t s) {
    k_field64_list<<<152 * 4, 256, 0, s>>>(f, list, list_n);
}

void launch_refresh64(const DevParticles &p, int64_t n, const FieldArgs &f, cudaStream_t s) {
    if (n > 0) k_refresh64<<<grid_for(n, 256), 256, 0, s>>>(p, n, f);
}

void launch_zero_field(const FieldArgs &f, int64_t n_tets, cudaStream_t s) {
    if (n_tets > 0) k_zero_field<<<grid_for(n_tets, 256), 256, 0, s>>>(f, n_tets);
}

void launch_count_lost(const int32_t *tet, int64_t n, unsigned long long *out, cudaStream_t s) {
    if (n <= 0) return;
    k_count_lost<<<grid_for(n, 256), 256, 0, s>>>(tet, n, out);
}

void launch_locate(const double *pos, int64_t n, const MeshDev &m, const int32_t *vox_seed,
                   const double *oi, const int32_t *dims, int max_cross, int32_t *tet_out, cudaStream_t s) {
    if (n <= 0) return;
    k_locate<<<grid_for(n, 128), 128, 0, s>>>(pos, n, m, vox_seed, oi[0], oi[1], oi[2], oi[3], oi[4], oi[5],
                                               dims[0], dims[1], dims[2], max_cross, tet_out);
}

void launch_init_particles(const double *pos, const double *vel, const int32_t *tet, int64_t n, DevParticles p,
                           cudaStream_t s, int64_t id_base) {
    if (n <= 0) return;
    k_init_particles<<<grid_for(n, 256), 256, 0, s>>>(pos, vel, tet, n, p, id_base);
}

void launch_upload(const double *pos, const double *vel, int64_t n, const MeshDev &m, const int32_t *vox_seed,
                   const double *oi, const int32_t *dims, int max_cross, const DevParticles &p,
                   const DevParticles32 &q, const double *cen, unsigned long long *lost, cudaStream_t s) {
    if (n <= 0) return;
    k_upload<<<grid_for(n, 128), 128, 0, s>>>(pos, vel, n, m, vox_seed, oi[0], oi[1], oi[2], oi[3], oi[4], oi[5],  // 128: staging
                                               dims[0], dims[1], dims[2], max_cross, p, q, cen, lost);
}

void launch_slot_of_id(const uint32_t *idf, int64_t n, int32_t *slot, cudaStream_t s) {
    if (n > 0) k_slot_of_id<<<grid_for(n, 256), 256, 0, s>>>(idf, n, slot);
}

void launch_gather_by_id(const DevParticles &p, int64_t n, int32_t *slot, double *pos, double *vel,
                         int32_t *tet, uint32_t *flags, cudaStream_t s) {
    if (n <= 0) return;
    launch_slot_of_id(p.idf, n, slot, s);
    k_gather_by_id<<<grid_for(n, 256), 256, 0, s>>>(p, n, slot, pos, vel, tet, flags);  // 256: the staging size
}

int64_t sort_scratch_words(int64_t n_tets) {
    const int64_t len = n_tets + 1;
    const int64_t nb = (len + kScanTile - 1) / kScanTile;
    // 64-bit occupied-tet counter (2 words), counts/offsets, tile sums
    return 2 + len + nb;
}

unsigned long long *sort_occupied_counter(int32_t *scratch) {
    return reinterpret_cast<unsigned long long *>(scratch);
}

int32_t *sort_offsets(int32_t *scratch) { return scratch + 2; }

void launch_sort_prepare(const int32_t *tet, const uint32_t *idf, int64_t n, int64_t n_tets, int32_t *scratch,
                         int64_t *n_alive_dev, cudaStream_t s) {
    const int64_t len = n_tets + 1;
    const int64_t nb = (len + kScanTile - 1) / kScanTile;
    unsigned long long *occupied = sort_occupied_counter(scratch);
    int32_t *cnt = sort_offsets(scratch);
    int32_t *sums = cnt + len;
    cudaMemsetAsync(cnt, 0, sizeof(int32_t) * len, s);
    cudaMemsetAsync(occupied, 0, sizeof(unsigned long long), s);
    if (n > 0) k_sort_hist<<<grid_for(n, kSortBlock), kSortBlock, 0, s>>>(tet, idf, n, int(n_tets), cnt);
    k_scan_tile<<<unsigned(nb), kScanThreads, 0, s>>>(cnt, len, int(n_tets), sums, occupied);
    k_scan_sums<<<1, 1024, 0, s>>>(sums, nb);
    k_scan_add<<<grid_for(len, 256), 256, 0, s>>>(cnt, len, sums, int(n_tets), n_alive_dev);
}

void launch_resort(const DevParticles &src, DevParticles dst, int64_t n, int64_t n_tets, int32_t *scratch,
                   int64_t *n_alive_dev, cudaStream_t s) {
    launch_sort_prepare(src.tet, src.idf, n, n_tets, scratch, n_alive_dev, s);
    if (n > 0)
        k_sort_scatter<<<grid_for(n, kSortBlock), kSortBlock, 0, s>>>(src, dst, n, int(n_tets), sort_offsets(scratch));
}

}  // namespace spg
