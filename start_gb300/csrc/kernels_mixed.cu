// Mixed-precision form of the particle step (SPG_MIXED).
//
// Particle state is 32 B: position in FP32 relative to the owning tet's
// centroid, velocity in FP32, tet and id/flags. Per tet a 64-B record holds
// the FP32 barycentric map about the centroid (lambda_{1..3} = 1/4 + M x),
// the FP32 push increment and the centroid in FP32 (for the modelling-box
// test). FP64 is kept where the result depends on a sign near zero or on
// cancellation:
//   * a barycentric coordinate within 1e-5 of zero is recomputed in FP64
//     (the FP64 map of the plain form, x promoted to FP64);
//   * a face crossing re-bases the position into the neighbour's frame,
//     x' = x + (c_old - c_new), with the centroids as FP32 pairs and
//     error-free sums: the FP32 rounding of the exact sum, as an FP64 sum
//     would give it, without the FP64 pipe;
//   * the deposit accumulates in 64-bit fixed point (exact).
// Every other operation (push, move, collision, exit parameter) is FP32,
// which on GB300 issues ~60x faster than FP64.
#include <algorithm>
#include <cmath>

#include "pdl.cuh"
#include "philox.h"
#include "deposit.cuh"
#include "field.cuh"
#include "sort_block.cuh"
#include "spg_internal.h"

namespace spg {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr float kPiF = 3.14159265358979323846f;
constexpr float kNearZero = 1e-5f;

enum { W_INSIDE = 0, W_SURFACE = 1, W_EXIT = 2, W_CAP = 3 };

struct Geo32 {
    float M[9];
};

__device__ __forceinline__ void load_geo32(const TetRec32 *__restrict__ rec, int t, Geo32 &g) {
    const float4 *rp = reinterpret_cast<const float4 *>(rec + t);
    const float4 a = __ldg(rp), b = __ldg(rp + 1);
    const float c = __ldg(&rec[t].M[8]);
    g.M[0] = a.x; g.M[1] = a.y; g.M[2] = a.z; g.M[3] = a.w;
    g.M[4] = b.x; g.M[5] = b.y; g.M[6] = b.z; g.M[7] = b.w; g.M[8] = c;
}

__device__ __forceinline__ void bary32(const Geo32 &g, float x, float y, float z, float l[4]) {
    l[1] = fmaf(g.M[2], z, fmaf(g.M[1], y, fmaf(g.M[0], x, 0.25f)));
    l[2] = fmaf(g.M[5], z, fmaf(g.M[4], y, fmaf(g.M[3], x, 0.25f)));
    l[3] = fmaf(g.M[8], z, fmaf(g.M[7], y, fmaf(g.M[6], x, 0.25f)));
    l[0] = 1.0f - l[1] - l[2] - l[3];
}

// FP64 barycentrics of an FP32 local position (near-zero decisions).
__device__ __noinline__ void bary64_local(const TetRec *__restrict__ rec64, int t, float x, float y, float z,
                                         float l[4]) {
    const double *M = rec64[t].M;
    const double dx = x, dy = y, dz = z;
    const double l1 = 0.25 + (M[0] * dx + M[1] * dy + M[2] * dz);
    const double l2 = 0.25 + (M[3] * dx + M[4] * dy + M[5] * dz);
    const double l3 = 0.25 + (M[6] * dx + M[7] * dy + M[8] * dz);
    const double l0 = 1.0 - l1 - l2 - l3;
    // keep only the sign information exactly; magnitudes are FP32-rounded
    l[0] = float(l0);
    l[1] = float(l1);
    l[2] = float(l2);
    l[3] = float(l3);
    for (int k = 0; k < 4; ++k)
        if (l[k] == 0.0f && (k == 0 ? l0 : (k == 1 ? l1 : (k == 2 ? l2 : l3))) < 0.0) l[k] = -1e-30f;
}

// The modelling-box test of a global FP32 position (the particle's tet's
// centroid plus its local position).
__device__ __forceinline__ bool in_box32(const StepConst &c, float gx, float gy, float gz) {
    return gx >= c.lo_f[0] && gx <= c.hi_f[0] && gy >= c.lo_f[1] && gy <= c.hi_f[1] && gz >= c.lo_f[2] &&
           gz <= c.hi_f[2];
}

__device__ __forceinline__ int comp(const int4 &v, int f) {
    return f == 0 ? v.x : (f == 1 ? v.y : (f == 2 ? v.z : v.w));
}

struct MixedArgs {
    DevParticles32 p;
    int64_t n;
    const TetRec32 *rec;
    const TetRec *rec64;
    const double *cen;    // 3 per tet
    const float *cen_lo;  // 3 per tet: cen - hi, hi the record's FP32 centroid
    const int4 *nbr, *ftri, *tet_nodes;
    int64_t n_tets;
};

// Inside test of an end point with FP64 rescue near zero.
__device__ __forceinline__ bool inside32(const MixedArgs &a, const Geo32 &g, int t, float x, float y, float z,
                                         float l[4]) {
    bary32(g, x, y, z, l);
    const float mn = fminf(fminf(l[0], l[1]), fminf(l[2], l[3]));
    if (mn > kNearZero) return true;
    if (mn < -kNearZero) return false;
    bary64_local(a.rec64, t, x, y, z, l);
    return l[0] >= 0.0f && l[1] >= 0.0f && l[2] >= 0.0f && l[3] >= 0.0f;
}

// Centroid of a tet as an unevaluated FP32 pair: c = hi + lo to about 2^-48
// relative (hi is the FP32 centroid of the tet's record).
struct Cen2 {
    float hx, hy, hz, lx, ly, lz;
};

__device__ __forceinline__ Cen2 load_cen2(const TetRec32 *__restrict__ rec, const float *__restrict__ cen_lo, int t) {
    const float4 c = __ldg(reinterpret_cast<const float4 *>(rec + t) + 3);
    return Cen2{c.x, c.y, c.z, __ldg(cen_lo + 3 * t), __ldg(cen_lo + 3 * t + 1), __ldg(cen_lo + 3 * t + 2)};
}

// Offset c_a - c_b of one coordinate as a pair (s, e): Knuth's TwoSum gives
// s + e = ah - bh exactly, the low parts are added to e.
__device__ __forceinline__ void cen_diff(float ah, float al, float bh, float bl, float &s, float &e) {
    s = ah - bh;
    const float bb = s - ah;
    e = ((ah - (s - bb)) + (-bh - bb)) + (al - bl);
}

// x + (s + e) rounded once in effect: TwoSum(x, s), then the low parts.
// Equal to the FP32 rounding of the exact sum except within ~2^-48 |c| of a
// rounding midpoint, so the re-based position is as good as one formed in
// FP64, with FP32 operations only.
__device__ __forceinline__ float add2(float x, float s, float e) {
    const float t = x + s;
    const float bb = t - x;
    const float err = (x - (t - bb)) + (s - bb);
    return t + (err + e);
}

// Re-base the local positions p0, p1 from tet a's frame to tet b's:
// p + (c_a - c_b).
__device__ __forceinline__ void rebase2(const Cen2 &a, const Cen2 &b, float &p0x, float &p0y, float &p0z, float &p1x,
                                        float &p1y, float &p1z) {
    float s, e;
    cen_diff(a.hx, a.lx, b.hx, b.lx, s, e);
    p0x = add2(p0x, s, e);
    p1x = add2(p1x, s, e);
    cen_diff(a.hy, a.ly, b.hy, b.ly, s, e);
    p0y = add2(p0y, s, e);
    p1y = add2(p1y, s, e);
    cen_diff(a.hz, a.lz, b.hz, b.lz, s, e);
    p0z = add2(p0z, s, e);
    p1z = add2(p1z, s, e);
}

struct Walk32 {
    int tet, status, tri, crossings, face;
    float hx, hy, hz;  // end (or hit) point in the final tet's frame
    float s;           // crossing parameter of the hit (W_SURFACE)
};

// Segment walk in local frames: p0, p1 are given in tet t's frame and are
// re-based on every crossing (FP32 pair arithmetic). Same exit rule as the
// FP64 walk (smallest crossing parameter among faces with lambda(p1) < 0,
// entry face excluded).
__device__ __noinline__ Walk32 walk32(const MixedArgs a, int t, float p0x, float p0y, float p0z, float p1x,
                                      float p1y, float p1z, int max_cross) {
    Walk32 o;
    o.crossings = 0;
    o.tri = -1;
    o.face = -1;
    o.s = 1.0f;
    int enter = -1;
    Geo32 g;
    load_geo32(a.rec, t, g);
    Cen2 ca = load_cen2(a.rec, a.cen_lo, t);
    for (;;) {
        float l1[4];
        if (inside32(a, g, t, p1x, p1y, p1z, l1)) {
            o.tet = t;
            o.status = W_INSIDE;
            o.hx = p1x;
            o.hy = p1y;
            o.hz = p1z;
            return o;
        }
        float l0[4];
        bary32(g, p0x, p0y, p0z, l0);
        int best = -1;
        float sb = 0.0f;
#pragma unroll
        for (int f = 0; f < 4; ++f) {
            if (f == enter || !(l1[f] < 0.0f)) continue;
            const float s = l0[f] / (l0[f] - l1[f]);
            if (best < 0 || s < sb) {
                best = f;
                sb = s;
            }
        }
        if (best < 0) {
            o.tet = t;
            o.status = W_INSIDE;
            o.hx = p1x;
            o.hy = p1y;
            o.hz = p1z;
            return o;
        }
        const int tri = comp(__ldg(a.ftri + t), best);
        if (tri >= 0) {
            o.tet = t;
            o.status = W_SURFACE;
            o.tri = tri;
            o.face = best;
            o.s = sb;
            o.hx = fmaf(sb, p1x - p0x, p0x);
            o.hy = fmaf(sb, p1y - p0y, p0y);
            o.hz = fmaf(sb, p1z - p0z, p0z);
            return o;
        }
        const int nb = comp(__ldg(a.nbr + t), best);
        if (nb < 0 || o.crossings == max_cross) {
            o.tet = t;
            o.status = nb < 0 ? W_EXIT : W_CAP;
            o.hx = p1x;
            o.hy = p1y;
            o.hz = p1z;
            return o;
        }
        o.crossings++;
        const int tn = nb >> 2;
        const Cen2 cb = load_cen2(a.rec, a.cen_lo, tn);
        rebase2(ca, cb, p0x, p0y, p0z, p1x, p1y, p1z);
        ca = cb;
        t = tn;
        enter = nb & 3;
        load_geo32(a.rec, t, g);
    }
}

// Whether step `step` is a candidate: its byte of the step's Philox block
// (one per sixteen steps) is zero.
__device__ __forceinline__ bool is_candidate(const StepConst &c, uint32_t id, uint64_t step) {
    return candidate_byte(candidate_block(step, id, c.seed_lo, c.seed_hi), step) == 0u;
}

// |v|^2 in the order every FP32 collision test and slow-particle test uses.
__device__ __forceinline__ float speed2(float vx, float vy, float vz) { return fmaf(vz, vz, fmaf(vy, vy, vx * vx)); }

// FP32 collision test of step `step` (the candidate-byte rule of philox.h
// with P_f = kp (v^2)^pexp; `cand`: the step's candidate byte is zero; v2 =
// speed2 of the velocity) and, on a hit, the scattering direction's cosine
// xc, sine xs and azimuth (cos, sin). A step that is no candidate with
// v^2 <= v2_cand_f has P_f < q: no collision, decided without P_f.
__device__ __forceinline__ bool collision_event32(const StepConst &c, uint32_t id, uint64_t step, bool cand,
                                                  float v2, float &xc, float &xs, float &cp, float &sp) {
    constexpr float qf = float(kCandQ);
    if (!cand && v2 <= c.v2_cand_f) return false;
    const float P = c.kp_f * exp2f(c.pexp_f * log2f(v2));
    bool hit;
    if (cand)
        hit = P > qf || float(collision_draw(step, 3u, id, c.seed_lo, c.seed_hi).v[0] >> 8) *
                                5.9604644775390625e-8f < P * 256.0f;
    else
        hit = P > qf && float(collision_draw(step, 4u, id, c.seed_lo, c.seed_hi).v[0] >> 8) *
                                5.9604644775390625e-8f < (P - qf) / (1.0f - qf);
    if (!hit) return false;
    const Philox4 r = collision_draw(step, 1u, id, c.seed_lo, c.seed_hi);
    const float u1 = float(r.v[0] >> 8) * 5.9604644775390625e-8f;
    const float u2 = float(r.v[2] >> 8) * 5.9604644775390625e-8f;
    if (c.model == SPG_COLL_HS)
        xc = -1.0f + 2.0f * u1;
    else if (c.model == SPG_COLL_VHS)
        xc = u1;
    else
        xc = 2.0f * powf(u1, c.inv_alpha_f) - 1.0f;
    xs = sqrtf(fmaxf(0.0f, 1.0f - xc * xc));
    sincosf((2.0f * kPiF) * u2, &sp, &cp);
    return true;
}

// Collision of step `step` in FP32 (same Philox streams and laws as the FP64
// form); `cand` and v2 as for collision_event32.
__device__ __forceinline__ bool collide32(const StepConst &c, uint32_t id, uint64_t step, bool cand, float v2,
                                          float &vx, float &vy, float &vz) {
    float xc, xs, cp, sp;
    if (!collision_event32(c, id, step, cand, v2, xc, xs, cp, sp)) return false;
    const float mcp = c.mass_cp_f, mct = c.mass_ct_f;
    const float pvx = mct * vx, pvy = mct * vy, pvz = mct * vz;
    const float mp = sqrtf(fmaf(pvz, pvz, fmaf(pvy, pvy, pvx * pvx)));
    float ex = xs * cp * mp, ey = xs * sp * mp, ez = xc * mp;
    if (c.model == SPG_COLL_VSS && mp > 0.0f) {
        // rotation by (beta, gamma) of the relative velocity, without the
        // angles: cos beta = pz/|p|, sin beta >= 0; (cos, sin) gamma from (px, py)
        const float cb = pvz / mp, sb = sqrtf(fmaxf(0.0f, 1.0f - cb * cb));
        const float rxy = sqrtf(fmaf(pvy, pvy, pvx * pvx));
        const float cg = rxy > 0.0f ? pvx / rxy : 1.0f, sg = rxy > 0.0f ? pvy / rxy : 0.0f;
        const float tx = cb * ex + sb * ez, tz = -sb * ex + cb * ez;
        ex = cg * tx - sg * ey;
        ey = sg * tx + cg * ey;
        ez = tz;
    }
    vx = fmaf(vx, mcp, ex);
    vy = fmaf(vy, mcp, ey);
    vz = fmaf(vz, mcp, ez);
    return true;
}

struct WalkItem32 {
    int32_t i;
    float x0, y0, z0;
};

// The eight 4-byte words of one particle.
struct Words32 {
    uint32_t idf;
    int t;
    float x, y, z, vx, vy, vz;
};

__device__ __forceinline__ Words32 load_words32(const DevParticles32 &p, int64_t i) {
    Words32 w;
    w.idf = p.idf[i];
    w.t = p.tet[i];
    w.x = p.x[i];
    w.y = p.y[i];
    w.z = p.z[i];
    w.vx = p.vx[i];
    w.vy = p.vy[i];
    w.vz = p.vz[i];
    return w;
}

// Append of this lane's item to the walk queue where the lane decides (the
// lanes converged there share one atomic; queue order does not matter).
__device__ __forceinline__ void queue_walk32(WalkItem32 *__restrict__ q, unsigned int *__restrict__ qn, int64_t i,
                                             float x, float y, float z) {
    const unsigned act = __activemask();
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(act) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(qn, unsigned(__popc(act)));
    base = __shfl_sync(act, base, leader);
    WalkItem32 &w = q[base + __popc(act & ((1u << lane) - 1u))];
    w.i = int32_t(i);
    w.x0 = x;
    w.y0 = y;
    w.z0 = z;
}

// Grid-stride over the particles: the next particle's words are loaded
// before the current one is computed, so each thread keeps a particle's
// loads in flight while it works (the kernel is bound by memory latency).
__global__ void __launch_bounds__(256, 4) k_step32(MixedArgs a, StepConst c, WalkItem32 *__restrict__ wq,
                                                unsigned int *__restrict__ wq_n, DevCounters *ctr) {
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    unsigned processed = 0, coll = 0, lost = 0;
    Words32 cur{};
    if (i < a.n) cur = load_words32(a.p, i);
    for (; i < a.n; i += stride) {
        Words32 nxt{};
        if (i + stride < a.n) nxt = load_words32(a.p, i + stride);
        const uint32_t idf = cur.idf;
        const int t = cur.t;
        const float x = cur.x, y = cur.y, z = cur.z;
        float vx = cur.vx, vy = cur.vy, vz = cur.vz;
        cur = nxt;
        if (idf & kDead) continue;
        processed++;
        // The whole 64-byte record in one round trip: M[0..7], {M[8], H}, {cen, ezero}.
        const float4 *rp = reinterpret_cast<const float4 *>(a.rec + t);
        const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1), r2 = __ldg(rp + 2), r3 = __ldg(rp + 3);
        const float vmin = c.vmin_f;
        const bool slow = fmaf(vz, vz, fmaf(vy, vy, vx * vx)) < vmin * vmin;
        const uint32_t flags = __float_as_uint(r3.w);
        if (slow || (!(flags & kRecInterior) && !in_box32(c, r3.x + x, r3.y + y, r3.z + z))) continue;
        if (!(flags & kRecEzero)) {
            const float hx = r2.y, hy = r2.z, hz = r2.w;
            vx = (vx + hx) + hx;
            vy = (vy + hy) + hy;
            vz = (vz + hz) + hz;
        }
        const float dt = c.dt_f;
        const float nx = fmaf(vx, dt, x), ny = fmaf(vy, dt, y), nz = fmaf(vz, dt, z);
        if (!(nx == x && ny == y && nz == z)) {
            // The walk decision needs only the positions, so it comes before the
            // collision (which changes the velocity alone) and the map's registers
            // are free again when the collision runs.
            if (!(isfinite(nx) && isfinite(ny) && isfinite(nz))) {
                a.p.idf[i] = idf | kLost;
                lost++;
            } else {
                const Geo32 g{{r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w, r2.x}};
                float l[4];
                bary32(g, nx, ny, nz, l);
                const float mn = fminf(fminf(l[0], l[1]), fminf(l[2], l[3]));
                if (!(mn > kNearZero)) queue_walk32(wq, wq_n, i, x, y, z);
                a.p.x[i] = nx;
                a.p.y[i] = ny;
                a.p.z[i] = nz;
            }
            if (c.model != SPG_COLL_NONE) {
                const uint32_t id = idf & kIdMask;
                const uint64_t step = uint64_t(c.step);
                coll += collide32(c, id, step, is_candidate(c, id, step), speed2(vx, vy, vz), vx, vy, vz) ? 1u : 0u;
            }
        }
        a.p.vx[i] = vx;
        a.p.vy[i] = vy;
        a.p.vz[i] = vz;
    }
    const unsigned long long s0 = __reduce_add_sync(kFull, processed), s1 = __reduce_add_sync(kFull, coll);
    const unsigned long long s2 = __reduce_add_sync(kFull, lost);
    if ((threadIdx.x & 31) == 0) {
        if (s0) atomicAdd(&ctr->processed, s0);
        if (s1) atomicAdd(&ctr->collisions, s1);
        if (s2) atomicAdd(&ctr->lost, s2);
    }
}

// Mixed form: E per tet in FP64 from phi (the FP32 potential differences
// across a tet would lose the field), then the FP32 push increment
// H = float(E c) with c = q dt / (2 m) formed once on the host, so no FP64
// division runs per tet. The FP64 record of the plain form is not touched.
__device__ __forceinline__ void field_of_tet32(const FieldArgs &f, int64_t t) {
    const int4 tn = __ldg(f.tet_nodes + t);
    const double f0 = f.phi[tn.x], f1 = f.phi[tn.y], f2 = f.phi[tn.z], f3 = f.phi[tn.w];
    const double d1 = f1 - f0, d2 = f2 - f0, d3 = f3 - f0;
    const TetRec &r = f.rec[t];
    double E[3];
    // Explicitly rounded products and sums: this file is built with FMA
    // contraction on, and E is the FP64 field the oracle computes unfused.
#pragma unroll
    for (int k = 0; k < 3; ++k)
        E[k] = -__dadd_rn(__dadd_rn(__dmul_rn(d1, r.M[k]), __dmul_rn(d2, r.M[3 + k])), __dmul_rn(d3, r.M[6 + k]));
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        f.efield[3 * t + k] = E[k];
        f.rec32[t].H[k] = float(E[k] * f.c32);
    }
    const bool null_field = E[0] == 0.0 && E[1] == 0.0 && E[2] == 0.0;
    f.rec32[t].ezero = (f.rec32[t].ezero & kRecInterior) | (null_field ? kRecEzero : 0u);
}

// With land != nullptr a particle that settles records the step, the exit
// face, its tet and the hit fraction (adjoint).
__global__ void __launch_bounds__(128) k_walk_queue32(MixedArgs a, int max_cross, const WalkItem32 *__restrict__ wq,
                                                      const unsigned int *__restrict__ wq_n,
                                                      unsigned int *__restrict__ tri_count, DevCounters *ctr,
                                                      LandRec *__restrict__ land, int64_t step,
                                                      const __grid_constant__ FieldArgs f) {
    const unsigned nq = *wq_n;
    unsigned cross = 0, settled = 0, lost = 0, capped = 0;
    for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x) {
        const WalkItem32 it = wq[q];
        const int64_t i = it.i;
        const int t = a.p.tet[i];
        const Walk32 w = walk32(a, t, it.x0, it.y0, it.z0, a.p.x[i], a.p.y[i], a.p.z[i], max_cross);
        cross += unsigned(w.crossings);
        a.p.x[i] = w.hx;
        a.p.y[i] = w.hy;
        a.p.z[i] = w.hz;
        const uint32_t idf = a.p.idf[i];
        if (w.status == W_SURFACE) {
            atomicAdd(tri_count + w.tri, 1u);
            a.p.idf[i] = idf | kSettled;
            settled++;
            if (land) {
                land[i].step = int32_t(step);
                land[i].face = w.face;
                land[i].tet = w.tet;
                land[i].s = double(w.s);
            }
        } else if (w.status != W_INSIDE) {
            a.p.idf[i] = idf | kLost;
            lost++;
            if (w.status == W_CAP) capped++;
        }
        if (w.tet != t) {
            a.p.tet[i] = w.tet;
            if (w.status == W_INSIDE) refresh_tet(f.stamp, f.epoch, w.tet, [&f](int tt) { field_of_tet32(f, tt); });
        }
    }
    const unsigned long long s0 = __reduce_add_sync(kFull, cross), s1 = __reduce_add_sync(kFull, settled);
    const unsigned long long s2 = __reduce_add_sync(kFull, lost), s3 = __reduce_add_sync(kFull, capped);
    if ((threadIdx.x & 31) == 0) {
        if (s0) atomicAdd(&ctr->crossings, s0);
        if (s1) atomicAdd(&ctr->settled, s1);
        if (s2) atomicAdd(&ctr->lost, s2);
        if (s3) atomicAdd(&ctr->capped, s3);
    }
}

// ---------------------------------------------------------------------------
// Segmented step: every step between two events of the time loop (a solve,
// a re-sort, the end of the call) in one pass over the particles. A particle
// keeps its state and its tet's record in registers and leaves the pass at
// the first step whose move needs the exact walk; it is queued with that
// step's index, the walk kernel walks it, and a resume pass runs it on from
// the next step. Each pass reads only fields that earlier launches wrote (a
// walk computes the field of the tet it enters; the particle is stepped
// there in the next launch), and every particle goes through the same FP32
// operations in the same order as in single steps, so the result is
// bit-identical to stepping one step per launch.

constexpr int kMaxSegment = 64;  // steps per segment at most

struct SegItem32 {  // a move of step s0 + step that needs the walk
    int32_t i, step;
    float x0, y0, z0;
};

struct SegQueues {
    SegItem32 *wq;           // walk items of the current round (at most one per particle)
    int2 *rq;                // resumed particles: {index, first step}
    unsigned int *wq_n;      // [L + 1]: walk items of round r
    unsigned int *rq_n;      // [L]: resumed particles of round r
    int L;                   // steps of the segment (steps s0 .. s0 + L - 1)
};

__device__ __forceinline__ void queue_seg32(SegItem32 *__restrict__ q, unsigned int *__restrict__ qn, int64_t i,
                                            int j, float x, float y, float z) {
    const unsigned act = __activemask();
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(act) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(qn, unsigned(__popc(act)));
    base = __shfl_sync(act, base, leader);
    SegItem32 &w = q[base + __popc(act & ((1u << lane) - 1u))];
    w.i = int32_t(i);
    w.step = j;
    w.x0 = x;
    w.y0 = y;
    w.z0 = z;
}

// Steps j0 .. L - 1 of particle i (state w, alive) in registers: the
// operations of k_step32 for each step. Leaves at the segment's end, when the
// particle is lost, when it stays put for good (too slow or outside the
// modelling box: nothing changes it any more) or with its move queued for
// the walk (round r's items go to wq_n[r]).
__device__ __forceinline__ void seg_steps32(const MixedArgs &a, const StepConst &c, int64_t i, const Words32 &w,
                                            int j0, const SegQueues &sq, unsigned int *__restrict__ qn,
                                            unsigned &processed, unsigned &coll, unsigned &lost) {
    const float4 *rp = reinterpret_cast<const float4 *>(a.rec + w.t);
    const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1), r2 = __ldg(rp + 2), r3 = __ldg(rp + 3);
    const Geo32 g{{r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w, r2.x}};
    const uint32_t flags = __float_as_uint(r3.w);
    const bool push = !(flags & kRecEzero), interior = flags & kRecInterior;
    const float hx = r2.y, hy = r2.z, hz = r2.w;
    const uint32_t id = w.idf & kIdMask;
    float x = w.x, y = w.y, z = w.z, vx = w.vx, vy = w.vy, vz = w.vz;
    const float vmin2 = c.vmin_f * c.vmin_f, dt = c.dt_f;
    float v2 = speed2(vx, vy, vz);  // of the current velocity
    bool dirty = false;
    // the candidate steps of the last sixteen-step group tested (cgroup: the
    // low 32 bits of its count; steps in a segment are consecutive, so the
    // key changes exactly when the group does)
    uint32_t cmask = 0u, cgroup = ~0u;
    const uint32_t step_lo = uint32_t(c.step);
    auto collide = [&](int j) -> unsigned {
        const uint32_t sj = step_lo + uint32_t(j);
        const uint64_t step = uint64_t(c.step) + uint64_t(j);
        if ((sj >> 4) != cgroup) {
            cgroup = sj >> 4;
            cmask = candidate_mask(candidate_block(step, id, c.seed_lo, c.seed_hi));
        }
        if (!collide32(c, id, step, (cmask >> (sj & 15u)) & 1u, v2, vx, vy, vz)) return 0u;
        v2 = speed2(vx, vy, vz);
        return 1u;
    };
    for (int j = j0; j < sq.L; ++j) {
        processed++;
        const bool slow = v2 < vmin2;
        if (slow || (!interior && !in_box32(c, r3.x + x, r3.y + y, r3.z + z))) {
            processed += unsigned(sq.L - 1 - j);
            break;
        }
        if (push) {
            vx = (vx + hx) + hx;
            vy = (vy + hy) + hy;
            vz = (vz + hz) + hz;
            v2 = speed2(vx, vy, vz);
            dirty = true;
        }
        const float nx = fmaf(vx, dt, x), ny = fmaf(vy, dt, y), nz = fmaf(vz, dt, z);
        if (nx == x && ny == y && nz == z) continue;
        if (!(isfinite(nx) && isfinite(ny) && isfinite(nz))) {
            a.p.idf[i] = w.idf | kLost;
            lost++;
            if (c.model != SPG_COLL_NONE) coll += collide(j);
            a.p.x[i] = x;
            a.p.y[i] = y;
            a.p.z[i] = z;
            a.p.vx[i] = vx;
            a.p.vy[i] = vy;
            a.p.vz[i] = vz;
            return;
        }
        float l[4];
        bary32(g, nx, ny, nz, l);
        const float mn = fminf(fminf(l[0], l[1]), fminf(l[2], l[3]));
        if (!(mn > kNearZero)) {
            queue_seg32(sq.wq, qn, i, j, x, y, z);
            if (c.model != SPG_COLL_NONE) coll += collide(j);
            a.p.x[i] = nx;
            a.p.y[i] = ny;
            a.p.z[i] = nz;
            a.p.vx[i] = vx;
            a.p.vy[i] = vy;
            a.p.vz[i] = vz;
            return;
        }
        x = nx;
        y = ny;
        z = nz;
        if (c.model != SPG_COLL_NONE) coll += collide(j);
        dirty = true;
    }
    if (dirty) {
        a.p.x[i] = x;
        a.p.y[i] = y;
        a.p.z[i] = z;
        a.p.vx[i] = vx;
        a.p.vy[i] = vy;
        a.p.vz[i] = vz;
    }
}

__device__ __forceinline__ void add_step_counters(DevCounters *ctr, unsigned processed, unsigned coll,
                                                  unsigned lost) {
    const unsigned long long s0 = __reduce_add_sync(kFull, processed), s1 = __reduce_add_sync(kFull, coll);
    const unsigned long long s2 = __reduce_add_sync(kFull, lost);
    if ((threadIdx.x & 31) == 0) {
        if (s0) atomicAdd(&ctr->processed, s0);
        if (s1) atomicAdd(&ctr->collisions, s1);
        if (s2) atomicAdd(&ctr->lost, s2);
    }
}

// The segment's first pass over every particle (grid-stride, the next
// particle's words loaded before the current one is stepped).
__global__ void __launch_bounds__(256, 3) k_seg32(MixedArgs a, StepConst c, SegQueues sq, DevCounters *ctr) {
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    unsigned processed = 0, coll = 0, lost = 0;
    Words32 cur{};
    if (i < a.n) cur = load_words32(a.p, i);
    for (; i < a.n; i += stride) {
        Words32 nxt{};
        if (i + stride < a.n) nxt = load_words32(a.p, i + stride);
        if (!(cur.idf & kDead)) seg_steps32(a, c, i, cur, 0, sq, sq.wq_n, processed, coll, lost);
        cur = nxt;
    }
    add_step_counters(ctr, processed, coll, lost);
}

// Round r's walks (the queued moves, each of its own step); a particle still
// inside with steps left is listed for the resume pass of round r.
__global__ void __launch_bounds__(128) k_seg_walk32(MixedArgs a, int max_cross, SegQueues sq, int r,
                                                    unsigned int *__restrict__ tri_count, DevCounters *ctr,
                                                    const __grid_constant__ FieldArgs f) {
    pdl_sync();
    const unsigned nq = sq.wq_n[r];
    unsigned cross = 0, settled = 0, lost = 0, capped = 0;
    for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x) {
        const SegItem32 it = sq.wq[q];
        const int64_t i = it.i;
        const int t = a.p.tet[i];
        const Walk32 w = walk32(a, t, it.x0, it.y0, it.z0, a.p.x[i], a.p.y[i], a.p.z[i], max_cross);
        cross += unsigned(w.crossings);
        a.p.x[i] = w.hx;
        a.p.y[i] = w.hy;
        a.p.z[i] = w.hz;
        const uint32_t idf = a.p.idf[i];
        if (w.status == W_SURFACE) {
            atomicAdd(tri_count + w.tri, 1u);
            a.p.idf[i] = idf | kSettled;
            settled++;
        } else if (w.status != W_INSIDE) {
            a.p.idf[i] = idf | kLost;
            lost++;
            if (w.status == W_CAP) capped++;
        }
        if (w.tet != t) {
            a.p.tet[i] = w.tet;
            if (w.status == W_INSIDE) refresh_tet(f.stamp, f.epoch, w.tet, [&f](int tt) { field_of_tet32(f, tt); });
        }
        if (w.status == W_INSIDE && it.step + 1 < sq.L) {
            const unsigned act = __activemask();
            const int lane = threadIdx.x & 31;
            const int leader = __ffs(act) - 1;
            unsigned base = 0;
            if (lane == leader) base = atomicAdd(sq.rq_n + r, unsigned(__popc(act)));
            base = __shfl_sync(act, base, leader);
            sq.rq[base + __popc(act & ((1u << lane) - 1u))] = make_int2(int(i), it.step + 1);
        }
    }
    const unsigned long long s0 = __reduce_add_sync(kFull, cross), s1 = __reduce_add_sync(kFull, settled);
    const unsigned long long s2 = __reduce_add_sync(kFull, lost), s3 = __reduce_add_sync(kFull, capped);
    if ((threadIdx.x & 31) == 0) {
        if (s0) atomicAdd(&ctr->crossings, s0);
        if (s1) atomicAdd(&ctr->settled, s1);
        if (s2) atomicAdd(&ctr->lost, s2);
        if (s3) atomicAdd(&ctr->capped, s3);
    }
}

// Round r's resume pass: the walked particles run on in registers from the
// step after their walk; their next walk goes to round r + 1. (Ordering each
// block's items by first step, so that a warp's lanes run the same steps,
// cost more in block barriers than it saved in idle lanes.)
__global__ void __launch_bounds__(256, 3) k_seg_resume32(MixedArgs a, StepConst c, SegQueues sq, int r,
                                                         DevCounters *ctr) {
    pdl_sync();
    const unsigned nr = sq.rq_n[r];
    unsigned processed = 0, coll = 0, lost = 0;
    for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < nr; q += gridDim.x * blockDim.x) {
        const int2 it = sq.rq[q];
        const Words32 w = load_words32(a.p, it.x);
        seg_steps32(a, c, it.x, w, it.y, sq, sq.wq_n + r + 1, processed, coll, lost);
    }
    add_step_counters(ctr, processed, coll, lost);
}

// round(x * 2^k) of a float (k <= 52), to nearest with ties to even, from the
// float's bits with 32-bit integer operations: a conversion to a 64-bit
// integer issues on the FP64 pipe, three per particle. x = mant 2^(e - 150),
// so x 2^k = mant 2^-sh with sh = 150 - e - k; a left shift past 39 bits
// (|x| 2^k >= 2^63, no barycentric) is clamped.
__device__ __forceinline__ long long fix_round32(float x, int k) {
    const int b = __float_as_int(x);
    const int e = (b >> 23) & 0xff;
    if (e == 0) return 0;  // zero or subnormal: |x| 2^k < 2^-74
    const unsigned mant = unsigned(b & 0x7FFFFF) | 0x800000u;
    const int sh = 150 - e - k;
    unsigned long long r;
    if (sh <= 0) {
        r = (unsigned long long)mant << min(-sh, 39);
    } else if (sh > 24) {
        r = 0;  // below half of one: mant < 2^24 <= 2^(sh - 1)
    } else {
        const unsigned q = mant >> sh, rem = mant & ((1u << sh) - 1u), half = 1u << (sh - 1);
        r = q + ((rem > half || (rem == half && (q & 1u))) ? 1u : 0u);
    }
    return b < 0 ? -(long long)r : (long long)r;
}

// The mixed form's particles for deposit_tiles: FP32 barycentrics of the
// tet-local position (20 B per particle).
struct DepSrc32 {
    struct Raw {
        uint32_t idf;
        int32_t tet;
        float x, y, z;
    };
    DevParticles32 p;
    const TetRec32 *rec;
    int k;
    long long one;
    __device__ __forceinline__ Raw load(int64_t i, int64_t n) const {
        Raw r{kDead, -1, 0.f, 0.f, 0.f};
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
        Geo32 g;
        load_geo32(rec, r.tet, g);
        float l[4];
        bary32(g, r.x, r.y, r.z, l);
        v[1] = fix_round32(l[1], k);
        v[2] = fix_round32(l[2], k);
        v[3] = fix_round32(l[3], k);
        v[0] = one - v[1] - v[2] - v[3];
        return r.tet;
    }
};

__global__ void __launch_bounds__(kDepThreads)
    k_deposit32(const DepSrc32 src, int64_t n, const int4 *__restrict__ tet_nodes,
                unsigned long long *__restrict__ node_fix, const OccList occ) {
    deposit_tiles(src, n, tet_nodes, node_fix, occ);
}

// The field of the tets listed by the deposit (each once).
__global__ void k_field32_list(const __grid_constant__ FieldArgs f, const int32_t *__restrict__ list,
                               const unsigned int *__restrict__ list_n) {
    const unsigned nl = *list_n;
    for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < nl; j += gridDim.x * blockDim.x) {
        const int t = list[j];
        field_of_tet32(f, t);
        f.stamp[t] = f.epoch;
    }
}

__global__ void k_field32_full(const __grid_constant__ FieldArgs f, int64_t n) {
    const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= n) return;
    field_of_tet32(f, t);
    f.stamp[t] = f.epoch;
}

// The field of every tet holding an alive particle. Particles are tet-sorted
// (up to the drift since the last re-sort), so only the first lane of each
// run of equal tets in a warp checks the stamp.
__global__ void k_refresh32(DevParticles32 p, int64_t n, const __grid_constant__ FieldArgs f) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int key = (i < n && !(p.idf[i] & kDead)) ? p.tet[i] : -1;
    const int prev = __shfl_up_sync(kFull, key, 1);
    if (key >= 0 && ((threadIdx.x & 31) == 0 || prev != key))
        refresh_tet(f.stamp, f.epoch, key, [&f](int t) { field_of_tet32(f, t); });
}

// Global FP64 state -> local FP32 state (and back).
__global__ void k_to_local(const double *__restrict__ pos, const double *__restrict__ vel,
                           const int32_t *__restrict__ tet, const double *__restrict__ cen, int64_t n,
                           DevParticles32 p, int64_t id_base) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t j = id_base + i;
    const int32_t t = tet[i];
    const int64_t tc = t < 0 ? 0 : t;
    p.x[j] = float(pos[3 * i] - (t < 0 ? 0.0 : cen[3 * tc]));
    p.y[j] = float(pos[3 * i + 1] - (t < 0 ? 0.0 : cen[3 * tc + 1]));
    p.z[j] = float(pos[3 * i + 2] - (t < 0 ? 0.0 : cen[3 * tc + 2]));
    p.vx[j] = float(vel[3 * i]);
    p.vy[j] = float(vel[3 * i + 1]);
    p.vz[j] = float(vel[3 * i + 2]);
    p.tet[j] = t;
    p.idf[j] = uint32_t(j) | (t < 0 ? kLost : 0u);
}

// One thread per id (slot from launch_slot_of_id): coalesced writes in id order.
// One thread per id, writes in id order; the block's xyz triples go out
// through shared memory as one contiguous run per array (whole lines per warp
// store, also when the arrays are the caller's pinned host memory).
__global__ void __launch_bounds__(256) k_gather32(DevParticles32 p, int64_t n, const int32_t *__restrict__ slot,
                                                  const double *__restrict__ cen, double *pos, double *vel,
                                                  int32_t *tet, uint32_t *flags) {
    __shared__ double sp[3 * 256], sv[3 * 256];
    const int64_t id0 = int64_t(blockIdx.x) * 256;
    const int64_t id = id0 + threadIdx.x;
    const int m = n - id0 < 256 ? int(n - id0) : 256;
    if (id < n) {
        const int64_t i = slot[id];
        const uint32_t idf = p.idf[i];
        const int32_t t = p.tet[i];
        const int64_t tc = t < 0 ? 0 : t;
        const double ox = t < 0 ? 0.0 : cen[3 * tc], oy = t < 0 ? 0.0 : cen[3 * tc + 1],
                     oz = t < 0 ? 0.0 : cen[3 * tc + 2];
        if (pos) {
            sp[3 * threadIdx.x] = ox + double(p.x[i]);
            sp[3 * threadIdx.x + 1] = oy + double(p.y[i]);
            sp[3 * threadIdx.x + 2] = oz + double(p.z[i]);
        }
        if (vel) {
            sv[3 * threadIdx.x] = p.vx[i];
            sv[3 * threadIdx.x + 1] = p.vy[i];
            sv[3 * threadIdx.x + 2] = p.vz[i];
        }
        if (tet) tet[id] = t;
        if (flags) flags[id] = ((idf & kSettled) ? SPG_FLAG_SETTLED : 0u) | ((idf & kLost) ? SPG_FLAG_LOST : 0u);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 3 * m; k += 256) {
        if (pos) pos[3 * id0 + k] = sp[k];
        if (vel) vel[3 * id0 + k] = sv[k];
    }
}

__global__ void __launch_bounds__(kSortBlock) k_sort_scatter32(DevParticles32 src, DevParticles32 dst, int64_t n,
                                                               int n_tets, int32_t *__restrict__ offs) {
    __shared__ SortTable t;
    sort_scatter_block(t, src, dst, n, n_tets, kDead, offs);
}

inline unsigned grid_for(int64_t n, int block) { return unsigned((n + block - 1) / block); }

// ------------------------------------------------------------ adjoint (FP32 form)
// The gradient of the FP32 step itself: the recorded FP32 velocities and the
// FP32 push increments rebuild the pushed velocity exactly as the forward
// computed it, and the adjoint recursion (the one of the FP64 form, see
// kernels_adjoint.cu) runs in FP64 on those values. Collision events are the
// FP32 form's own decisions, recomputed from the same FP32 velocity.

__global__ void k_record32(DevParticles32 p, int64_t n, AdjHist h, int k) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t o = int64_t(k) * n + i;
    h.tet[o] = (p.idf[i] & kDead) ? -1 : p.tet[i];
    h.vx[o] = double(p.vx[i]);
    h.vy[o] = double(p.vy[i]);
    h.vz[o] = double(p.vz[i]);
}

// dg/dr of each landed particle (r = centroid + local position, in FP64) and
// the sums of g and of the landed count.
__global__ void k_objective32(MixedArgs a, const LandRec *__restrict__ land, double tx, double ty, double tz,
                              double inv_2s2, double *__restrict__ gr, double *__restrict__ sums) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    double g = 0.0, cnt = 0.0;
    if (i < a.n) {
        gr[3 * i] = gr[3 * i + 1] = gr[3 * i + 2] = 0.0;
        if ((a.p.idf[i] & kSettled) && land[i].step >= 0) {
            const int t = a.p.tet[i];
            const double dx = (a.cen[3 * t] + double(a.p.x[i])) - tx;
            const double dy = (a.cen[3 * t + 1] + double(a.p.y[i])) - ty;
            const double dz = (a.cen[3 * t + 2] + double(a.p.z[i])) - tz;
            g = exp(-(dx * dx + dy * dy + dz * dz) * inv_2s2);
            const double f = -2.0 * inv_2s2 * g;
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

__global__ void __launch_bounds__(128) k_backward32(MixedArgs a, AdjHist h, int k0, int k1,
                                                    const LandRec *__restrict__ land, const double *__restrict__ gr,
                                                    double gscale, double *__restrict__ ax, double *__restrict__ av,
                                                    double *__restrict__ gE, StepConst c, double cq,
                                                    const double *__restrict__ G) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int64_t n = a.n;
    const LandRec L = land[i];
    const int N = L.step < 0 ? -1 : int(int64_t(L.step) - c.step);
    if (N < k0) return;
    const uint32_t id = a.p.idf[i] & kIdMask;
    double Ax = ax[3 * i], Ay = ax[3 * i + 1], Az = ax[3 * i + 2];
    double Vx = av[3 * i], Vy = av[3 * i + 1], Vz = av[3 * i + 2];
    const float vmin = c.vmin_f;
    const double mcp = double(c.mass_cp_f), mct = double(c.mass_ct_f);
    int run = -1;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int k = min(k1 - 1, N); k >= k0; --k) {
        const int64_t o = int64_t(k - k0) * n + i;
        const int t = h.tet[o];
        if (t < 0) continue;
        float vx = float(h.vx[o]), vy = float(h.vy[o]), vz = float(h.vz[o]);
        if (fmaf(vz, vz, fmaf(vy, vy, vx * vx)) < vmin * vmin) continue;  // the step did not move it
        const TetRec32 &R = a.rec[t];
        if (!(R.ezero & kRecEzero)) {
            vx = (vx + R.H[0]) + R.H[0];
            vy = (vy + R.H[1]) + R.H[1];
            vz = (vz + R.H[2]) + R.H[2];
        }
        const double wx = vx, wy = vy, wz = vz;  // pushed velocity, as the forward had it
        double bx, by, bz;
        if (k == N) {
            const double *M = a.rec64[L.tet].M;  // exit-face normal from the FP64 map
            double nn[3];
            for (int q = 0; q < 3; ++q)
                nn[q] = L.face == 0 ? -(M[q] + M[3 + q] + M[6 + q]) : M[3 * (L.face - 1) + q];
            const double gx = gr[3 * i] * gscale, gy = gr[3 * i + 1] * gscale, gz = gr[3 * i + 2] * gscale;
            const double nv = nn[0] * wx + nn[1] * wy + nn[2] * wz;
            const double vg = (wx * gx + wy * gy + wz * gz) / nv;
            Ax = gx - nn[0] * vg;
            Ay = gy - nn[1] * vg;
            Az = gz - nn[2] * vg;
            const double sdt = L.s * c.dt;
            bx = sdt * Ax;
            by = sdt * Ay;
            bz = sdt * Az;
        } else {
            float xc, xs, cp, sp;
            const uint64_t sk = uint64_t(c.step + k);
            if (c.model != SPG_COLL_NONE &&
                collision_event32(c, id, sk, is_candidate(c, id, sk), speed2(vx, vy, vz), xc, xs, cp, sp)) {
                // v' = m_cp v + m_ct |v| n:  J^T a = m_cp a + m_ct v/|v| (n . a)
                const double vm = sqrt(wx * wx + wy * wy + wz * wz);
                const double na = (double(xs * cp) * Vx + double(xs * sp) * Vy + double(xc) * Vz) * mct / vm;
                Vx = mcp * Vx + na * wx;
                Vy = mcp * Vy + na * wy;
                Vz = mcp * Vz + na * wz;
            }
            bx = Vx + c.dt * Ax;
            by = Vy + c.dt * Ay;
            bz = Vz + c.dt * Az;
        }
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
        if (G && !(R.ezero & kRecEzero)) {
            // the pushed velocity's dependence on the position through the
            // recovered field: abar_x += cq G^T abar_va
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

__global__ void k_gather_adj32(DevParticles32 p, int64_t n, const double *__restrict__ ax,
                               const double *__restrict__ av, double *dx, double *dv) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t id = p.idf[i] & kIdMask;
    for (int k = 0; k < 3; ++k) {
        if (dx) dx[3 * id + k] = ax[3 * i + k];
        if (dv) dv[3 * id + k] = av[3 * i + k];
    }
}

MixedArgs make_args(const DevParticles32 &p, int64_t n, const MeshDev32 &m) {
    MixedArgs a;
    a.p = p;
    a.n = n;
    a.rec = m.rec;
    a.rec64 = m.rec64;
    a.cen = m.cen;
    a.cen_lo = m.cen_lo;
    a.nbr = m.nbr;
    a.ftri = m.ftri;
    a.tet_nodes = m.tet_nodes;
    a.n_tets = m.n_tets;
    return a;
}

}  // namespace

void launch_step32(const DevParticles32 &p, int64_t n, const MeshDev32 &m, const StepConst &c,
                   unsigned int *tri_count, void *wq, unsigned int *wq_n, DevCounters *ctr, const FieldArgs &f,
                   cudaStream_t s, LandRec *land) {
    if (n <= 0) return;
    const MixedArgs a = make_args(p, n, m);
    cudaMemsetAsync(wq_n, 0, sizeof(unsigned int), s);
    static int step32_blocks = 0;  // SMs x resident blocks of k_step32 (same on every device of this build)
    if (!step32_blocks) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step32, 256, 0);
        step32_blocks = std::max(1, sms * std::max(1, per_sm));
    }
    const unsigned grid = unsigned(std::min<int64_t>(grid_for(n, 256), step32_blocks));
    k_step32<<<grid, 256, 0, s>>>(a, c, static_cast<WalkItem32 *>(wq), wq_n, ctr);
    k_walk_queue32<<<152 * 8, 128, 0, s>>>(a, c.max_cross, static_cast<WalkItem32 *>(wq), wq_n, tri_count, ctr,
                                            land, c.step, f);
}

int launch_segment32(const DevParticles32 &p, int64_t n, const MeshDev32 &m, const StepConst &c, int L,
                     unsigned int *tri_count, void *wq, int2 *rq, unsigned int *q_n, DevCounters *ctr,
                     const FieldArgs &f, cudaStream_t s) {
    if (n <= 0 || L <= 0 || L > kMaxSegment) return 0;
    const MixedArgs a = make_args(p, n, m);
    SegQueues sq;
    sq.wq = static_cast<SegItem32 *>(wq);
    sq.rq = rq;
    sq.wq_n = q_n;
    sq.rq_n = q_n + L + 1;
    sq.L = L;
    cudaMemsetAsync(q_n, 0, sizeof(unsigned int) * size_t(2 * L + 1), s);
    // one wave of each kernel: SMs x resident blocks (same on every device of this build)
    static int seg_blocks = 0, walk_blocks = 0, resume_blocks = 0;
    if (!seg_blocks) {
        int dev = 0, sms = 0, b0 = 0, b1 = 0, b2 = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b0, k_seg32, 256, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b1, k_seg_walk32, 128, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b2, k_seg_resume32, 256, 0);
        walk_blocks = std::max(1, sms * std::max(1, b1));
        resume_blocks = std::max(1, sms * std::max(1, b2));
        seg_blocks = std::max(1, sms * std::max(1, b0));
    }
    const unsigned grid = unsigned(std::min<int64_t>(grid_for(n, 256), seg_blocks));
    k_seg32<<<grid, 256, 0, s>>>(a, c, sq, ctr);
    int launches = 1;
    for (int r = 0; r < L; ++r) {
        launch_pdl(k_seg_walk32, walk_blocks, 128, s, a, c.max_cross, sq, r, tri_count, ctr, f);
        ++launches;
        if (r + 1 < L) {
            launch_pdl(k_seg_resume32, resume_blocks, 256, s, a, c, sq, r, ctr);
            ++launches;
        }
    }
    return launches;
}

void launch_deposit32(const DevParticles32 &p, int64_t n, const MeshDev32 &m, int k, unsigned long long *node_fix,
                      const OccList &occ, cudaStream_t s) {
    if (n <= 0) return;
    static int blocks = 0;  // one wave
    if (blocks == 0) blocks = resident_blocks(k_deposit32, kDepThreads);
    const DepSrc32 src{p, m.rec, k, 1LL << k};
    const unsigned grid = unsigned(std::min<int64_t>(grid_for(n, kDepThreads), blocks));
    k_deposit32<<<grid, kDepThreads, 0, s>>>(src, n, m.tet_nodes, node_fix, occ);
}

void launch_record32(const DevParticles32 &p, int64_t n, const AdjHist &h, int k, cudaStream_t s) {
    if (n > 0) k_record32<<<grid_for(n, 256), 256, 0, s>>>(p, n, h, k);
}

void launch_objective32(const DevParticles32 &p, int64_t n, const MeshDev32 &m, const LandRec *land,
                        const double *target, double sigma, double *gr, double *sums, cudaStream_t s) {
    if (n > 0)
        k_objective32<<<grid_for(n, 256), 256, 0, s>>>(make_args(p, n, m), land, target[0], target[1], target[2],
                                                        1.0 / (2.0 * sigma * sigma), gr, sums);
}

void launch_backward32(const DevParticles32 &p, int64_t n, const MeshDev32 &m, const AdjHist &h, int k0, int k1,
                       const LandRec *land, const double *gr, double gscale, double *ax, double *av, double *gE,
                       const StepConst &c, cudaStream_t s, const double *G) {
    if (n > 0)
        k_backward32<<<grid_for(n, 128), 128, 0, s>>>(make_args(p, n, m), h, k0, k1, land, gr, gscale, ax, av, gE, c,
                                                       c.charge / c.mass * c.dt, G);
}

void launch_gather_adj32(const DevParticles32 &p, int64_t n, const double *ax, const double *av, double *dx,
                         double *dv, cudaStream_t s) {
    if (n > 0) k_gather_adj32<<<grid_for(n, 256), 256, 0, s>>>(p, n, ax, av, dx, dv);
}

void launch_field32_full(const FieldArgs &f, int64_t n_tets, cudaStream_t s) {
    if (n_tets > 0) k_field32_full<<<grid_for(n_tets, 256), 256, 0, s>>>(f, n_tets);
}

void launch_field32_list(const FieldArgs &f, const int32_t *list, const unsigned int *list_n, cudaStream_t s) {
    k_field32_list<<<152 * 4, 256, 0, s>>>(f, list, list_n);
}

void launch_refresh32(const DevParticles32 &p, int64_t n, const FieldArgs &f, cudaStream_t s) {
    if (n > 0) k_refresh32<<<grid_for(n, 256), 256, 0, s>>>(p, n, f);
}

void launch_to_local(const double *pos, const double *vel, const int32_t *tet, const double *cen, int64_t n,
                     DevParticles32 p, cudaStream_t s, int64_t id_base) {
    if (n <= 0) return;
    k_to_local<<<grid_for(n, 256), 256, 0, s>>>(pos, vel, tet, cen, n, p, id_base);
}

void launch_gather32(const DevParticles32 &p, int64_t n, int32_t *slot, const double *cen, double *pos, double *vel,
                     int32_t *tet, uint32_t *flags, cudaStream_t s) {
    if (n <= 0) return;
    launch_slot_of_id(p.idf, n, slot, s);
    k_gather32<<<grid_for(n, 256), 256, 0, s>>>(p, n, slot, cen, pos, vel, tet, flags);
}

void launch_resort32(const DevParticles32 &src, DevParticles32 dst, int64_t n, int64_t n_tets, int32_t *scratch,
                     int64_t *n_alive_dev, cudaStream_t s) {
    launch_sort_prepare(src.tet, src.idf, n, n_tets, scratch, n_alive_dev, s);
    if (n > 0)
        k_sort_scatter32<<<grid_for(n, kSortBlock), kSortBlock, 0, s>>>(src, dst, n, int(n_tets),
                                                                        sort_offsets(scratch));
}

size_t walk_item32_bytes() { return sizeof(WalkItem32); }

}  // namespace spg
