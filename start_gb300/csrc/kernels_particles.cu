// Particle kernels of the FP64 form: fused push + move + gas collision +
// tet walk + surface settle, P1 deposit, per-tet E, point location, re-sort.
//
// Compiled with --fmad=false: every a*b+c stays a separate multiply and add,
// matching the CPU oracle (built with -ffp-contract=off) bit for bit on the
// collisionless path. Division and sqrt are IEEE (CUDA defaults for double).
#include <cmath>
#include <cstdio>

#include "philox.h"
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

__device__ __forceinline__ void load_geo(const TetRec *__restrict__ rec, int t, TetGeo &g, double E[3]) {
    const double2 *rp = reinterpret_cast<const double2 *>(rec + t);
    double2 a = __ldg(rp + 0), b = __ldg(rp + 1), c = __ldg(rp + 2), d = __ldg(rp + 3);
    double2 e = __ldg(rp + 4), f = __ldg(rp + 5);
    g.M[0] = a.x; g.M[1] = a.y; g.M[2] = b.x; g.M[3] = b.y; g.M[4] = c.x; g.M[5] = c.y;
    g.M[6] = d.x; g.M[7] = d.y; g.M[8] = e.x;
    g.x0[0] = e.y; g.x0[1] = f.x; g.x0[2] = f.y;
    if (E) {
        double2 h = __ldg(rp + 6), k = __ldg(rp + 7);
        E[0] = h.x; E[1] = h.y; E[2] = k.x;
    }
}

// Barycentric coordinates; same expression order as the oracle.
__device__ __forceinline__ void bary(const TetGeo &g, double px, double py, double pz, double l[4]) {
    const double d0 = px - g.x0[0], d1 = py - g.x0[1], d2 = pz - g.x0[2];
    l[1] = g.M[0] * d0 + g.M[1] * d1 + g.M[2] * d2;
    l[2] = g.M[3] * d0 + g.M[4] * d1 + g.M[5] * d2;
    l[3] = g.M[6] * d0 + g.M[7] * d1 + g.M[8] * d2;
    l[0] = 1.0 - l[1] - l[2] - l[3];
}

__device__ __forceinline__ int comp(const int4 &v, int f) {
    return f == 0 ? v.x : (f == 1 ? v.y : (f == 2 ? v.z : v.w));
}

struct WalkOut {
    int tet, status, tri, crossings;
    double s;
};

// Straight walk of the segment p0 -> p1 starting in tet t (geometry g).
// In each tet: if p1 is inside (all lambda >= 0) stop. Otherwise leave through
// the face, other than the entry face, with lambda(p1) < 0 whose crossing
// parameter s = l0/(l0 - l1) along the segment is smallest (lowest local face
// index on ties). A face carrying a surface triangle stops the walk there
// (when stop_surface); a boundary face without one is an exit.
__device__ WalkOut walk64(const MeshDev &m, int t, TetGeo g, double p0x, double p0y, double p0z, double p1x,
                          double p1y, double p1z, int max_cross, bool stop_surface) {
    WalkOut o;
    o.crossings = 0;
    o.tri = -1;
    o.s = 1.0;
    int enter = -1;
    for (;;) {
        double l1[4];
        bary(g, p1x, p1y, p1z, l1);
        if (l1[0] >= 0.0 && l1[1] >= 0.0 && l1[2] >= 0.0 && l1[3] >= 0.0) {
            o.tet = t;
            o.status = W_INSIDE;
            return o;
        }
        double l0[4];
        bary(g, p0x, p0y, p0z, l0);
        int best = -1;
        double sb = 0.0;
#pragma unroll
        for (int f = 0; f < 4; ++f) {
            if (f == enter || !(l1[f] < 0.0)) continue;
            const double s = l0[f] / (l0[f] - l1[f]);
            if (best < 0 || s < sb) {
                best = f;
                sb = s;
            }
        }
        if (best < 0) {
            o.tet = t;
            o.status = W_INSIDE;
            return o;
        }
        const int tri = comp(__ldg(m.ftri + t), best);
        if (stop_surface && tri >= 0) {
            o.tet = t;
            o.status = W_SURFACE;
            o.tri = tri;
            o.s = sb;
            return o;
        }
        const int nb = comp(__ldg(m.nbr + t), best);
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
        load_geo(m.rec, t, g, nullptr);
    }
}

// Gas collision of one particle: HSModel.cpp:6-42, VHSModel.cpp:6-52,
// VSSModel.cpp:6-54. Stationary target; v' = m_p/(m_p+m_t) v + |m_t/(m_p+m_t) v| n.
__device__ bool collide64(const StepConst &c, uint32_t id, double &vx, double &vy, double &vz) {
    const double vmod = sqrt(vx * vx + vy * vy + vz * vz);
    double sigma;
    if (c.model == SPG_COLL_HS) {
        sigma = c.sigma_hs;
    } else {
        const double base = c.two_kT / ((c.mr * vmod) * vmod);
        const double d2 = c.vhs_c1 * pow(base, c.expo);
        sigma = kPi * d2;
    }
    const double P = ((sigma * vmod) * c.gas_n) * c.dt;
    const Philox4 r = collision_draw(uint64_t(c.step), 0u, id, c.seed_lo, c.seed_hi);
    const double u0 = u01_from(r.v[0], r.v[1]);
    if (!(u0 < P)) return false;
    const double u1 = u01_from(r.v[2], r.v[3]);
    const Philox4 r2 = collision_draw(uint64_t(c.step), 1u, id, c.seed_lo, c.seed_hi);
    const double u2 = u01_from(r2.v[0], r2.v[1]);
    double xi_cos;
    if (c.model == SPG_COLL_HS)
        xi_cos = -1.0 + 2.0 * u1;
    else if (c.model == SPG_COLL_VHS)
        xi_cos = u1;
    else
        xi_cos = 2.0 * pow(u1, c.inv_alpha) - 1.0;
    const double xi_sin = sqrt(1.0 - xi_cos * xi_cos);
    const double phi = (2.0 * kPi) * u2;
    const double nx = xi_sin * cos(phi), ny = xi_sin * sin(phi), nz = xi_cos;
    const double cmx = vx * c.mass_cp, cmy = vy * c.mass_cp, cmz = vz * c.mass_cp;
    const double pvx = c.mass_ct * vx, pvy = c.mass_ct * vy, pvz = c.mass_ct * vz;
    const double mp = sqrt(pvx * pvx + pvy * pvy + pvz * pvz);
    double ex = nx * mp, ey = ny * mp, ez = nz * mp;
    if (c.model == SPG_COLL_VSS) {
        // GeometryVector::calcBetaGamma + rotation (GeometryVector.hpp:448-471, 66-90)
        const double beta = acos(pvz / mp), gamma = atan2(pvy, pvx);
        const double cb = cos(beta), sb = sin(beta);
        const double tx = cb * ex + sb * ez, tz = -sb * ex + cb * ez;
        ex = tx;
        ez = tz;
        const double cg = cos(gamma), sg = sin(gamma);
        const double ux = cg * ex - sg * ey, uy = sg * ex + cg * ey;
        ex = ux;
        ey = uy;
    }
    vx = ex + cmx;
    vy = ey + cmy;
    vz = ez + cmz;
    return true;
}

__device__ __forceinline__ unsigned long long warp_sum(unsigned v) { return __reduce_add_sync(kFull, v); }

// One particle step (ParticleDynamicsProcessor.cpp:161-200 order):
// settled? -> |v| < vmin? -> outside bbox? -> E push (Boris, B = 0) -> move ->
// gas collision -> surface crossing along the move segment.
__global__ void __launch_bounds__(256) k_step64(DevParticles p, int64_t n, MeshDev m, StepConst c,
                                                unsigned int *__restrict__ tri_count, DevCounters *ctr) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    unsigned processed = 0, coll = 0, cross = 0, settled = 0, lost = 0, capped = 0;
    if (i < n) {
        uint32_t idf = p.idf[i];
        if (!(idf & kDead)) {
            processed = 1;
            const int t = p.tet[i];
            double x = p.x[i], y = p.y[i], z = p.z[i];
            double vx = p.vx[i], vy = p.vy[i], vz = p.vz[i];
            const double vmod = sqrt(vx * vx + vy * vy + vz * vz);
            const bool inside_box = x >= c.lo[0] && x <= c.hi[0] && y >= c.lo[1] && y <= c.hi[1] &&
                                    z >= c.lo[2] && z <= c.hi[2];
            if (!(vmod < c.vmin) && inside_box) {
                TetGeo g;
                double E[3];
                load_geo(m.rec, t, g, E);
                if (!(E[0] == 0.0 && E[1] == 0.0 && E[2] == 0.0)) {
                    // Particle::electroMagneticPush (Particle.cpp:196-234) with B = 0:
                    // v- = v + a dt/2, rotation is the identity, v = v- + a dt/2.
                    const double ax = (c.charge * E[0]) / c.mass;
                    const double ay = (c.charge * E[1]) / c.mass;
                    const double az = (c.charge * E[2]) / c.mass;
                    const double hx = (ax * c.dt) / 2.0, hy = (ay * c.dt) / 2.0, hz = (az * c.dt) / 2.0;
                    vx = (vx + hx) + hx;
                    vy = (vy + hy) + hy;
                    vz = (vz + hz) + hz;
                }
                // Particle::updatePosition (Particle.cpp:157-165)
                const double nx = x + vx * c.dt, ny = y + vy * c.dt, nz = z + vz * c.dt;
                if (!(nx == x && ny == y && nz == z)) {
                    const uint32_t id = idf & kIdMask;
                    if (c.model != SPG_COLL_NONE) coll = collide64(c, id, vx, vy, vz) ? 1u : 0u;
                    if (!(isfinite(nx) && isfinite(ny) && isfinite(nz))) {
                        idf |= kLost;
                        lost = 1;
                        p.idf[i] = idf;
                    } else {
                        const WalkOut w = walk64(m, t, g, x, y, z, nx, ny, nz, c.max_cross, true);
                        cross = unsigned(w.crossings);
                        if (w.status == W_INSIDE) {
                            x = nx;
                            y = ny;
                            z = nz;
                        } else if (w.status == W_SURFACE) {
                            x = x + w.s * (nx - x);
                            y = y + w.s * (ny - y);
                            z = z + w.s * (nz - z);
                            atomicAdd(tri_count + w.tri, 1u);
                            idf |= kSettled;
                            settled = 1;
                            p.idf[i] = idf;
                        } else {
                            x = nx;
                            y = ny;
                            z = nz;
                            idf |= kLost;
                            lost = 1;
                            capped = w.status == W_CAP ? 1u : 0u;
                            p.idf[i] = idf;
                        }
                        if (w.tet != t) p.tet[i] = w.tet;
                        p.x[i] = x;
                        p.y[i] = y;
                        p.z[i] = z;
                    }
                }
                p.vx[i] = vx;
                p.vy[i] = vy;
                p.vz[i] = vz;
            }
        }
    }
    // Block-level counter reduction, one atomic per counter per block.
    __shared__ unsigned long long sh[8][6];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned long long a0 = warp_sum(processed), a1 = warp_sum(coll), a2 = warp_sum(cross);
    unsigned long long a3 = warp_sum(settled), a4 = warp_sum(lost), a5 = warp_sum(capped);
    if (lane == 0) {
        sh[wid][0] = a0; sh[wid][1] = a1; sh[wid][2] = a2;
        sh[wid][3] = a3; sh[wid][4] = a4; sh[wid][5] = a5;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        unsigned long long s = 0;
        const int nw = blockDim.x >> 5;
        for (int w = 0; w < nw; ++w) s += sh[w][threadIdx.x];
        if (s) {
            unsigned long long *dst = threadIdx.x == 0   ? &ctr->processed
                                      : threadIdx.x == 1 ? &ctr->collisions
                                      : threadIdx.x == 2 ? &ctr->crossings
                                      : threadIdx.x == 3 ? &ctr->settled
                                      : threadIdx.x == 4 ? &ctr->lost
                                                         : &ctr->capped;
            atomicAdd(dst, s);
        }
    }
}

// P1 deposit: node_q[n] += w q lambda_n(x_p) for every alive particle.
// Lanes of a warp hold consecutive (tet-sorted) particles; equal tets form
// runs, each run is summed with a segmented shuffle scan and its last lane
// issues the four atomics, so a warp inside one tet does 4 atomics, not 128.
__global__ void __launch_bounds__(256) k_deposit64(DevParticles p, int64_t n, MeshDev m, double wq,
                                                   double *__restrict__ node_q) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    int key = -1;
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    if (i < n && !(p.idf[i] & kDead)) {
        key = p.tet[i];
        TetGeo g;
        load_geo(m.rec, key, g, nullptr);
        double l[4];
        bary(g, p.x[i], p.y[i], p.z[i], l);
        v[0] = wq * l[0];
        v[1] = wq * l[1];
        v[2] = wq * l[2];
        v[3] = wq * l[3];
    }
    const int prev = __shfl_up_sync(kFull, key, 1);
    const bool head = lane == 0 || prev != key;
    const unsigned heads = __ballot_sync(kFull, head);
    const unsigned le = kFull >> (31 - lane);
    const int start = 31 - __clz(heads & le);
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const double up = __shfl_up_sync(kFull, v[k], off);
            if (lane - off >= start) v[k] += up;
        }
    }
    const bool tail = lane == 31 || ((heads >> (lane + 1)) & 1u);
    if (tail && key >= 0) {
        const int4 tn = __ldg(m.tet_nodes + key);
        atomicAdd(node_q + tn.x, v[0]);
        atomicAdd(node_q + tn.y, v[1]);
        atomicAdd(node_q + tn.z, v[2]);
        atomicAdd(node_q + tn.w, v[3]);
    }
}

// E per tet: E = -sum_i phi_i grad(lambda_i) = -sum_r (phi_{r+1} - phi_0) M_r.
// (VolumetricMesh::computeElectricFields, VolumetricMesh.cpp:382-411, with the
// sign and scale of E = -grad(phi).)
__global__ void k_efield64(MeshDev m, TetRec *__restrict__ rec, const double *__restrict__ phi) {
    const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= m.n_tets) return;
    const int4 tn = __ldg(m.tet_nodes + t);
    const double f0 = phi[tn.x], f1 = phi[tn.y], f2 = phi[tn.z], f3 = phi[tn.w];
    const double d1 = f1 - f0, d2 = f2 - f0, d3 = f3 - f0;
    TetRec &r = rec[t];
    double E[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) E[k] = -((d1 * r.M[k] + d2 * r.M[3 + k]) + d3 * r.M[6 + k]);
    r.E[0] = E[0];
    r.E[1] = E[1];
    r.E[2] = E[2];
}

// Point location: walk from the centroid of the voxel's seed tet to p.
__global__ void k_locate(const double *__restrict__ pos, int64_t n, MeshDev m, const int32_t *__restrict__ vox_seed,
                         double ox, double oy, double oz, double ix, double iy, double iz, int dx, int dy, int dz,
                         int max_cross, int32_t *__restrict__ tet_out) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double px = pos[3 * i], py = pos[3 * i + 1], pz = pos[3 * i + 2];
    if (!(isfinite(px) && isfinite(py) && isfinite(pz))) {
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
    TetGeo g;
    load_geo(m.rec, seed, g, nullptr);
    const WalkOut w = walk64(m, seed, g, c[0], c[1], c[2], px, py, pz, max_cross, false);
    tet_out[i] = w.status == W_INSIDE ? w.tet : -1;
}

__global__ void k_init_particles(const double *__restrict__ pos, const double *__restrict__ vel,
                                 const int32_t *__restrict__ tet, int64_t n, DevParticles p) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    p.x[i] = pos[3 * i];
    p.y[i] = pos[3 * i + 1];
    p.z[i] = pos[3 * i + 2];
    p.vx[i] = vel[3 * i];
    p.vy[i] = vel[3 * i + 1];
    p.vz[i] = vel[3 * i + 2];
    const int32_t t = tet[i];
    p.tet[i] = t;
    p.idf[i] = uint32_t(i) | (t < 0 ? kLost : 0u);
}

__global__ void k_gather_by_id(DevParticles p, int64_t n, double *pos, double *vel, int32_t *tet, uint32_t *flags) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t idf = p.idf[i];
    const int64_t id = idf & kIdMask;
    if (pos) {
        pos[3 * id] = p.x[i];
        pos[3 * id + 1] = p.y[i];
        pos[3 * id + 2] = p.z[i];
    }
    if (vel) {
        vel[3 * id] = p.vx[i];
        vel[3 * id + 1] = p.vy[i];
        vel[3 * id + 2] = p.vz[i];
    }
    if (tet) tet[id] = p.tet[i];
    if (flags) flags[id] = ((idf & kSettled) ? SPG_FLAG_SETTLED : 0u) | ((idf & kLost) ? SPG_FLAG_LOST : 0u);
}

// ------------------------------------------------------------------ re-sort
// Counting sort by tet (dead particles get key n_tets and go last).

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int sort_key(const DevParticles &p, int64_t i, int n_tets) {
    return (p.idf[i] & kDead) ? n_tets : p.tet[i];
}

__global__ void k_sort_hist(DevParticles p, int64_t n, int n_tets, int32_t *__restrict__ cnt) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int key = i < n ? sort_key(p, i, n_tets) : -1;
    const unsigned peers = __match_any_sync(kFull, key);
    const int lane = threadIdx.x & 31;
    if (key >= 0 && lane == __ffs(peers) - 1) atomicAdd(cnt + key, __popc(peers));
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
    // exclusive scan of per-thread runs across the block
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

__global__ void k_sort_scatter(DevParticles src, DevParticles dst, int64_t n, int n_tets, int32_t *__restrict__ offs) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int key = i < n ? sort_key(src, i, n_tets) : -1;
    const unsigned peers = __match_any_sync(kFull, key);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    int32_t base = 0;
    if (key >= 0 && lane == leader) base = atomicAdd(offs + key, __popc(peers));
    base = __shfl_sync(kFull, base, leader);
    if (key < 0) return;
    const int64_t j = base + __popc(peers & ((1u << lane) - 1u));
    dst.x[j] = src.x[i];
    dst.y[j] = src.y[i];
    dst.z[j] = src.z[i];
    dst.vx[j] = src.vx[i];
    dst.vy[j] = src.vy[i];
    dst.vz[j] = src.vz[i];
    dst.tet[j] = src.tet[i];
    dst.idf[j] = src.idf[i];
}

inline unsigned grid_for(int64_t n, int block) { return unsigned((n + block - 1) / block); }

}  // namespace

void launch_step64(const DevParticles &p, int64_t n, const MeshDev &m, const StepConst &c, unsigned int *tri_count,
                   DevCounters *ctr, cudaStream_t s) {
    if (n <= 0) return;
    k_step64<<<grid_for(n, 256), 256, 0, s>>>(p, n, m, c, tri_count, ctr);
}

void launch_deposit64(const DevParticles &p, int64_t n, const MeshDev &m, double wq, double *node_q,
                      cudaStream_t s) {
    if (n <= 0) return;
    k_deposit64<<<grid_for(n, 256), 256, 0, s>>>(p, n, m, wq, node_q);
}

void launch_efield64(const MeshDev &m, TetRec *rec, const double *phi, cudaStream_t s) {
    k_efield64<<<grid_for(m.n_tets, 256), 256, 0, s>>>(m, rec, phi);
}

void launch_locate(const double *pos, int64_t n, const MeshDev &m, const int32_t *vox_seed,
                   const double *oi, const int32_t *dims, int max_cross, int32_t *tet_out, cudaStream_t s) {
    if (n <= 0) return;
    k_locate<<<grid_for(n, 128), 128, 0, s>>>(pos, n, m, vox_seed, oi[0], oi[1], oi[2], oi[3], oi[4], oi[5],
                                               dims[0], dims[1], dims[2], max_cross, tet_out);
}

void launch_init_particles(const double *pos, const double *vel, const int32_t *tet, int64_t n, DevParticles p,
                           cudaStream_t s) {
    if (n <= 0) return;
    k_init_particles<<<grid_for(n, 256), 256, 0, s>>>(pos, vel, tet, n, p);
}

void launch_gather_by_id(const DevParticles &p, int64_t n, double *pos, double *vel, int32_t *tet, uint32_t *flags,
                         cudaStream_t s) {
    if (n <= 0) return;
    k_gather_by_id<<<grid_for(n, 256), 256, 0, s>>>(p, n, pos, vel, tet, flags);
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

void launch_resort(const DevParticles &src, DevParticles dst, int64_t n, int64_t n_tets, int32_t *scratch,
                   int64_t *n_alive_dev, cudaStream_t s) {
    const int64_t len = n_tets + 1;
    const int64_t nb = (len + kScanTile - 1) / kScanTile;
    unsigned long long *occupied = sort_occupied_counter(scratch);
    int32_t *cnt = scratch + 2;
    int32_t *sums = cnt + len;
    cudaMemsetAsync(cnt, 0, sizeof(int32_t) * len, s);
    cudaMemsetAsync(occupied, 0, sizeof(unsigned long long), s);
    if (n > 0) k_sort_hist<<<grid_for(n, 256), 256, 0, s>>>(src, n, int(n_tets), cnt);
    k_scan_tile<<<unsigned(nb), kScanThreads, 0, s>>>(cnt, len, int(n_tets), sums, occupied);
    k_scan_sums<<<1, 1024, 0, s>>>(sums, nb);
    k_scan_add<<<grid_for(len, 256), 256, 0, s>>>(cnt, len, sums, int(n_tets), n_alive_dev);
    if (n > 0) k_sort_scatter<<<grid_for(n, 256), 256, 0, s>>>(src, dst, n, int(n_tets), cnt);
}

}  // namespace spg

namespace spg {
namespace {
__global__ void k_zero_efield(TetRec *__restrict__ rec, int64_t n) {
    const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= n) return;
    rec[t].E[0] = 0.0;
    rec[t].E[1] = 0.0;
    rec[t].E[2] = 0.0;
}
__global__ void k_count_lost(const int32_t *__restrict__ tet, int64_t n, unsigned long long *out) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const unsigned v = (i < n && tet[i] < 0) ? 1u : 0u;
    const unsigned s = __reduce_add_sync(0xffffffffu, v);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(out, (unsigned long long)s);
}
}  // namespace

void launch_zero_efield(TetRec *rec, int64_t n_tets, cudaStream_t s) {
    k_zero_efield<<<unsigned((n_tets + 255) / 256), 256, 0, s>>>(rec, n_tets);
}

void launch_count_lost(const int32_t *tet, int64_t n, unsigned long long *out, cudaStream_t s) {
    if (n <= 0) return;
    k_count_lost<<<unsigned((n + 255) / 256), 256, 0, s>>>(tet, n, out);
}
}  // namespace spg
