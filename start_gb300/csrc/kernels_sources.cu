// Particle sources sampled on the device (spg_generate_particles). The
// sampling laws are those of the host sources (start_gb300/sources.py):
//   disk:   r = R sqrt(u0), psi = 2 pi u1 in the plane of the normal;
//   rect:   x, y uniform over the rectangle at z;
//   cone:   cos(theta) = 1 - u2 (1 - cos(half_angle)), phi = 2 pi u3;
//   cosine: sin(theta) = sqrt(u2), phi = 2 pi u3 (Lambert law);
//   Thompson: E = U s / (1 - s), s = sqrt(u4) Emax / (Emax + U);
// and the reference's own sources (ParticleGeneratorHost.cpp:33-160):
//   point:  every particle at the centre;
//   cells:  particle i at the centre of its cell (counts split evenly, the
//           remainder one each to seed-chosen cells, decided on the host);
//   fan:    theta = theta0 + (2 u2 - 1) expansion, phi = phi0, about the normal
//           (theta0, phi0) of the source or of the particle's cell;
// then the ParticleDisplacer shift: for the fan law one vector per point
// source or per cell, along the source's direction or the cell's normal
// (ParticleDisplacer.cpp:48-133); for the cone and cosine laws
// p += d / max|d_k| * displacement along the particle's own direction.
// Particle i takes its uniforms from Philox4x32-10 keyed by the seed and
// counted by (its id, block, tag), one thread per particle.
#include <cmath>

#include "philox.h"
#include "spg_internal.h"

namespace spg {

namespace {

constexpr uint32_t kSourceTag = 0x534f5552u;  // counter word that separates these streams from others
constexpr double kTwoPi = 6.283185307179586476925286766559;

__device__ __forceinline__ Philox4 source_draw(int64_t i, uint32_t block, const SourceConst &c) {
    Philox4 ctr;
    ctr.v[0] = uint32_t(i);
    ctr.v[1] = uint32_t(uint64_t(i) >> 32);
    ctr.v[2] = block;
    ctr.v[3] = kSourceTag;
    return philox4x32_10(ctr, c.seed_lo, c.seed_hi);
}

__global__ void k_generate(const __grid_constant__ SourceConst c, int64_t n, double *__restrict__ pos,
                           double *__restrict__ vel) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t id = c.id_base + i;
    const Philox4 r0 = source_draw(id, 0, c), r1 = source_draw(id, 1, c);
    const double u0 = u01_from(r0.v[0], r0.v[1]), u1 = u01_from(r0.v[2], r0.v[3]);
    const double u2 = u01_from(r1.v[0], r1.v[1]), u3 = u01_from(r1.v[2], r1.v[3]);
    double p[3];
    double theta0 = c.theta0, phi0 = c.phi0;
    const double *fan = c.fan_shift;
    if (c.shape == SPG_SRC_CELLS) {
        int lo = 0, hi = c.n_cells - 1;  // the cell with cell_first[k] <= i < cell_first[k + 1]
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (c.cell_first[mid] <= i)
                lo = mid;
            else
                hi = mid - 1;
        }
        const double *cc = c.cells + 8 * lo;
        p[0] = cc[0];
        p[1] = cc[1];
        p[2] = cc[2];
        theta0 = cc[3];
        phi0 = cc[4];
        fan = cc + 5;
    } else if (c.shape == SPG_SRC_POINT) {
        p[0] = c.centre[0];
        p[1] = c.centre[1];
        p[2] = c.centre[2];
    } else if (c.shape == SPG_SRC_DISK) {
        const double r = c.radius * sqrt(u0), ps = kTwoPi * u1;
        double sp, cp;
        sincos(ps, &sp, &cp);
        for (int k = 0; k < 3; ++k) p[k] = c.centre[k] + (r * cp) * c.e1[k] + (r * sp) * c.e2[k];
    } else {
        p[0] = c.xlim[0] + (c.xlim[1] - c.xlim[0]) * u0;
        p[1] = c.ylim[0] + (c.ylim[1] - c.ylim[0]) * u1;
        p[2] = c.z;
    }
    double d[3];
    if (c.directions == SPG_DIR_FAN) {
        const double th = theta0 + (2.0 * u2 - 1.0) * c.expansion;
        double sth, cth, sph, cph;
        sincos(th, &sth, &cth);
        sincos(phi0, &sph, &cph);
        d[0] = sth * cph;
        d[1] = sth * sph;
        d[2] = cth;
    } else {
        double ct, st;
        if (c.directions == SPG_DIR_CONE) {
            ct = 1.0 - u2 * c.one_minus_cos;
            st = sqrt(fmax(0.0, 1.0 - ct * ct));
        } else {
            st = sqrt(u2);
            ct = sqrt(fmax(0.0, 1.0 - st * st));
        }
        double sph, cph;
        sincos(kTwoPi * u3, &sph, &cph);
        for (int k = 0; k < 3; ++k) d[k] = (st * cph) * c.e1[k] + (st * sph) * c.e2[k] + ct * c.nrm[k];
    }
    double speed = c.speed_mono;
    if (c.energy == SPG_ENERGY_THOMPSON) {
        const Philox4 r2 = source_draw(id, 2, c);
        const double s = sqrt(u01_from(r2.v[0], r2.v[1])) * c.s_max;
        const double E = c.binding_j * s / (1.0 - s);
        speed = sqrt(2.0 * E / c.mass);
    }
    if (c.directions == SPG_DIR_FAN) {
        for (int k = 0; k < 3; ++k) {
            pos[3 * i + k] = p[k] + fan[k];
            vel[3 * i + k] = d[k] * speed;
        }
    } else {
        const double m = fmax(fabs(d[0]), fmax(fabs(d[1]), fabs(d[2])));
        const double shift = m > 2.220446049250313e-16 ? c.displacement / m : 0.0;
        for (int k = 0; k < 3; ++k) {
            pos[3 * i + k] = p[k] + d[k] * shift;
            vel[3 * i + k] = d[k] * speed;
        }
    }
}

}  // namespace

void launch_generate(const SourceConst &c, int64_t n, double *pos, double *vel, cudaStream_t s) {
    if (n > 0) k_generate<<<unsigned((n + 255) / 256), 256, 0, s>>>(c, n, pos, vel);
}

}  // namespace spg
