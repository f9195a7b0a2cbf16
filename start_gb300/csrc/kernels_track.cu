// Trajectory sampling of a fixed set of particles (spg_track_particles), the
// GPU counterpart of ParticleMovementTracker::recordMovement
// (src/ParticleInCellEngine/ParticleDynamicsProcessor/ParticleMovementTracker.cpp:4-16):
// before each step the position of every tracked particle that is still
// alive is appended to its row of a device buffer. Re-sorts move particles
// between slots, so the slot of each tracked id is looked up again after
// every re-sort through an id -> track table.
#include "spg_internal.h"

namespace spg {

namespace {

__global__ void k_track_map(const int64_t *__restrict__ ids, int k, int32_t *__restrict__ track_of_id) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < k) track_of_id[ids[t]] = t;
}

__global__ void k_track_find(const uint32_t *__restrict__ idf, int64_t n, const int32_t *__restrict__ track_of_id,
                             int64_t table_n, int32_t *__restrict__ slot) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t id = idf[i] & kIdMask;
    if (int64_t(id) >= table_n) return;  // injected after the tracking began
    const int32_t t = track_of_id[id];
    if (t >= 0) slot[t] = int32_t(i);
}

// FP64 state: global positions. FP32 state (cen != nullptr): centroid of the
// owning tet + local position.
template <class T>
__global__ void k_track_record(const T *__restrict__ x, const T *__restrict__ y, const T *__restrict__ z,
                               const int32_t *__restrict__ tet, const uint32_t *__restrict__ idf,
                               const double *__restrict__ cen, const int32_t *__restrict__ slot, int k, int cap,
                               int32_t *__restrict__ count, double *__restrict__ xyz) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= k) return;
    const int32_t i = slot[t];
    if (i < 0 || (idf[i] & kDead)) return;
    const int c = count[t];
    if (c >= cap) return;
    double px = double(x[i]), py = double(y[i]), pz = double(z[i]);
    if (cen) {
        const int32_t tt = tet[i];
        px += cen[3 * tt];
        py += cen[3 * tt + 1];
        pz += cen[3 * tt + 2];
    }
    double *o = xyz + 3 * (int64_t(t) * cap + c);
    o[0] = px;
    o[1] = py;
    o[2] = pz;
    count[t] = c + 1;
}

// Current position and flags of each tracked particle (the settle point of a
// settled one, which the reference's surface handler appends to its track).
template <class T>
__global__ void k_track_current(const T *__restrict__ x, const T *__restrict__ y, const T *__restrict__ z,
                                const int32_t *__restrict__ tet, const uint32_t *__restrict__ idf,
                                const double *__restrict__ cen, const int32_t *__restrict__ slot, int k,
                                double *__restrict__ xyz, uint32_t *__restrict__ flags) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= k) return;
    const int32_t i = slot[t];
    if (i < 0) {
        flags[t] = 0;
        return;
    }
    double px = double(x[i]), py = double(y[i]), pz = double(z[i]);
    if (cen) {
        const int32_t tt = tet[i];
        px += cen[3 * tt];
        py += cen[3 * tt + 1];
        pz += cen[3 * tt + 2];
    }
    xyz[3 * t] = px;
    xyz[3 * t + 1] = py;
    xyz[3 * t + 2] = pz;
    const uint32_t f = idf[i];
    flags[t] = ((f & kSettled) ? SPG_FLAG_SETTLED : 0u) | ((f & kLost) ? SPG_FLAG_LOST : 0u);
}

}  // namespace

void launch_track_current64(const DevParticles &p, const int32_t *slot, int k, double *xyz, uint32_t *flags,
                            cudaStream_t s) {
    if (k > 0)
        k_track_current<double><<<(k + 127) / 128, 128, 0, s>>>(p.x, p.y, p.z, p.tet, p.idf, nullptr, slot, k, xyz,
                                                                flags);
}

void launch_track_current32(const DevParticles32 &p, const double *cen, const int32_t *slot, int k, double *xyz,
                            uint32_t *flags, cudaStream_t s) {
    if (k > 0)
        k_track_current<float><<<(k + 127) / 128, 128, 0, s>>>(p.x, p.y, p.z, p.tet, p.idf, cen, slot, k, xyz, flags);
}

void launch_track_map(const int64_t *ids, int k, int32_t *track_of_id, cudaStream_t s) {
    if (k > 0) k_track_map<<<(k + 127) / 128, 128, 0, s>>>(ids, k, track_of_id);
}

void launch_track_find(const uint32_t *idf, int64_t n, const int32_t *track_of_id, int64_t table_n, int32_t *slot,
                       cudaStream_t s) {
    if (n > 0) k_track_find<<<unsigned((n + 255) / 256), 256, 0, s>>>(idf, n, track_of_id, table_n, slot);
}

void launch_track_record64(const DevParticles &p, const int32_t *slot, int k, int cap, int32_t *count, double *xyz,
                           cudaStream_t s) {
    if (k > 0)
        k_track_record<double><<<(k + 127) / 128, 128, 0, s>>>(p.x, p.y, p.z, p.tet, p.idf, nullptr, slot, k, cap,
                                                               count, xyz);
}

void launch_track_record32(const DevParticles32 &p, const double *cen, const int32_t *slot, int k, int cap,
                           int32_t *count, double *xyz, cudaStream_t s) {
    if (k > 0)
        k_track_record<float><<<(k + 127) / 128, 128, 0, s>>>(p.x, p.y, p.z, p.tet, p.idf, cen, slot, k, cap, count,
                                                              xyz);
}

}  // namespace spg
