// Block-level reduction of tet-sorted P1 charge contributions and the atomic
// flush into the fixed-point node accumulators, shared by the FP64 and the
// mixed-form deposit kernels.
//
// Each thread holds one particle's four fixed-point weights v[0..3] and its
// tet (key, -1 for none). Consecutive threads hold consecutive particles of
// the tet-sorted order, so equal keys form runs. A segmented shuffle scan
// sums each run within a warp; thread 0 then chains the runs that cross warp
// boundaries (a run can span several warps when a tet holds hundreds of
// particles), and only the last lane of each run of the block adds the four
// sums to the nodes. Integer sums do not depend on order, so the result is
// the same as one atomic per particle; there are just far fewer atomics on
// the few nodes of densely occupied tets.
#ifndef SPG_DEPOSIT_CUH
#define SPG_DEPOSIT_CUH

#include <cstdint>

namespace spg {

template <int NT>
__device__ __forceinline__ void deposit_block_flush(int key, long long v[4], const int4 *__restrict__ tet_nodes,
                                                    unsigned long long *__restrict__ node_fix) {
    constexpr unsigned kAll = 0xffffffffu;
    constexpr int NW = NT / 32;
    __shared__ int s_kf[NW], s_kl[NW], s_whole[NW];
    __shared__ long long s_sl[NW][4], s_carry[NW][4];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int prev = __shfl_up_sync(kAll, key, 1);
    const bool head = lane == 0 || prev != key;
    const unsigned heads = __ballot_sync(kAll, head);
    if (heads != 1u) {
        const int start = 31 - __clz(heads & (kAll >> (31 - lane)));
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const long long up = __shfl_up_sync(kAll, v[q], off);
                if (lane - off >= start) v[q] += up;
            }
        }
    } else {
        // One run covers the warp (the common case: hundreds of particles per
        // occupied tet); only its total is used (at lane 31). It goes through
        // the integer reduce unit instead of 64-bit shuffles: each value is
        // split into 21-bit pieces whose 32-lane sums cannot overflow 32 bits
        // (a particle's weights are at most 2^52 in magnitude, so the top
        // piece v >> 42 is at most 2^10).
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const unsigned b0 = unsigned(v[q] & 0x1FFFFF), b1 = unsigned((v[q] >> 21) & 0x1FFFFF);
            const int b2 = int(v[q] >> 42);
            const unsigned s0 = __reduce_add_sync(kAll, b0), s1 = __reduce_add_sync(kAll, b1);
            const int s2 = __reduce_add_sync(kAll, b2);
            v[q] = (long long)s0 + (long long)s1 * (1LL << 21) + (long long)s2 * (1LL << 42);
        }
    }
    if (lane == 0) s_kf[w] = key;
    if (lane == 31) {
        s_kl[w] = key;
        s_whole[w] = heads == 1u;
#pragma unroll
        for (int q = 0; q < 4; ++q) s_sl[w][q] = v[q];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) s_carry[0][q] = 0;
        for (int u = 1; u < NW; ++u) {
            const bool cont = s_kf[u] >= 0 && s_kl[u - 1] == s_kf[u];
#pragma unroll
            for (int q = 0; q < 4; ++q)
                s_carry[u][q] = cont ? s_sl[u - 1][q] + (s_whole[u - 1] ? s_carry[u - 1][q] : 0) : 0;
        }
    }
    __syncthreads();
    const bool tail = lane == 31 || ((heads >> (lane + 1)) & 1u);
    if (!tail || key < 0) return;
    if (lane == 31 && w + 1 < NW && s_kf[w + 1] == key) return;  // the run goes on in the next warp
    const bool first_run = (heads & (kAll >> (31 - lane))) == 1u;
    long long t[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) t[q] = v[q] + (first_run ? s_carry[w][q] : 0);
    const int4 tn = __ldg(tet_nodes + key);
    atomicAdd(node_fix + tn.x, (unsigned long long)t[0]);
    atomicAdd(node_fix + tn.y, (unsigned long long)t[1]);
    atomicAdd(node_fix + tn.z, (unsigned long long)t[2]);
    atomicAdd(node_fix + tn.w, (unsigned long long)t[3]);
}

}  // namespace spg

#endif
