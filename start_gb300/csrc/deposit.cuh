// Block-level reduction of P1 charge contributions and the atomic flush into
// the fixed-point node accumulators, shared by the FP64 and the mixed-form
// deposit kernels.
//
// Each thread holds one particle's fixed-point weights v[1..3] (v[0] = one -
// v[1] - v[2] - v[3], one = 2^k) and its tet (key, -1 for none). The lanes
// of a warp with equal keys (match_any: contiguous runs of the tet-sorted
// order, and lanes of a tet that drifted apart since the last re-sort) are
// summed by the integer reduce unit; the lowest lane of each group adds the
// four node sums into a per-block hash table of nodes in shared memory, and
// the table is flushed with one global atomic per distinct node. Integer sums
// do not depend on order, so the result is the same as one atomic per
// particle.
#ifndef SPG_DEPOSIT_CUH
#define SPG_DEPOSIT_CUH

#include <cstdint>

#include "spg_internal.h"

namespace spg {

template <int NT>
__device__ __forceinline__ void deposit_block_flush(int key, const long long v[4], long long one,
                                                    const int4 *__restrict__ tet_nodes,
                                                    unsigned long long *__restrict__ node_fix, const OccList &occ) {
    constexpr unsigned kAll = 0xffffffffu;
    constexpr int HS = 2 * NT;  // hash slots: node -> block sum
    __shared__ int s_node[HS];
    __shared__ unsigned long long s_sum[HS];
    for (int k = threadIdx.x; k < HS; k += NT) {
        s_node[k] = -1;
        s_sum[k] = 0ull;
    }
    const int lane = threadIdx.x & 31;
    const unsigned grp = __match_any_sync(kAll, key);
    // Group sums of v[1..3]: each value is split into 21-bit pieces whose sums
    // over at most 32 lanes fit 32 bits (a weight is at most 2^52 in
    // magnitude, so the signed top piece v >> 42 is at most 2^10). When every
    // weight of the warp is below 2^41 in magnitude (one <= 2^41, more than
    // 2e6 particles, and barycentrics in about [-1, 1]) two pieces do: the
    // signed v >> 21 is below 2^20.
    bool big = false;
#pragma unroll
    for (int q = 1; q < 4; ++q) {
        const long long t = v[q] >> 41;
        big = big || (t != 0 && t != -1);
    }
    long long sum[4];
    if (!__any_sync(kAll, big)) {
#pragma unroll
        for (int q = 1; q < 4; ++q) {
            const unsigned b0 = unsigned(v[q] & 0x1FFFFF);
            const int b1 = int(v[q] >> 21);
            const unsigned s0 = __reduce_add_sync(grp, b0);
            const int s1 = __reduce_add_sync(grp, b1);
            sum[q] = (long long)s0 + (long long)s1 * (1LL << 21);
        }
    } else {
#pragma unroll
        for (int q = 1; q < 4; ++q) {
            const unsigned b0 = unsigned(v[q] & 0x1FFFFF), b1 = unsigned((v[q] >> 21) & 0x1FFFFF);
            const int b2 = int(v[q] >> 42);
            const unsigned s0 = __reduce_add_sync(grp, b0), s1 = __reduce_add_sync(grp, b1);
            const int s2 = __reduce_add_sync(grp, b2);
            sum[q] = (long long)s0 + (long long)s1 * (1LL << 21) + (long long)s2 * (1LL << 42);
        }
    }
    sum[0] = (long long)__popc(grp) * one - sum[1] - sum[2] - sum[3];
    __syncthreads();  // the table is cleared
    // The lowest lane of each group adds its four node sums to the block's
    // table (open addressing, linear probing); a full table falls back to a
    // global atomic.
    if (key >= 0 && lane == __ffs(grp) - 1) {
        if (occ.list && __ldcg(occ.gen_of + key) != occ.gen && atomicExch(occ.gen_of + key, occ.gen) != occ.gen)
            occ.list[atomicAdd(occ.n, 1u)] = key;
        const int4 tn = __ldg(tet_nodes + key);
        const int nodes[4] = {tn.x, tn.y, tn.z, tn.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int node = nodes[q];
            int h = int((unsigned(node) * 2654435761u) >> 8) & (HS - 1);
            bool placed = false;
            for (int probe = 0; probe < HS; ++probe) {
                const int old = atomicCAS(&s_node[h], -1, node);
                if (old == -1 || old == node) {
                    atomicAdd(&s_sum[h], (unsigned long long)sum[q]);
                    placed = true;
                    break;
                }
                h = (h + 1) & (HS - 1);
            }
            if (!placed) atomicAdd(node_fix + node, (unsigned long long)sum[q]);
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < HS; k += NT) {
        const int node = s_node[k];
        if (node >= 0) atomicAdd(node_fix + node, s_sum[k]);
    }
}

}  // namespace spg

#endif
