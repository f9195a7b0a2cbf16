// Block-level reduction of tet-sorted P1 charge contributions and the atomic
// flush into the fixed-point node accumulators, shared by the FP64 and the
// mixed-form deposit kernels.
//
// Each thread holds one particle's four fixed-point weights v[0..3] and its
// tet (key, -1 for none). Consecutive threads hold consecutive particles of
// the tet-sorted order, so equal keys form runs. A segmented shuffle scan
// sums each run within a warp; the last lane of each run adds its four sums
// into a per-block hash table of nodes in shared memory, and the table is
// flushed with one global atomic per distinct node. Runs that cross warps,
// and runs of one tet broken up once particles have drifted since the last
// re-sort, merge in the table, so a block issues about as many global
// atomics as it touches nodes. Integer sums do not depend on order, so the
// result is the same as one atomic per particle.
#ifndef SPG_DEPOSIT_CUH
#define SPG_DEPOSIT_CUH

#include <cstdint>

namespace spg {

template <int NT>
__device__ __forceinline__ void deposit_block_flush(int key, long long v[4], const int4 *__restrict__ tet_nodes,
                                                    unsigned long long *__restrict__ node_fix) {
    constexpr unsigned kAll = 0xffffffffu;
    constexpr int HS = 2 * NT;  // hash slots: node -> block sum
    __shared__ int s_node[HS];
    __shared__ unsigned long long s_sum[HS];
    for (int k = threadIdx.x; k < HS; k += NT) {
        s_node[k] = -1;
        s_sum[k] = 0ull;
    }
    const int lane = threadIdx.x & 31;
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
    __syncthreads();  // the table is cleared
    // The last lane of each run adds its four node sums to the block's table
    // (open addressing, linear probing); a full table falls back to a global atomic.
    const bool tail = lane == 31 || ((heads >> (lane + 1)) & 1u);
    if (tail && key >= 0) {
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
                    atomicAdd(&s_sum[h], (unsigned long long)v[q]);
                    placed = true;
                    break;
                }
                h = (h + 1) & (HS - 1);
            }
            if (!placed) atomicAdd(node_fix + node, (unsigned long long)v[q]);
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
