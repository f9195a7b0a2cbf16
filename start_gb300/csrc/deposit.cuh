// Persistent P1 charge deposit into the fixed-point node accumulators, shared
// by the FP64 and the mixed-form deposit kernels.
//
// Each block walks one contiguous range of 256-particle tiles (the grid is
// one wave of blocks), with the next tile's particle loads issued before the
// current tile is reduced. A warp whose tile lies in one tet (the common case
// in tet-sorted order: a beam puts thousands of particles in a tet) adds the
// weights to per-lane running sums and reduces them only when its tet
// changes. In other tiles (the ends of runs, and particles that moved to
// other tets since the last re-sort) the lanes with equal tets (match_any)
// are summed by the integer reduce unit. Either way the lowest lane adds the
// tet's four sums to the block's table of tets in shared memory: one probe,
// four adds to adjacent words. The table is flushed into the node
// accumulators at the end of the range (four global atomics per listed tet),
// and also every kDepCheckTiles tiles if it is more than half full, so a
// range whose particles are spread over many tets keeps aggregating. While
// the table is over half full a tet it does not hold goes to the node
// accumulators directly. Integer sums do not depend on order, so the result
// is the same as one atomic per particle.
#ifndef SPG_DEPOSIT_CUH
#define SPG_DEPOSIT_CUH

#include <algorithm>
#include <cstdint>

#include "spg_internal.h"

namespace spg {

constexpr int kDepThreads = 256;
constexpr int kDepSlots = 1024;          // tet slots of a block's table
constexpr int kDepOpen = kDepSlots / 2;  // new tets enter while the table holds fewer
constexpr int kDepCheckTiles = 16;       // tiles between checks of the table's fill

struct DepositTable {
    int tet[kDepSlots];  // -1: free; a slot's tet does not change until the table is cleared
    unsigned long long sum[kDepSlots][4];
    unsigned int held;
};

// Sums of v[0..3] over the lanes of this lane's group (equal keys); returns
// the group's lane mask. v[1..3] are split into 21-bit pieces whose sums over
// at most 32 lanes fit 32 bits (a weight is at most 2^52 in magnitude, so the
// signed top piece v >> 42 is at most 2^10). When every weight of the warp is
// below 2^41 in magnitude (one <= 2^41, more than 2e6 particles, and
// barycentrics in about [-1, 1]) two pieces do: the signed v >> 21 is below
// 2^20. v[0] = one - v[1] - v[2] - v[3] sums to count * one minus the others.
__device__ __forceinline__ unsigned group_sums(int key, const long long v[4], long long one, long long sum[4]) {
    constexpr unsigned kAll = 0xffffffffu;
    const unsigned grp = __match_any_sync(kAll, key);
    bool big = false;
#pragma unroll
    for (int q = 1; q < 4; ++q) {
        const long long t = v[q] >> 41;
        big = big || (t != 0 && t != -1);
    }
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
    return grp;
}

// Appends tet `key` to the list of occupied tets once per deposit (the
// generation stamp of the tet says whether it is listed already).
__device__ __forceinline__ void list_tet(const OccList &occ, int key) {
    if (occ.list && __ldcg(occ.gen_of + key) != occ.gen && atomicExch(occ.gen_of + key, occ.gen) != occ.gen)
        occ.list[atomicAdd(occ.n, 1u)] = key;
}

// A tet's four node sums into the node accumulators.
__device__ __forceinline__ void tet_to_nodes(int key, const unsigned long long sum[4],
                                             const int4 *__restrict__ tet_nodes,
                                             unsigned long long *__restrict__ node_fix, const OccList &occ) {
    list_tet(occ, key);
    const int4 tn = __ldg(tet_nodes + key);
    if (sum[0]) atomicAdd(node_fix + tn.x, sum[0]);
    if (sum[1]) atomicAdd(node_fix + tn.y, sum[1]);
    if (sum[2]) atomicAdd(node_fix + tn.z, sum[2]);
    if (sum[3]) atomicAdd(node_fix + tn.w, sum[3]);
}

// Adds a tet's four sums to its slot (open addressing, linear probing). A
// free slot is claimed by compare-and-swap only while the table is at most
// half full; otherwise a tet the table does not hold goes to the node
// accumulators. The probe run ends at the tet or a free slot: fewer than
// kDepOpen + kDepThreads slots are ever taken between clears.
__device__ __forceinline__ void table_add(DepositTable &s, int key, const long long sum[4],
                                          const int4 *__restrict__ tet_nodes,
                                          unsigned long long *__restrict__ node_fix, const OccList &occ) {
    int h = int((unsigned(key) * 2654435761u) >> 8) & (kDepSlots - 1);
    for (int probe = 0; probe < kDepSlots; ++probe) {
        int cur = s.tet[h];
        if (cur == -1) {
            if (*(volatile unsigned int *)&s.held >= unsigned(kDepOpen)) break;
            cur = atomicCAS(&s.tet[h], -1, key);
            if (cur == -1) {
                atomicAdd(&s.held, 1u);
                cur = key;
            }
        }
        if (cur == key) {
            atomicAdd(&s.sum[h][0], (unsigned long long)sum[0]);
            atomicAdd(&s.sum[h][1], (unsigned long long)sum[1]);
            atomicAdd(&s.sum[h][2], (unsigned long long)sum[2]);
            atomicAdd(&s.sum[h][3], (unsigned long long)sum[3]);
            return;
        }
        h = (h + 1) & (kDepSlots - 1);
    }
    const unsigned long long u[4] = {(unsigned long long)sum[0], (unsigned long long)sum[1],
                                     (unsigned long long)sum[2], (unsigned long long)sum[3]};
    tet_to_nodes(key, u, tet_nodes, node_fix, occ);
}

__device__ __forceinline__ void table_clear(DepositTable &s) {
    for (int k = threadIdx.x; k < kDepSlots; k += kDepThreads) {
        s.tet[k] = -1;
        s.sum[k][0] = s.sum[k][1] = s.sum[k][2] = s.sum[k][3] = 0ull;
    }
    if (threadIdx.x == 0) s.held = 0u;
}

// Every held tet's sums into the node accumulators (after a barrier).
__device__ __forceinline__ void table_flush(const DepositTable &s, const int4 *__restrict__ tet_nodes,
                                            unsigned long long *__restrict__ node_fix, const OccList &occ) {
    for (int k = threadIdx.x; k < kDepSlots; k += kDepThreads)
        if (s.tet[k] >= 0) tet_to_nodes(s.tet[k], s.sum[k], tet_nodes, node_fix, occ);
}

// Warp sum of 64-bit values modulo 2^64 (three 21-bit pieces, the top one
// signed): exact whenever the true sum fits 64 bits.
__device__ __forceinline__ unsigned long long warp_sum64(unsigned long long v) {
    constexpr unsigned kAll = 0xffffffffu;
    const unsigned s0 = __reduce_add_sync(kAll, unsigned(v & 0x1FFFFFull));
    const unsigned s1 = __reduce_add_sync(kAll, unsigned((v >> 21) & 0x1FFFFFull));
    const int s2 = __reduce_add_sync(kAll, int((long long)v >> 42));
    return (unsigned long long)s0 + ((unsigned long long)s1 << 21) + ((unsigned long long)(long long)s2 << 42);
}

// The warp's running sums of tet key, reduced and added to the table by lane 0.
__device__ __forceinline__ void flush_running(DepositTable &s, int key, unsigned long long a1, unsigned long long a2,
                                              unsigned long long a3, int acnt, long long one,
                                              const int4 *__restrict__ tet_nodes,
                                              unsigned long long *__restrict__ node_fix, const OccList &occ) {
    long long sum[4];
    sum[1] = (long long)warp_sum64(a1);
    sum[2] = (long long)warp_sum64(a2);
    sum[3] = (long long)warp_sum64(a3);
    const unsigned long long cnt = __reduce_add_sync(0xffffffffu, unsigned(acnt));
    sum[0] = (long long)(cnt * (unsigned long long)one - (unsigned long long)sum[1] - (unsigned long long)sum[2] -
                         (unsigned long long)sum[3]);
    if ((threadIdx.x & 31) == 0) table_add(s, key, sum, tet_nodes, node_fix, occ);
}

// The deposit of particles [0, n) by one block of kDepThreads threads, its
// range of tiles given by blockIdx and gridDim. Src provides
//   Raw load(int64_t i, int64_t n): the particle's fields (a dead marker for i >= n);
//   int weights(const Raw &, long long v[4]): the tet (or -1: dead) and the
//     fixed-point weights v[0..3] summing to one (zeros for a dead particle);
//   long long one: the fixed-point one.
template <class Src>
__device__ __forceinline__ void deposit_tiles(const Src &src, int64_t n, const int4 *__restrict__ tet_nodes,
                                              unsigned long long *__restrict__ node_fix, const OccList &occ) {
    constexpr unsigned kAll = 0xffffffffu;
    __shared__ DepositTable s;
    table_clear(s);
    __syncthreads();
    const int64_t tiles = (n + kDepThreads - 1) / kDepThreads;
    const int64_t per = (tiles + gridDim.x - 1) / gridDim.x;
    const int64_t t0 = int64_t(blockIdx.x) * per;
    const int64_t t1 = t0 + per < tiles ? t0 + per : tiles;
    const int lane = threadIdx.x & 31;
    int acc_key = -1;                           // warp-uniform: the tet of the running sums (-1: none)
    unsigned long long a1 = 0, a2 = 0, a3 = 0;  // modulo 2^64: the node totals fit 63 bits
    int acnt = 0;                               // this lane's alive particles in the running sums
    int64_t i = t0 * kDepThreads + threadIdx.x;
    typename Src::Raw nxt = src.load(i, t0 < t1 ? n : 0);
    for (int64_t t = t0; t < t1; ++t, i += kDepThreads) {
        if ((t - t0) % kDepCheckTiles == kDepCheckTiles - 1) {  // block-uniform
            __syncthreads();
            if (s.held >= unsigned(kDepOpen)) {
                table_flush(s, tet_nodes, node_fix, occ);
                __syncthreads();
                table_clear(s);
            }
            __syncthreads();
        }
        const typename Src::Raw cur = nxt;
        nxt = src.load(i + kDepThreads, t + 1 < t1 ? n : 0);
        long long v[4];
        const int key = src.weights(cur, v);
        const int kmax = __reduce_max_sync(kAll, key);
        if (__all_sync(kAll, key == kmax || key < 0)) {
            if (kmax != acc_key && kmax >= 0) {
                if (acc_key >= 0) flush_running(s, acc_key, a1, a2, a3, acnt, src.one, tet_nodes, node_fix, occ);
                acc_key = kmax;
                a1 = a2 = a3 = 0;
                acnt = 0;
            }
            a1 += (unsigned long long)v[1];
            a2 += (unsigned long long)v[2];
            a3 += (unsigned long long)v[3];
            acnt += key >= 0;
        } else {
            long long sum[4];
            const unsigned grp = group_sums(key, v, src.one, sum);
            if (key >= 0 && lane == __ffs(grp) - 1) table_add(s, key, sum, tet_nodes, node_fix, occ);
        }
    }
    if (acc_key >= 0) flush_running(s, acc_key, a1, a2, a3, acnt, src.one, tet_nodes, node_fix, occ);
    __syncthreads();
    table_flush(s, tet_nodes, node_fix, occ);
}

// Blocks of `kernel` resident on the whole GPU at once (the deposit's one wave).
template <class K>
inline int resident_blocks(K kernel, int threads) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0);
    return std::max(1, sms * std::max(1, per_sm));
}

}  // namespace spg

#endif
