// Block-level aggregation for the counting sort of particles by tet.
//
// The particles are already close to tet order when they are re-sorted, and a
// beam puts hundreds of them in one tet, so consecutive warps hit the same
// global bin. Warp groups of equal keys (match_any) are merged per block in a
// shared open-addressing table first: each bin then takes one global atomic
// per block instead of one per warp.
#pragma once
#include <cstdint>

namespace spg {

constexpr int kSortBlock = 256;
constexpr int kSortSlots = 2 * kSortBlock;  // at most kSortBlock distinct keys per block

struct SortTable {
    int key[kSortSlots];
    int count[kSortSlots];
    int base[kSortSlots];
};

__device__ __forceinline__ void sort_table_clear(SortTable &t) {
    for (int s = threadIdx.x; s < kSortSlots; s += blockDim.x) {
        t.key[s] = -1;
        t.count[s] = 0;
    }
}

// Slot of key (inserted if absent). The table has twice as many slots as the
// block has threads, so a free slot exists and the probe ends within
// kSortSlots steps.
__device__ __forceinline__ int sort_table_slot(SortTable &t, int key) {
    int h = int((unsigned(key) * 2654435761u) >> 23);  // 9 bits: kSortSlots = 512
    for (int probe = 0; probe < kSortSlots; ++probe) {
        const int old = atomicCAS(&t.key[h], -1, key);
        if (old == -1 || old == key) return h;
        h = (h + 1) & (kSortSlots - 1);
    }
    return -1;  // unreachable: at most kSortBlock keys are inserted
}

// Histogram of keys (key < 0: no particle) into cnt.
__device__ __forceinline__ void sort_hist_block(SortTable &t, int key, int32_t *cnt) {
    sort_table_clear(t);
    __syncthreads();
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int lane = threadIdx.x & 31;
    if (key >= 0 && lane == __ffs(peers) - 1) {
        const int h = sort_table_slot(t, key);
        if (h >= 0) atomicAdd(&t.count[h], __popc(peers));
    }
    __syncthreads();
    for (int s = threadIdx.x; s < kSortSlots; s += blockDim.x)
        if (t.key[s] >= 0) atomicAdd(cnt + t.key[s], t.count[s]);
}

// Destination index of this thread's particle (key < 0: none, returns -1):
// offs[key] is the next free index of bin key.
__device__ __forceinline__ int64_t sort_dest_block(SortTable &t, int key, int32_t *offs) {
    sort_table_clear(t);
    __syncthreads();
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    int h = -1, local = 0;
    if (key >= 0 && lane == leader) {
        h = sort_table_slot(t, key);
        if (h >= 0) local = atomicAdd(&t.count[h], __popc(peers));
    }
    __syncthreads();
    for (int s = threadIdx.x; s < kSortSlots; s += blockDim.x)
        if (t.key[s] >= 0) t.base[s] = atomicAdd(offs + t.key[s], t.count[s]);
    __syncthreads();
    int64_t first = 0;
    if (key >= 0 && lane == leader && h >= 0) first = int64_t(t.base[h]) + local;
    first = __shfl_sync(0xffffffffu, first, leader);
    if (key < 0) return -1;
    return first + __popc(peers & ((1u << lane) - 1u));
}

// Counting-sort scatter of one particle array set (DevParticles or
// DevParticles32): the eight fields are loaded before the bin offsets are
// taken, so the loads overlap the atomics.
template <class P>
__device__ __forceinline__ void sort_scatter_block(SortTable &t, const P &src, P &dst, int64_t n, int n_tets,
                                                   uint32_t dead_mask, int32_t *offs) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const bool have = i < n;
    const int64_t k = have ? i : 0;
    const auto x = src.x[k], y = src.y[k], z = src.z[k];
    const auto vx = src.vx[k], vy = src.vy[k], vz = src.vz[k];
    const int32_t tet = src.tet[k];
    const uint32_t idf = src.idf[k];
    const int key = have ? ((idf & dead_mask) ? n_tets : tet) : -1;
    const int64_t j = sort_dest_block(t, key, offs);
    if (j < 0) return;
    dst.x[j] = x;
    dst.y[j] = y;
    dst.z[j] = z;
    dst.vx[j] = vx;
    dst.vy[j] = vy;
    dst.vz[j] = vz;
    dst.tet[j] = tet;
    dst.idf[j] = idf;
}

}  // namespace spg
