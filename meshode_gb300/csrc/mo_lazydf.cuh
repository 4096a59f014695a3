// On-demand distance-field cells: the bit sets and the queue shared by the
// fused step (which queues the cells its vertices move into) and the fills
// (mo_lazydf.cu).
#pragma once

#include "mo_df_eval.cuh"

namespace mo {

// Packet index of voxel (x, y, z): 4 x 4 x 2 voxels, x fastest.
__device__ __forceinline__ int lazy_packet(int N, int x, int y, int z) {
    const int bx = (N + 3) >> 2, by = (N + 3) >> 2;
    return ((z >> 1) * by + (y >> 2)) * bx + (x >> 2);
}

__host__ __device__ __forceinline__ int64_t lazy_cell_words(int N) {
    const int64_t M = N - 1;
    return (M * M * M + 31) / 32;
}

__host__ __device__ __forceinline__ int64_t lazy_packet_words(int N) {
    const int64_t b = (N + 3) / 4;
    return (b * b * ((N + 1) / 2) + 31) / 32;
}

// Append (a, b) for every converged lane with `want`: one atomicAdd per
// warp for the lanes that append together.
__device__ __forceinline__ void warp_append(bool want, int a, int b, int32_t* __restrict__ queue,
                                            int32_t* __restrict__ count, int cap, int32_t* __restrict__ status) {
    const unsigned act = __activemask();
    const unsigned m = __ballot_sync(act, want);
    if (!want) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(count, __popc(m));
    base = __shfl_sync(m, base, leader);
    const int slot = base + __popc(m & ((1u << lane) - 1));
    if (slot < cap) {
        queue[2 * (int64_t)slot] = a;
        queue[2 * (int64_t)slot + 1] = b;
    } else {
        atomicOr(status, 8);  // cannot happen: the queues hold a cell per vertex, 8 packets per cell
    }
}

// Set bit i of a bit set; true when this call set it.
__device__ __forceinline__ bool lazy_claim(uint32_t* __restrict__ bits, int i) {
    uint32_t* wd = bits + (i >> 5);
    const uint32_t bit = 1u << (i & 31);
    if (__ldcg(wd) & bit) return false;
    return !(atomicOr(wd, bit) & bit);
}

// Queue cell c (-1: none) of pair `pair` unless it is queued already (its
// bit stays set from the step that queued it; the fill after that step
// writes it), with the packets of its corners not queued before.  Every
// lane of the warp that reached the cell test calls it.
__device__ __forceinline__ void lazy_queue_cell(const MoPair& P, int pair, int c, int32_t* __restrict__ queue,
                                                int32_t* __restrict__ pqueue, int32_t* __restrict__ counts,
                                                int cap) {
    const bool mine = c >= 0 && lazy_claim(P.df_cells, c);
    warp_append(mine, pair, c, queue, counts, cap, P.df_status);
    if (!mine) return;
    const int N = P.N, M = N - 1;
    const int cx = c % M, cy = (c / M) % M, cz = c / (M * M);
    int seen[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int pk = lazy_packet(N, cx + (j & 1), cy + ((j >> 1) & 1), cz + (j >> 2));
        seen[j] = pk;
        bool dup = false;
#pragma unroll
        for (int jj = 0; jj < j; ++jj) dup |= seen[jj] == pk;
        if (dup || !lazy_claim(P.df_packets, pk)) continue;
        const int slot = atomicAdd(counts + 1, 1);
        if (slot < 8 * cap) {
            pqueue[2 * (int64_t)slot] = pair;
            pqueue[2 * (int64_t)slot + 1] = pk;
        } else {
            atomicOr(P.df_status, 8);
        }
    }
}

// Cell of a position, as df_eval finds it; -1 when the lookup reads no cell.
__device__ __forceinline__ int lazy_cell_of(int N, float x, float y, float z) {
    const float Nf = (float)N;
    const int px = trunc_i32_x86(MUL(x, Nf)), py = trunc_i32_x86(MUL(y, Nf)), pz = trunc_i32_x86(MUL(z, Nf));
    const int M = N - 1;
    if (px < 0 || py < 0 || pz < 0 || px >= M || py >= M || pz >= M) return -1;
    return (pz * M + py) * M + px;
}

}  // namespace mo
