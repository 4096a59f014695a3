// On-demand distance field for the serving pool.
//
// The reference builds the whole grid before the optimisation loop
// (Mesh::ConstructDistanceField, src/lib/mesh.cc:106-152) and every step reads
// the eight corners of the cell each vertex lies in (UniformGrid::
// DistanceFloat, src/lib/uniformgrid.cc:85-150).  Over a whole fit the
// vertices visit a small part of the grid, so here a cell's corners are
// computed the first time a vertex reaches the cell:
//   * admission: the target's traversal tree (mo_df_tree_build), and the
//     cells of the starting positions (mo_df_lazy_seed + mo_df_lazy_fill);
//   * step t (k_fused_step): a vertex whose new position lies in another cell
//     queues that cell unless its bit in df_cells is already set, and with it
//     the 4x4x2 voxel packets of the cell's corners whose bits in df_packets
//     are not set;
//   * after step t (mo_df_lazy_fill): one warp per queued packet computes its
//     32 voxels with the same per-voxel walk as the full build
//     (df_voxel_value), then one thread per queued cell writes its 8 corners
//     into the cell-layout grid.
// Every cell a step reads was written before that step, with the value the
// full build stores for each voxel (the exact minimum over all triangles,
// whatever the packet or visit order), so losses and trajectories are the
// full grid's bit for bit.
#include <cstdint>

#include "mo_df_trav.cuh"
#include "mo_lazydf.cuh"

namespace mo {

__global__ void __launch_bounds__(256) k_lazy_seed(const MoPair* __restrict__ pairs, int pair,
                                                   const float4* __restrict__ pos, int64_t nv,
                                                   int32_t* __restrict__ queue, int32_t* __restrict__ pqueue,
                                                   int32_t* __restrict__ counts, int cap) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const MoPair& P = pairs[pair];
    if (P.N > MO_DF_LAZY_MAX_N) {
        atomicOr(P.df_status, 16);
        return;
    }
    const float4 p = pos[i];
    lazy_queue_cell(P, pair, lazy_cell_of(P.N, p.x, p.y, p.z), queue, pqueue, counts, cap);
}

// One warp per queued packet: its 32 voxel values (4 x 4 x 2, x fastest).
__global__ void __launch_bounds__(TRAV_WARPS * 32) k_lazy_packets(const MoPair* __restrict__ pairs,
                                                                  const int32_t* __restrict__ pqueue,
                                                                  const int32_t* __restrict__ counts, int cap) {
    __shared__ int stack[TRAV_WARPS][TRAV_STACK];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t n = min((int64_t)counts[1], 8 * (int64_t)cap);
    for (int64_t e = (int64_t)blockIdx.x * TRAV_WARPS + w; e < n; e += (int64_t)gridDim.x * TRAV_WARPS) {
        const int pair = pqueue[2 * e], pk = pqueue[2 * e + 1];
        const MoPair& P = pairs[pair];
        const int N = P.N;
        const int bx = (N + 3) >> 2, by = (N + 3) >> 2;
        const int ix = pk % bx, iy = (pk / bx) % by, iz = pk / (bx * by);
        const int x = ix * 4 + (lane & 3), y = iy * 4 + ((lane >> 2) & 3), z = iz * 2 + (lane >> 4);
        const bool valid = x < N && y < N && z < N;
        const float band = P.df_band;
        const float band2 = band > 0.f ? band * band : FLT_MAX;
        const float4* tris = reinterpret_cast<const float4*>(P.df_tree);
        const float4* nodes = tris + tree_nodes_offset_f4(P.df_ntri);
        const float v = df_voxel_value(nodes, tris, P.df_ntri, N, band, band2, x, y, z, valid, stack[w],
                                       P.df_status);
        if (valid) P.df_lin[((int64_t)z * N + y) * N + x] = v;
        __syncwarp();
    }
}

// One thread per queued cell: its 8 corners (k = (bz<<2)|(by<<1)|bx) from the
// voxel values into the cell-layout grid.
__global__ void __launch_bounds__(256) k_lazy_cells(const MoPair* __restrict__ pairs,
                                                    const int32_t* __restrict__ queue,
                                                    const int32_t* __restrict__ counts, int cap,
                                                    unsigned long long* __restrict__ totals) {
    const int64_t n = min(counts[0], cap);
    if (totals && blockIdx.x == 0 && threadIdx.x == 0) {
        atomicAdd(totals, (unsigned long long)n);
        atomicAdd(totals + 1, (unsigned long long)min((int64_t)counts[1], 8 * (int64_t)cap));
    }
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const int pair = queue[2 * e], c = queue[2 * e + 1];
        const MoPair& P = pairs[pair];
        const int N = P.N, M = N - 1;
        const int cx = c % M, cy = (c / M) % M, cz = c / (M * M);
        const float* g = P.df_lin;
        const int64_t b = ((int64_t)cz * N + cy) * N + cx, sy = N, sz = (int64_t)N * N;
        float4* out = reinterpret_cast<float4*>(const_cast<float*>(P.grid)) + 2 * (int64_t)c;
        out[0] = make_float4(g[b], g[b + 1], g[b + sy], g[b + sy + 1]);
        out[1] = make_float4(g[b + sz], g[b + sz + 1], g[b + sz + sy], g[b + sz + sy + 1]);
    }
}

}  // namespace mo

using namespace mo;

extern "C" size_t mo_df_lazy_bytes(int N) {
    if (N < 2 || N > MO_DF_LAZY_MAX_N) return 0;
    return 4 * (size_t)(lazy_cell_words(N) + lazy_packet_words(N));
}

extern "C" int mo_df_lazy_seed(const MoPair* pairs, int pair, const float* pos4, int64_t nv, int32_t* queue,
                               int32_t* pqueue, int32_t* counts, int cap, void* stream) {
    MO_CHECK_ARG(nv >= 0 && pair >= 0 && cap >= 0, "negative size");
    MO_CHECK_ARG(cap < (1 << 28), "queue capacity too large");
    if (nv == 0) return MO_OK;
    MO_CHECK_ARG(pairs && pos4 && queue && pqueue && counts, "null pointer");
    MO_CHECK_ARG(aligned(pos4, 16), "positions must be 16-byte aligned float4");
    k_lazy_seed<<<ceil_div(nv, 256), 256, 0, as_stream(stream)>>>(pairs, pair, reinterpret_cast<const float4*>(pos4),
                                                                  nv, queue, pqueue, counts, cap);
    ::mo::note_launch();
    MO_LAUNCH_CHECK("k_lazy_seed");
    return MO_OK;
}

extern "C" int mo_df_lazy_fill(const MoPair* pairs, const int32_t* queue, const int32_t* pqueue,
                               const int32_t* counts, int cap, int64_t* totals, void* stream) {
    MO_CHECK_ARG(cap >= 0 && cap < (1 << 28), "bad queue capacity");
    MO_CHECK_ARG(pairs && queue && pqueue && counts, "null pointer");
    cudaStream_t s = as_stream(stream);
    // fixed grids (the counts are only known on the device), striding over
    // the queued packets, then the queued cells
    const int sms = device_sm_count();
    k_lazy_packets<<<4 * sms, TRAV_WARPS * 32, 0, s>>>(pairs, pqueue, counts, cap);
    ::mo::note_launch();
    k_lazy_cells<<<sms, 256, 0, s>>>(pairs, queue, counts, cap, reinterpret_cast<unsigned long long*>(totals));
    ::mo::note_launch();
    MO_LAUNCH_CHECK("k_lazy_cells");
    return MO_OK;
}
