// Optimiser-step kernels: the stand-alone Adam update and the fused
// multi-pair step (DF loss + gradient, CSR-ordered edge gradient, mask and
// weights, Adam, loss partials) that advances every active deformation pair
// by one step per launch.
// Reference: the loop body of src/python/rigid_deform.py:35-39 with
// RigidLossFunction (src/python/layers/rigid_loss_layer.py:7-27) or
// GraphLossFunction (src/python/layers/graph_loss_layer.py:9-43) and
// torch.optim.Adam.
#include "mo_lazydf.cuh"

namespace mo {

// torch/optim/adam.py _single_tensor_adam for one element:
//   m.lerp_(g, 1-b1); v.mul_(b2).addcmul_(g, g, value=1-b2);
//   denom = v.sqrt()/bc2_sqrt + eps; p.addcdiv_(m, denom, value=-step_size)
__device__ __forceinline__ void adam_elem(float& p, float g, float& m, float& v, float omb1, float b2, float omb2,
                                          float eps, float step_size, float bc2s) {
    m = fmaf(omb1, g - m, m);
    v = ADD(MUL(v, b2), MUL(MUL(omb2, g), g));
    const float denom = ADD(__fdiv_rn(__fsqrt_rn(v), bc2s), eps);
    p = fmaf(-step_size, __fdiv_rn(m, denom), p);
}

__global__ void __launch_bounds__(256) k_adam(float* __restrict__ P, const float* __restrict__ G,
                                              float* __restrict__ M, float* __restrict__ Vs, int64_t n,
                                              float omb1, float b2, float omb2, float eps, float step_size,
                                              float bc2s) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float p = P[i], m = M[i], v = Vs[i];
    adam_elem(p, G[i], m, v, omb1, b2, omb2, eps, step_size, bc2s);
    P[i] = p; M[i] = m; Vs[i] = v;
}

constexpr int STEP_THREADS = 256;  // 8 warps = up to 8 slices of 32 vertices
constexpr int TILE_WARPS = STEP_THREADS / 32;
static_assert(TILE_WARPS == MO_TILE_WARPS, "tile warps");
constexpr int REC_UNROLL = 3;      // record rows whose neighbours are gathered together

template <int LAYOUT>
__device__ __forceinline__ DFJet df_eval_layout(const float* grid, int N, float Nf, float Cf, float x, float y,
                                                float z) {
    return df_eval<LAYOUT, true>(grid, N, Nf, Cf, x, y, z);
}

// Every warp owns one 32-vertex slice of a tile and never waits for the
// other warps of its block.  ON_DEMAND: the pairs' grids are filled on
// demand, and a vertex moving into a cell not yet filled queues it (a
// separate instantiation: the queueing code slows the plain kernel down even
// when it is skipped).  WEIGHTED: every record carries a weight
// (MoPair.sell_w, NULL: 1): the gradient takes r * w^2 and the energy
// (r * w)^2 (CadEdgeLoss), another separate instantiation.
template <bool ON_DEMAND, bool WEIGHTED = false>
__global__ void __launch_bounds__(STEP_THREADS, 4) k_fused_step(const MoPair* __restrict__ pairs,
                                                             const MoTile* __restrict__ tiles,
                                                             const int* __restrict__ ntiles_p, int max_tiles,
                                                             int k, float* __restrict__ tile_loss) {
    const int ntiles = min(*ntiles_p, max_tiles);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const MoTile T = tiles[tile];
        const MoPair& P = pairs[T.pair];
        float* out = tile_loss + ((int64_t)k * max_tiles + tile) * TILE_WARPS + w;
        const int t = P.t0 + k + 1;
        if (t > P.t_end || w >= T.nslices) {  // warp-uniform
            if (lane == 0) *out = 0.f;
            continue;
        }
        const int slice = T.slice0 + w;
        const int nv = P.nv;
        const int i = slice * 32 + lane;
        const bool valid = i < nv;
        const float4* __restrict__ Vin = reinterpret_cast<const float4*>((t & 1) ? P.pos0 : P.pos1);
        float4* __restrict__ Vout = reinterpret_cast<float4*>((t & 1) ? P.pos1 : P.pos0);
        const float4* __restrict__ R = reinterpret_cast<const float4*>(P.rest);
        const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 p = valid ? Vin[i] : zero;
        const float4 r0 = valid ? __ldg(R + i) : zero;
        float* __restrict__ Mm = P.adam_m + 3 * (int64_t)i;
        float* __restrict__ Vv = P.adam_v + 3 * (int64_t)i;
        if (valid) {  // the moments are read after the edge loop
            asm volatile("prefetch.global.L1 [%0];" :: "l"(Mm));
            asm volatile("prefetch.global.L1 [%0];" :: "l"(Vv));
        }
        // The first record rows are requested before the distance-field cell
        // so that both gathers are in flight together.
        const int rb = P.slice_ptr[slice];
        const int rows = (P.slice_ptr[slice + 1] - rb) >> 5;
        const int* __restrict__ rec = P.sell + rb + lane;
        int c[REC_UNROLL];
#pragma unroll
        for (int u = 0; u < REC_UNROLL; ++u) c[u] = (u < rows) ? __ldg(rec + u * 32) : -1;
        const float* __restrict__ recw = WEIGHTED && P.sell_w ? P.sell_w + rb + lane : nullptr;
        const int N = P.N;
        const float Nf = (float)N, Cf = (float)((double)(N - 1) - 1e-3);
        const DFJet j = (P.layout == MO_LAYOUT_CELL)
                            ? df_eval_layout<MO_LAYOUT_CELL>(P.grid, N, Nf, Cf, p.x, p.y, p.z)
                            : (P.layout == MO_LAYOUT_BRICK4)
                                  ? df_eval_layout<MO_LAYOUT_BRICK4>(P.grid, N, Nf, Cf, p.x, p.y, p.z)
                                  : df_eval_layout<MO_LAYOUT_LINEAR>(P.grid, N, Nf, Cf, p.x, p.y, p.z);
        const float dsq = MUL(j.d, j.d);
        float gdx = df_grad_component(j.d, j.gx);
        float gdy = df_grad_component(j.d, j.gy);
        float gdz = df_grad_component(j.d, j.gz);
        if (P.use_mask) {
            const float mk = (MUL(dsq, 0.5f) < P.mask_thresh) ? 1.0f : 0.0f;
            gdx = MUL(gdx, mk); gdy = MUL(gdy, mk); gdz = MUL(gdz, mk);
        }
        // Edge residuals over this vertex's sliced-ELL column, in the order
        // of the reference's serial scatter.  Rest offset = rest[v1] - rest[v0].
        // The next rows' records are requested while this row's neighbours
        // are gathered.
        float grx = 0.f, gry = 0.f, grz = 0.f, esq = 0.f;
        for (int row = 0; row < rows; row += REC_UNROLL) {
            float4 q[REC_UNROLL], sr[REC_UNROLL];
#pragma unroll
            for (int u = 0; u < REC_UNROLL; ++u) {
                if (c[u] != -1) {
                    const int o = c[u] & 0x7fffffff;
                    q[u] = Vin[o];
                    sr[u] = __ldg(R + o);
                } else {
                    q[u] = zero;
                    sr[u] = zero;
                }
            }
            int cn[REC_UNROLL];
#pragma unroll
            for (int u = 0; u < REC_UNROLL; ++u)
                cn[u] = (row + REC_UNROLL + u < rows) ? __ldg(rec + (row + REC_UNROLL + u) * 32) : -1;
            // As v0 of a half-edge the vertex takes g -= r with r = (v1 - v0) - off;
            // as v1 it takes g += (v0 - v1) - (-off), which is the same
            // rounding of the same r with its sign flipped, so both roles
            // subtract r = (q - p) - (rest[q] - rest[p]); only v0 adds the
            // edge's energy.  Padding (-1) follows the last real record.
#pragma unroll
            for (int u = 0; u < REC_UNROLL; ++u) {
                const float rx = SUB(SUB(q[u].x, p.x), SUB(sr[u].x, r0.x));
                const float ry = SUB(SUB(q[u].y, p.y), SUB(sr[u].y, r0.y));
                const float rz = SUB(SUB(q[u].z, p.z), SUB(sr[u].z, r0.z));
                if (WEIGHTED) {
                    // (v1 - v0 - off) * (w * w) as cad_layer.cc:195-202
                    // rounds it; the v1 role's r is the v0 role's negated
                    const float we_ = (recw && c[u] != -1) ? __ldg(recw + (row + u) * 32) : 1.0f;
                    const float l2 = MUL(we_, we_);
                    if (c[u] != -1) {
                        grx = SUB(grx, MUL(rx, l2)); gry = SUB(gry, MUL(ry, l2)); grz = SUB(grz, MUL(rz, l2));
                    }
                    if (c[u] >= 0) {
                        const float ex = MUL(rx, we_), ey = MUL(ry, we_), ez = MUL(rz, we_);
                        esq += ex * ex + ey * ey + ez * ez;
                    }
                } else {
                    if (c[u] != -1) {
                        grx = SUB(grx, rx); gry = SUB(gry, ry); grz = SUB(grz, rz);
                    }
                    if (c[u] >= 0) esq += rx * rx + ry * ry + rz * rz;
                }
            }
            if (c[REC_UNROLL - 1] == -1) break;
#pragma unroll
            for (int u = 0; u < REC_UNROLL; ++u) c[u] = cn[u];
        }
        // grad_h * (gD + gR * w)  (graph_loss_layer.py:42, rigid_loss_layer.py:27)
        const float we = P.w_edge, gh = P.grad_scale;
        const float gx = MUL(gh, ADD(gdx, MUL(grx, we)));
        const float gy = MUL(gh, ADD(gdy, MUL(gry, we)));
        const float gz = MUL(gh, ADD(gdz, MUL(grz, we)));
        float part = 0.f;
        if (valid) {
            if (P.grad_dbg) {
                P.grad_dbg[3 * (int64_t)i] = gx;
                P.grad_dbg[3 * (int64_t)i + 1] = gy;
                P.grad_dbg[3 * (int64_t)i + 2] = gz;
            }
            const float2 ab = __ldg(reinterpret_cast<const float2*>(P.adam_tab) + (t - 1));
            float m0 = Mm[0], m1 = Mm[1], m2 = Mm[2];
            float v0 = Vv[0], v1 = Vv[1], v2 = Vv[2];
            float px = p.x, py = p.y, pz = p.z;
            adam_elem(px, gx, m0, v0, P.one_minus_b1, P.b2, P.one_minus_b2, P.eps, ab.x, ab.y);
            adam_elem(py, gy, m1, v1, P.one_minus_b1, P.b2, P.one_minus_b2, P.eps, ab.x, ab.y);
            adam_elem(pz, gz, m2, v2, P.one_minus_b1, P.b2, P.one_minus_b2, P.eps, ab.x, ab.y);
            Mm[0] = m0; Mm[1] = m1; Mm[2] = m2;
            Vv[0] = v0; Vv[1] = v1; Vv[2] = v2;
            Vout[i] = make_float4(px, py, pz, 0.f);
            if (ON_DEMAND && P.df_cells != nullptr && t < P.t_end) {  // the next step's cell
                int cn = lazy_cell_of(N, px, py, pz);
                if (cn == lazy_cell_of(N, p.x, p.y, p.z)) cn = -1;  // read by this step: written
                lazy_queue_cell(P, T.pair, cn, P.df_queue, P.df_pqueue, P.df_queue_count + 2 * k,
                                P.df_queue_cap);
            }
            part = 0.5f * dsq + we * (0.5f * esq);
        }
        for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
        if (lane == 0) *out = part;
    }
}

// One warp per (pair, launch): lane l sums the pair's tile partials l, l+32,
// ... in double, then a fixed shuffle tree adds the 32 lane sums.  The order
// is fixed, so the result does not depend on scheduling.
__global__ void __launch_bounds__(128) k_pair_loss(const MoPair* __restrict__ pairs, int npairs, int max_tiles,
                                                   int nlaunch, const float* __restrict__ tile_loss,
                                                   double* __restrict__ out) {
    const int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (q >= (int64_t)npairs * nlaunch) return;  // warp-uniform
    const int p = (int)(q % npairs), k = (int)(q / npairs);
    const MoPair& P = pairs[p];
    const float* base = tile_loss + (int64_t)k * max_tiles * TILE_WARPS;
    const int64_t t0 = (int64_t)P.tile0 * TILE_WARPS, t1 = (int64_t)(P.tile0 + P.ntiles) * TILE_WARPS;
    double s = 0.0;
    for (int64_t t = t0 + lane; t < t1; t += 32) s += (double)base[t];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) out[(int64_t)k * npairs + p] = s;
}

__global__ void k_pack(const float* __restrict__ V, int64_t n, float4* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = make_float4(V[3 * i], V[3 * i + 1], V[3 * i + 2], 0.f);
}

__global__ void k_unpack(const float4* __restrict__ P, int64_t n, float* __restrict__ V) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const float4 p = P[i];
        V[3 * i] = p.x; V[3 * i + 1] = p.y; V[3 * i + 2] = p.z;
    }
}

static int g_step_ctas = 0;

static int step_ctas() {
    if (g_step_ctas == 0) {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fused_step<false>, STEP_THREADS, 0) !=
                cudaSuccess ||
            per_sm <= 0)
            per_sm = 4;
        g_step_ctas = per_sm * device_sm_count();
    }
    return g_step_ctas;
}

}  // namespace mo

using namespace mo;

extern "C" int mo_adam_step(float* P, const float* G, float* M, float* Vsq, int64_t n, float one_minus_b1, float b2,
                            float one_minus_b2, float eps, float step_size, float bc2_sqrt, void* stream) {
    MO_CHECK_ARG(n >= 0, "negative size");
    if (n == 0) return MO_OK;
    MO_CHECK_ARG(P && G && M && Vsq, "null pointer");
    k_adam<<<ceil_div(n, 256), 256, 0, as_stream(stream)>>>(P, G, M, Vsq, n, one_minus_b1, b2, one_minus_b2, eps,
                                                           step_size, bc2_sqrt); ::mo::note_launch();
    MO_LAUNCH_CHECK("k_adam");
    return MO_OK;
}

static int launch_fused_step(int variant, const MoPair* pairs, const MoTile* tiles, const int32_t* ntiles,
                             int max_tiles, int launch_index, float* tile_loss, int grid_ctas, void* stream) {
    MO_CHECK_ARG(pairs && tiles && ntiles && tile_loss, "null pointer");
    MO_CHECK_ARG(max_tiles >= 0 && launch_index >= 0, "negative size");
    if (max_tiles == 0) return MO_OK;
    int ctas = grid_ctas > 0 ? grid_ctas : step_ctas();
    if (ctas > max_tiles) ctas = max_tiles;
    if (variant == 1)
        k_fused_step<true><<<ctas, STEP_THREADS, 0, as_stream(stream)>>>(pairs, tiles, ntiles, max_tiles,
                                                                         launch_index, tile_loss);
    else if (variant == 2)
        k_fused_step<false, true><<<ctas, STEP_THREADS, 0, as_stream(stream)>>>(pairs, tiles, ntiles, max_tiles,
                                                                                launch_index, tile_loss);
    else
        k_fused_step<false><<<ctas, STEP_THREADS, 0, as_stream(stream)>>>(pairs, tiles, ntiles, max_tiles,
                                                                          launch_index, tile_loss);
    ::mo::note_launch();
    MO_LAUNCH_CHECK("k_fused_step");
    return MO_OK;
}

extern "C" int mo_fused_step(const MoPair* pairs, const MoTile* tiles, const int32_t* ntiles, int max_tiles,
                             int launch_index, float* tile_loss, int grid_ctas, void* stream) {
    return launch_fused_step(0, pairs, tiles, ntiles, max_tiles, launch_index, tile_loss, grid_ctas, stream);
}

extern "C" int mo_fused_step_weighted(const MoPair* pairs, const MoTile* tiles, const int32_t* ntiles, int max_tiles,
                                      int launch_index, float* tile_loss, int grid_ctas, void* stream) {
    return launch_fused_step(2, pairs, tiles, ntiles, max_tiles, launch_index, tile_loss, grid_ctas, stream);
}

extern "C" int mo_fused_step_on_demand(const MoPair* pairs, const MoTile* tiles, const int32_t* ntiles,
                                       int max_tiles, int launch_index, float* tile_loss, int grid_ctas,
                                       void* stream) {
    return launch_fused_step(1, pairs, tiles, ntiles, max_tiles, launch_index, tile_loss, grid_ctas, stream);
}

extern "C" int mo_pair_loss(const MoPair* pairs, int npairs, int max_tiles, int nlaunch, const float* tile_loss,
                            double* pair_loss, void* stream) {
    MO_CHECK_ARG(npairs >= 0 && nlaunch >= 0 && max_tiles >= 0, "negative size");
    const int64_t n = (int64_t)npairs * nlaunch;
    if (n == 0) return MO_OK;
    MO_CHECK_ARG(pairs && tile_loss && pair_loss, "null pointer");
    k_pair_loss<<<ceil_div(n, 4), 128, 0, as_stream(stream)>>>(pairs, npairs, max_tiles, nlaunch, tile_loss,
                                                              pair_loss); ::mo::note_launch();
    MO_LAUNCH_CHECK("k_pair_loss");
    return MO_OK;
}

extern "C" int mo_pack_pos(const float* V, int64_t n, float* pos4, void* stream) {
    MO_CHECK_ARG(n >= 0, "negative size");
    if (n == 0) return MO_OK;
    MO_CHECK_ARG(V && pos4 && aligned(pos4, 16), "null or misaligned pointer");
    k_pack<<<ceil_div(n, 256), 256, 0, as_stream(stream)>>>(V, n, reinterpret_cast<float4*>(pos4)); ::mo::note_launch();
    MO_LAUNCH_CHECK("k_pack");
    return MO_OK;
}

extern "C" int mo_unpack_pos(const float* pos4, int64_t n, float* V, void* stream) {
    MO_CHECK_ARG(n >= 0, "negative size");
    if (n == 0) return MO_OK;
    MO_CHECK_ARG(V && pos4 && aligned(pos4, 16), "null or misaligned pointer");
    k_unpack<<<ceil_div(n, 256), 256, 0, as_stream(stream)>>>(reinterpret_cast<const float4*>(pos4), n, V); ::mo::note_launch();
    MO_LAUNCH_CHECK("k_unpack");
    return MO_OK;
}

extern "C" int mo_abi_sizes(size_t* pair_bytes, size_t* tile_bytes) {
    MO_CHECK_ARG(pair_bytes && tile_bytes, "null pointer");
    *pair_bytes = sizeof(MoPair);
    *tile_bytes = sizeof(MoTile);
    return MO_OK;
}
