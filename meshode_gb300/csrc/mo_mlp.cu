// Fused kernels of the velocity-field MLP (3 -> 256 -> 256 -> 256 -> 3,
// softplus), the dense contraction of the velocity-field ODE deformation
// (the NeuralODE variant of src/python/layers/neuralode_fast.py:10-31,55-57,
// widened to 256 units, autonomous, integrated by fixed-step RK4).
//
// All arithmetic is FP32 on the SIMT pipes (packed FFMA2): the fit's
// parameter gradients must stay within 1e-5 of FP64, which TF32 or BF16
// tensor-core products would miss.
//
//   k_mlp_fwd    one MLP evaluation of a 64-vertex tile with its RK4 stage
//                update: the 3-wide input layer, the two 256x256 layers and
//                the 3-wide output layer; the tile's 64x256 activations stay
//                in shared memory between layers (k-major, padded), the
//                weights stream through a double-buffered cp.async stage.
//                Optionally stores Z and H of the three hidden layers for the
//                backward.
//   k_mlp_bwd    the vector-Jacobian product of one evaluation for a tile:
//                g_z3 = (g_k W4) * sigmoid(z3), g_z2 = (g_z3 W3) *
//                sigmoid(z2), g_z1 = (g_z2 W2) * sigmoid(z1), g_u = g_z1 W1;
//                the gradients g_z3 and g_z2 go to global memory for the
//                weight gradients, the small ones (dW4, db4, db3, db2, db1,
//                dW1) to one partial row per warp.
//   k_mlp_wgrad  dW += A^T B over many rows (A = g_z, B = H of all four
//                stages of an RK4 step): split over rows, one 128x128
//                output block per CTA, partial sums reduced in a fixed order
//                by k_mlp_wgrad_reduce (deterministic).
//
// A hidden width below 256 is run as 256 with zero-padded weights: a padded
// unit's pre-activation is 0 and its outgoing weights are 0, so every real
// unit's value is the unpadded one exactly (x + 0*h == x).
#include "mo_common.cuh"

namespace mo {
namespace mlp {

constexpr int M = 256;         // hidden width
constexpr int BM = 64;         // vertices per CTA tile
constexpr int THREADS = 256;   // 8 warps; warp w owns tile rows 8w..8w+7
constexpr int BK = 16;         // weight rows per staged chunk
constexpr int AT_LD = BM + 4;  // row stride (floats) of the k-major activation tile
constexpr int PW = 3 * M + 4 + 3 * M + 3 * M;  // partial row: dW4[3][M], db4[4], db3, db2, db1, dW1[M][3]
constexpr int P_DW4 = 0, P_DB4 = 3 * M, P_DB3 = 3 * M + 4, P_DB2 = P_DB3 + M, P_DB1 = P_DB2 + M, P_DW1 = P_DB1 + M;
static_assert(P_DW1 + 3 * M == PW, "partial row layout");

struct Smem {
    float at[M * AT_LD];  // activations of the tile, at[k * AT_LD + row]
    float bs[2][BK * M];  // two chunks of BK weight rows
};
constexpr size_t SMEM_BYTES = sizeof(Smem);

__device__ __forceinline__ float softplus(float z) { return z > 20.f ? z : log1pf(expf(z)); }
__device__ __forceinline__ float sigmoid(float z) { return 1.f / (1.f + expf(-z)); }

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
// 16 bytes, or zeros when !pred (the source is not read then)
__device__ __forceinline__ void cp_async16_zfill(void* smem, const void* gmem, bool pred) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    const int n = pred ? 16 : 0;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(n));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

// The thread's columns: pairs j = 0, 1 at 4*lane + 2j, pairs j = 2, 3 at
// 128 + 4*lane + 2(j-2) (two float4 per row, conflict-free in shared memory).
__device__ __forceinline__ int col_of(int lane, int j, int e) { return (j < 2 ? 0 : 128) + 4 * lane + 2 * (j & 1) + e; }

// Weight rows [kc*BK, kc*BK + BK) of the row-major M x M matrix B.
__device__ __forceinline__ void load_chunk(float* bs, const float* __restrict__ B, int kc, int tid) {
    const float* src = B + (size_t)kc * BK * M;
#pragma unroll
    for (int j = 0; j < BK * M / 4 / THREADS; ++j) {
        const int f = tid + j * THREADS;
        cp_async16(bs + 4 * f, src + 4 * f);
    }
}

// acc[i][j] += sum_k at[k][8w + i] * B[k][cols of pair j], k = 0..M-1.
// Starts and ends with all threads synchronised (the caller may then
// overwrite `at`).
__device__ __forceinline__ void gemm_tile(Smem& S, const float* __restrict__ B, float2 (&acc)[8][4], int tid, int w,
                                          int lane) {
    load_chunk(S.bs[0], B, 0, tid);
    cp_async_commit();
#pragma unroll 1
    for (int kc = 0; kc < M / BK; ++kc) {
        const float* cur = S.bs[kc & 1];
        if (kc + 1 < M / BK) {
            load_chunk(S.bs[(kc + 1) & 1], B, kc + 1, tid);
            cp_async_commit();
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            const float* ap = S.at + (kc * BK + kk) * AT_LD + 8 * w;
            const float4 a0 = *reinterpret_cast<const float4*>(ap);
            const float4 a1 = *reinterpret_cast<const float4*>(ap + 4);
            const float4 b0 = *reinterpret_cast<const float4*>(cur + kk * M + 4 * lane);
            const float4 b1 = *reinterpret_cast<const float4*>(cur + kk * M + 128 + 4 * lane);
            const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float2 bb[4] = {make_float2(b0.x, b0.y), make_float2(b0.z, b0.w), make_float2(b1.x, b1.y),
                                  make_float2(b1.z, b1.w)};
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const float2 ai = make_float2(av[i], av[i]);
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = __ffma2_rn(ai, bb[j], acc[i][j]);
            }
        }
        __syncthreads();
    }
}

__device__ __forceinline__ void zero_acc(float2 (&acc)[8][4]) {
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = make_float2(0.f, 0.f);
}

// v[i][c] (8 rows x the thread's 8 columns, as pairs) into the k-major tile.
__device__ __forceinline__ void put_tile(Smem& S, const float2 (&v)[8][4], int w, int lane) {
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            float* p = S.at + col_of(lane, j, e) * AT_LD + 8 * w;
            const float r[8] = {e ? v[0][j].y : v[0][j].x, e ? v[1][j].y : v[1][j].x, e ? v[2][j].y : v[2][j].x,
                                e ? v[3][j].y : v[3][j].x, e ? v[4][j].y : v[4][j].x, e ? v[5][j].y : v[5][j].x,
                                e ? v[6][j].y : v[6][j].x, e ? v[7][j].y : v[7][j].x};
            *reinterpret_cast<float4*>(p) = make_float4(r[0], r[1], r[2], r[3]);
            *reinterpret_cast<float4*>(p + 4) = make_float4(r[4], r[5], r[6], r[7]);
        }
}

// Row r's 8 values of the thread (two float4) to / from a row-major n x M array.
__device__ __forceinline__ void store_row(float* __restrict__ dst, int64_t r, const float2 (&v)[4], int lane) {
    float* p = dst + r * M;
    *reinterpret_cast<float4*>(p + 4 * lane) = make_float4(v[0].x, v[0].y, v[1].x, v[1].y);
    *reinterpret_cast<float4*>(p + 128 + 4 * lane) = make_float4(v[2].x, v[2].y, v[3].x, v[3].y);
}
__device__ __forceinline__ void load_row(const float* __restrict__ src, int64_t r, float2 (&v)[4], int lane) {
    const float* p = src + r * M;
    const float4 x = __ldg(reinterpret_cast<const float4*>(p + 4 * lane));
    const float4 y = __ldg(reinterpret_cast<const float4*>(p + 128 + 4 * lane));
    v[0] = make_float2(x.x, x.y);
    v[1] = make_float2(x.z, x.w);
    v[2] = make_float2(y.x, y.y);
    v[3] = make_float2(y.z, y.w);
}

// Sum over the warp's 32 lanes (all lanes get the sum), fixed order.
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// One MLP evaluation k = f(u) of the tile's rows, then
// unext = x + a*k (when unext != NULL) and acc = (init ? x : acc) + w*k.
// store (when not NULL): Z1, H1, Z2, H2, Z3, H3 at store + a*astride,
// each n x M row-major.
__global__ void __launch_bounds__(THREADS, 2)
    k_mlp_fwd(const float* __restrict__ u, const float* __restrict__ x, int64_t n, const float* __restrict__ W1,
              const float* __restrict__ b1, const float* __restrict__ W2T, const float* __restrict__ b2,
              const float* __restrict__ W3T, const float* __restrict__ b3, const float* __restrict__ W4,
              const float* __restrict__ b4, float a, float wgt, int init_acc, float* __restrict__ unext,
              float* __restrict__ accum, float* __restrict__ store, int64_t astride) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem& S = *reinterpret_cast<Smem*>(smem_raw);
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    const int64_t row0 = (int64_t)blockIdx.x * BM + 8 * w;
    float2 v[8][4];
    // input layer: z1 = u W1^T + b1 (fma order of the 3 terms: x, y, z)
    {
        float ux[8], uy[8], uz[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int64_t r = row0 + i;
            ux[i] = r < n ? __ldg(u + 3 * r) : 0.f;
            uy[i] = r < n ? __ldg(u + 3 * r + 1) : 0.f;
            uz[i] = r < n ? __ldg(u + 3 * r + 2) : 0.f;
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int c = col_of(lane, j, e);
                const float w0 = __ldg(W1 + 3 * c), w1 = __ldg(W1 + 3 * c + 1), w2 = __ldg(W1 + 3 * c + 2);
                const float bc = __ldg(b1 + c);
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const float z = fmaf(uz[i], w2, fmaf(uy[i], w1, fmaf(ux[i], w0, bc)));
                    if (e) v[i][j].y = z; else v[i][j].x = z;
                }
            }
    }
#pragma unroll
    for (int layer = 0; layer < 3; ++layer) {
        // v holds z of this layer: store z, h; h -> the tile
        if (layer > 0) {
            const float* b = layer == 1 ? b2 : b3;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float bx = __ldg(b + col_of(lane, j, 0)), by = __ldg(b + col_of(lane, j, 1));
#pragma unroll
                for (int i = 0; i < 8; ++i) v[i][j] = make_float2(v[i][j].x + bx, v[i][j].y + by);
            }
        }
        if (store) {
            float* Z = store + (2 * layer) * astride;
#pragma unroll
            for (int i = 0; i < 8; ++i)
                if (row0 + i < n) store_row(Z, row0 + i, v[i], lane);
        }
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) v[i][j] = make_float2(softplus(v[i][j].x), softplus(v[i][j].y));
        if (store) {
            float* H = store + (2 * layer + 1) * astride;
#pragma unroll
            for (int i = 0; i < 8; ++i)
                if (row0 + i < n) store_row(H, row0 + i, v[i], lane);
        }
        if (layer == 2) break;
        put_tile(S, v, w, lane);
        // (gemm_tile synchronises before its first read of the tile)
        zero_acc(v);
        gemm_tile(S, layer == 0 ? W2T : W3T, v, tid, w, lane);
    }
    // output layer: k = h3 W4^T + b4, summed over the warp's lanes
    float p[8][3];
#pragma unroll
    for (int i = 0; i < 8; ++i) p[i][0] = p[i][1] = p[i][2] = 0.f;
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const int c = col_of(lane, j, e);
            const float w0 = __ldg(W4 + c), w1 = __ldg(W4 + M + c), w2 = __ldg(W4 + 2 * M + c);
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const float h = e ? v[i][j].y : v[i][j].x;
                p[i][0] = fmaf(h, w0, p[i][0]);
                p[i][1] = fmaf(h, w1, p[i][1]);
                p[i][2] = fmaf(h, w2, p[i][2]);
            }
        }
    float mine[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const float s = warp_sum(p[i][d]);
            if (lane == i) mine[d] = s;
        }
    const int64_t r = row0 + lane;
    if (lane < 8 && r < n) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const float kv = mine[d] + __ldg(b4 + d);
            const int64_t q = 3 * r + d;
            if (unext) unext[q] = fmaf(a, kv, x[q]);
            accum[q] = fmaf(wgt, kv, init_acc ? x[q] : accum[q]);
        }
    }
}

// The vector-Jacobian product of one evaluation for the tile's rows (see the
// file comment).  store: Z1, H1, Z2, H2, Z3, H3 of the evaluation
// (k_mlp_fwd's layout).  gz3 / gz2: n x M outputs.  partial: one PW-float
// row per warp, at (blockIdx.x * 8 + warp).
__global__ void __launch_bounds__(THREADS, 2)
    k_mlp_bwd(const float* __restrict__ gk, const float* __restrict__ u, int64_t n, const float* __restrict__ W1,
              const float* __restrict__ W2, const float* __restrict__ W3, const float* __restrict__ W4,
              const float* __restrict__ store, int64_t astride, float* __restrict__ gz3, float* __restrict__ gz2,
              float* __restrict__ gu, float* __restrict__ partial) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem& S = *reinterpret_cast<Smem*>(smem_raw);
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    const int64_t row0 = (int64_t)blockIdx.x * BM + 8 * w;
    float* prow = partial + ((int64_t)blockIdx.x * 8 + w) * PW;
    const float* Z1 = store;
    const float* Z2 = store + 2 * astride;
    const float* Z3 = store + 4 * astride;
    const float* H3 = store + 5 * astride;
    float g[8][3];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int64_t r = row0 + i;
#pragma unroll
        for (int d = 0; d < 3; ++d) g[i][d] = r < n ? __ldg(gk + 3 * r + d) : 0.f;
    }
    float2 v[8][4];
    // g_z3 = (g W4) * sigmoid(z3); dW4 += g^T h3; db3 += g_z3; db4 += g
    {
        float dw4[3][8], db3[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) dw4[0][c] = dw4[1][c] = dw4[2][c] = db3[c] = 0.f;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int64_t r = row0 + i;
            float2 z[4], h[4];
            if (r < n) {
                load_row(Z3, r, z, lane);
                load_row(H3, r, h, lane);
            } else {
#pragma unroll
                for (int j = 0; j < 4; ++j) z[j] = h[j] = make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j)
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    const int c = col_of(lane, j, e);
                    const float gh = fmaf(g[i][2], __ldg(W4 + 2 * M + c),
                                          fmaf(g[i][1], __ldg(W4 + M + c), g[i][0] * __ldg(W4 + c)));
                    const float zz = e ? z[j].y : z[j].x, hh = e ? h[j].y : h[j].x;
                    const float gz = gh * sigmoid(zz);
                    if (e) v[i][j].y = gz; else v[i][j].x = gz;
                    const int cc = 2 * j + e;
                    dw4[0][cc] = fmaf(g[i][0], hh, dw4[0][cc]);
                    dw4[1][cc] = fmaf(g[i][1], hh, dw4[1][cc]);
                    dw4[2][cc] = fmaf(g[i][2], hh, dw4[2][cc]);
                    db3[cc] += gz;
                }
            if (r < n) store_row(gz3, r, v[i], lane);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int c = col_of(lane, j, e), cc = 2 * j + e;
                prow[P_DW4 + c] = dw4[0][cc];
                prow[P_DW4 + M + c] = dw4[1][cc];
                prow[P_DW4 + 2 * M + c] = dw4[2][cc];
                prow[P_DB3 + c] = db3[cc];
            }
        if (lane == 0) {
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                float s = 0.f;
#pragma unroll
                for (int i = 0; i < 8; ++i) s += g[i][d];
                prow[P_DB4 + d] = s;
            }
            prow[P_DB4 + 3] = 0.f;
        }
    }
    // two hidden layers back: g_z2 = (g_z3 W3) * sigmoid(z2), then
    // g_z1 = (g_z2 W2) * sigmoid(z1)
#pragma unroll
    for (int l = 0; l < 2; ++l) {
        put_tile(S, v, w, lane);
        zero_acc(v);
        gemm_tile(S, l == 0 ? W3 : W2, v, tid, w, lane);
        float db[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) db[c] = 0.f;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int64_t r = row0 + i;
            float2 z[4];
            if (r < n) {
                load_row(l == 0 ? Z2 : Z1, r, z, lane);
            } else {
#pragma unroll
                for (int j = 0; j < 4; ++j) z[j] = make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                v[i][j] = make_float2(v[i][j].x * sigmoid(z[j].x), v[i][j].y * sigmoid(z[j].y));
                db[2 * j] += v[i][j].x;
                db[2 * j + 1] += v[i][j].y;
            }
            if (l == 0 && r < n) store_row(gz2, r, v[i], lane);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int e = 0; e < 2; ++e) prow[(l == 0 ? P_DB2 : P_DB1) + col_of(lane, j, e)] = db[2 * j + e];
    }
    // v = g_z1: dW1 += g_z1^T u, g_u = g_z1 W1
    {
        float ux[8], uy[8], uz[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int64_t r = row0 + i;
            ux[i] = r < n ? __ldg(u + 3 * r) : 0.f;
            uy[i] = r < n ? __ldg(u + 3 * r + 1) : 0.f;
            uz[i] = r < n ? __ldg(u + 3 * r + 2) : 0.f;
        }
        float p[8][3];
#pragma unroll
        for (int i = 0; i < 8; ++i) p[i][0] = p[i][1] = p[i][2] = 0.f;
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int c = col_of(lane, j, e);
                const float w0 = __ldg(W1 + 3 * c), w1 = __ldg(W1 + 3 * c + 1), w2 = __ldg(W1 + 3 * c + 2);
                float d0 = 0.f, d1 = 0.f, d2 = 0.f;
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const float gz = e ? v[i][j].y : v[i][j].x;
                    p[i][0] = fmaf(gz, w0, p[i][0]);
                    p[i][1] = fmaf(gz, w1, p[i][1]);
                    p[i][2] = fmaf(gz, w2, p[i][2]);
                    d0 = fmaf(gz, ux[i], d0);
                    d1 = fmaf(gz, uy[i], d1);
                    d2 = fmaf(gz, uz[i], d2);
                }
                prow[P_DW1 + 3 * c] = d0;
                prow[P_DW1 + 3 * c + 1] = d1;
                prow[P_DW1 + 3 * c + 2] = d2;
            }
        float mine[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const float s = warp_sum(p[i][d]);
                if (lane == i) mine[d] = s;
            }
        const int64_t r = row0 + lane;
        if (lane < 8 && r < n) {
#pragma unroll
            for (int d = 0; d < 3; ++d) gu[3 * r + d] = mine[d];
        }
    }
}

// The small gradients, in two passes with a fixed order: pass 1 sums the
// rows of group blockIdx.y into mid[blockIdx.y][p]; pass 2 adds the groups'
// sums, in group order, into the gradients.
constexpr int RED_GROUPS = 128;
__global__ void k_mlp_partial_sum(const float* __restrict__ partial, int64_t rows, int64_t rows_per_group,
                                  float* __restrict__ mid) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= PW) return;
    const int64_t t0 = (int64_t)blockIdx.y * rows_per_group;
    const int64_t t1 = min(rows, t0 + rows_per_group);
    float s = 0.f;
    for (int64_t t = t0; t < t1; ++t) s += partial[t * PW + p];
    mid[(int64_t)blockIdx.y * PW + p] = s;
}

__global__ void k_mlp_partial_reduce(const float* __restrict__ mid, int groups, float* __restrict__ dW4,
                                     float* __restrict__ db4, float* __restrict__ db3, float* __restrict__ db2,
                                     float* __restrict__ db1, float* __restrict__ dW1) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= PW) return;
    float s = 0.f;
    for (int g = 0; g < groups; ++g) s += mid[(int64_t)g * PW + p];
    if (p < P_DB4) {
        dW4[p] += s;  // [3][M] as stored
    } else if (p < P_DB3) {
        if (p - P_DB4 < 3) db4[p - P_DB4] += s;
    } else if (p < P_DB2) {
        db3[p - P_DB3] += s;
    } else if (p < P_DB1) {
        db2[p - P_DB2] += s;
    } else if (p < P_DW1) {
        db1[p - P_DB1] += s;
    } else {
        dW1[p - P_DW1] += s;  // [M][3]
    }
}

// C[o][i] = sum over rows r in this CTA's range of A[r][o] * B[r][i], for
// the 128 x 128 block (blockIdx.x / 2, blockIdx.x % 2); written to
// partial[blockIdx.y][o][i].
constexpr int WG_T = 128, WG_K = 16;
__global__ void __launch_bounds__(THREADS, 2)
    k_mlp_wgrad(const float* __restrict__ A, const float* __restrict__ B, int64_t rows, int64_t rows_per_split,
                float* __restrict__ partial) {
    __shared__ __align__(16) float as[2][WG_K * WG_T];
    __shared__ __align__(16) float bs[2][WG_K * WG_T];
    const int tid = threadIdx.x;
    const int o0 = (blockIdx.x >> 1) * WG_T, i0 = (blockIdx.x & 1) * WG_T;
    const int64_t r_begin = (int64_t)blockIdx.y * rows_per_split;
    const int64_t r_end = min(rows, r_begin + rows_per_split);
    const int to = tid >> 4, ti = tid & 15;
    float2 acc[8][4];
    zero_acc(acc);
    const int nchunks = r_begin < r_end ? (int)((r_end - r_begin + WG_K - 1) / WG_K) : 0;
    auto load = [&](int c, int buf) {
#pragma unroll
        for (int j = 0; j < WG_K * WG_T / 4 / THREADS; ++j) {
            const int f = tid + j * THREADS;
            const int rr = f / (WG_T / 4), c4 = f % (WG_T / 4);
            const int64_t r = r_begin + (int64_t)c * WG_K + rr;
            const bool ok = r < r_end;
            const int64_t rs = ok ? r : r_begin;  // any valid address when the copy is skipped
            cp_async16_zfill(&as[buf][rr * WG_T + 4 * c4], A + rs * M + o0 + 4 * c4, ok);
            cp_async16_zfill(&bs[buf][rr * WG_T + 4 * c4], B + rs * M + i0 + 4 * c4, ok);
        }
    };
    if (nchunks > 0) {
        load(0, 0);
        cp_async_commit();
    }
#pragma unroll 1
    for (int c = 0; c < nchunks; ++c) {
        if (c + 1 < nchunks) {
            load(c + 1, (c + 1) & 1);
            cp_async_commit();
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const float* ab = as[c & 1];
        const float* bb_ = bs[c & 1];
#pragma unroll
        for (int k = 0; k < WG_K; ++k) {
            const float4 a0 = *reinterpret_cast<const float4*>(ab + k * WG_T + 4 * to);
            const float4 a1 = *reinterpret_cast<const float4*>(ab + k * WG_T + 64 + 4 * to);
            const float4 b0 = *reinterpret_cast<const float4*>(bb_ + k * WG_T + 4 * ti);
            const float4 b1 = *reinterpret_cast<const float4*>(bb_ + k * WG_T + 64 + 4 * ti);
            const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float2 bv[4] = {make_float2(b0.x, b0.y), make_float2(b0.z, b0.w), make_float2(b1.x, b1.y),
                                  make_float2(b1.z, b1.w)};
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const float2 ai = make_float2(av[i], av[i]);
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = __ffma2_rn(ai, bv[j], acc[i][j]);
            }
        }
        __syncthreads();
    }
    float* out = partial + (int64_t)blockIdx.y * M * M;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int o = o0 + (i < 4 ? 4 * to + i : 64 + 4 * to + (i - 4));
        float* p = out + (int64_t)o * M + i0;
        *reinterpret_cast<float4*>(p + 4 * ti) = make_float4(acc[i][0].x, acc[i][0].y, acc[i][1].x, acc[i][1].y);
        *reinterpret_cast<float4*>(p + 64 + 4 * ti) = make_float4(acc[i][2].x, acc[i][2].y, acc[i][3].x, acc[i][3].y);
    }
}

// dW[e] += sum over splits s (in order) of partial[s][e].
__global__ void k_mlp_wgrad_reduce(const float* __restrict__ partial, int splits, float* __restrict__ dW) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= M * M) return;
    float s = 0.f;
    for (int k = 0; k < splits; ++k) s += partial[(int64_t)k * M * M + e];
    dW[e] += s;
}

__global__ void k_transpose_m(const float* __restrict__ W, float* __restrict__ WT) {
    __shared__ float t[32][33];
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += 8) t[k][threadIdx.x] = W[(by + k) * M + bx + threadIdx.x];
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += 8) WT[(bx + k) * M + by + threadIdx.x] = t[threadIdx.x][k];
}

}  // namespace mlp
}  // namespace mo

using namespace mo;
using namespace mo::mlp;

static bool g_mlp_attr_done = false;

static int mlp_attrs() {
    if (g_mlp_attr_done) return MO_OK;
    MO_CUDA(cudaFuncSetAttribute(k_mlp_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES));
    MO_CUDA(cudaFuncSetAttribute(k_mlp_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES));
    g_mlp_attr_done = true;
    return MO_OK;
}

extern "C" int mo_mlp_width(void) { return M; }
extern "C" int64_t mo_mlp_tiles(int64_t n) { return n < 0 ? -1 : (n + BM - 1) / BM; }
extern "C" int mo_mlp_partial_floats(void) { return PW; }

extern "C" int mo_mlp_transpose(const float* W, float* WT, void* stream) {
    MO_CHECK_ARG(W && WT && W != WT, "null or aliased pointer");
    k_transpose_m<<<dim3(M / 32, M / 32), dim3(32, 8), 0, as_stream(stream)>>>(W, WT); ::mo::note_launch();
    MO_LAUNCH_CHECK("k_transpose_m");
    return MO_OK;
}

extern "C" int mo_mlp_fwd(const float* u, const float* x, int64_t n, const float* W1, const float* b1,
                          const float* W2T, const float* b2, const float* W3T, const float* b3, const float* W4,
                          const float* b4, float a, float w, int init_acc, float* unext, float* acc, float* store,
                          int64_t astride, void* stream) {
    MO_CHECK_ARG(n >= 0 && n < ((int64_t)1 << 31), "bad row count %lld", (long long)n);
    if (n == 0) return MO_OK;
    MO_CHECK_ARG(u && x && W1 && b1 && W2T && b2 && W3T && b3 && W4 && b4 && acc, "null pointer");
    MO_CHECK_ARG(aligned(W2T, 16) && aligned(W3T, 16), "weights must be 16-byte aligned");
    MO_CHECK_ARG(!store || (aligned(store, 16) && astride >= n * M && astride % 4 == 0),
                 "store must be 16-byte aligned with an array stride >= n*%d", M);
    int rc = mlp_attrs();
    if (rc) return rc;
    k_mlp_fwd<<<(unsigned)mo_mlp_tiles(n), THREADS, SMEM_BYTES, as_stream(stream)>>>(
        u, x, n, W1, b1, W2T, b2, W3T, b3, W4, b4, a, w, init_acc, unext, acc, store, astride);
    ::mo::note_launch();
    MO_LAUNCH_CHECK("k_mlp_fwd");
    return MO_OK;
}

extern "C" int mo_mlp_bwd(const float* gk, const float* u, int64_t n, const float* W1, const float* W2,
                          const float* W3, const float* W4, const float* store, int64_t astride, float* gz3,
                          float* gz2, float* gu, float* partial, void* stream) {
    MO_CHECK_ARG(n >= 0 && n < ((int64_t)1 << 31), "bad row count %lld", (long long)n);
    if (n == 0) return MO_OK;
    MO_CHECK_ARG(gk && u && W1 && W2 && W3 && W4 && store && gz3 && gz2 && gu && partial, "null pointer");
    MO_CHECK_ARG(aligned(W2, 16) && aligned(W3, 16) && aligned(store, 16) && aligned(gz3, 16) && aligned(gz2, 16),
                 "weights, stored activations and gradients must be 16-byte aligned");
    MO_CHECK_ARG(astride >= n * M && astride % 4 == 0, "array stride must be >= n*%d", M);
    int rc = mlp_attrs();
    if (rc) return rc;
    k_mlp_bwd<<<(unsigned)mo_mlp_tiles(n), THREADS, SMEM_BYTES, as_stream(stream)>>>(
        gk, u, n, W1, W2, W3, W4, store, astride, gz3, gz2, gu, partial);
    ::mo::note_launch();
    MO_LAUNCH_CHECK("k_mlp_bwd");
    return MO_OK;
}

extern "C" size_t mo_mlp_partial_reduce_bytes(void) { return (size_t)RED_GROUPS * PW * sizeof(float); }

extern "C" int mo_mlp_partial_reduce(const float* partial, int64_t rows, float* scratch, float* dW4, float* db4,
                                     float* db3, float* db2, float* db1, float* dW1, void* stream) {
    MO_CHECK_ARG(rows >= 0, "negative row count");
    if (rows == 0) return MO_OK;
    MO_CHECK_ARG(partial && scratch && dW4 && db4 && db3 && db2 && db1 && dW1, "null pointer");
    const int64_t per = (rows + RED_GROUPS - 1) / RED_GROUPS;
    const int groups = (int)((rows + per - 1) / per);
    cudaStream_t s = as_stream(stream);
    k_mlp_partial_sum<<<dim3(ceil_div(PW, 128), groups), 128, 0, s>>>(partial, rows, per, scratch);
    ::mo::note_launch();
    MO_LAUNCH_CHECK("k_mlp_partial_sum");
    k_mlp_partial_reduce<<<ceil_div(PW, 256), 256, 0, s>>>(scratch, groups, dW4, db4, db3, db2, db1, dW1);
    ::mo::note_launch();
    MO_LAUNCH_CHECK("k_mlp_partial_reduce");
    return MO_OK;
}

extern "C" size_t mo_mlp_wgrad_partial_bytes(int splits) { return splits > 0 ? (size_t)splits * M * M * 4 : 0; }

extern "C" int mo_mlp_wgrad(const float* A, const float* B, int64_t rows, int splits, float* partial, float* dW,
                            void* stream) {
    MO_CHECK_ARG(rows >= 0 && splits >= 1 && splits <= 65535, "bad rows or splits");
    MO_CHECK_ARG(A && B && partial && dW, "null pointer");
    MO_CHECK_ARG(aligned(A, 16) && aligned(B, 16) && aligned(partial, 16), "arrays must be 16-byte aligned");
    if (rows == 0) return MO_OK;
    const int64_t per = ((rows + splits - 1) / splits + WG_K - 1) / WG_K * WG_K;
    k_mlp_wgrad<<<dim3(4, splits), THREADS, 0, as_stream(stream)>>>(A, B, rows, per, partial); ::mo::note_launch();
    MO_LAUNCH_CHECK("k_mlp_wgrad");
    k_mlp_wgrad_reduce<<<M * M / 256, 256, 0, as_stream(stream)>>>(partial, splits, dW); ::mo::note_launch();
    MO_LAUNCH_CHECK("k_mlp_wgrad_reduce");
    return MO_OK;
}
