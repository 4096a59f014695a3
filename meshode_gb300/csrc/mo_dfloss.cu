// DistanceFieldLoss forward / backward kernels (one thread per vertex) and the
// grid relayout.  Reference: src/interface/distance_layer.cc:8-81.
#include "mo_df_eval.cuh"

namespace mo {

static inline float far_offset(int N) { return (float)((double)(N - 1) - 1e-3); }

template <int LAYOUT, bool FWD, bool BWD>
__global__ void __launch_bounds__(256) k_dfloss(const float* __restrict__ V, int64_t n,
                                                const float* __restrict__ grid, int N, float Nf, float Cf,
                                                float* __restrict__ loss, float* __restrict__ grad,
                                                int use_mask, float mask_thresh) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x = V[3 * i], y = V[3 * i + 1], z = V[3 * i + 2];
    const DFJet j = df_eval<LAYOUT, BWD>(grid, N, Nf, Cf, x, y, z);
    const float dsq = MUL(j.d, j.d);  // distance_layer.cc:33
    if (FWD && loss) loss[i] = dsq;
    if (BWD) {
        float g0 = df_grad_component(j.d, j.gx);
        float g1 = df_grad_component(j.d, j.gy);
        float g2 = df_grad_component(j.d, j.gz);
        if (use_mask) {  // graph_loss_layer.py:18,40: grad *= (0.5*d^2 < thresh)
            const float m = (MUL(dsq, 0.5f) < mask_thresh) ? 1.0f : 0.0f;
            g0 = MUL(g0, m); g1 = MUL(g1, m); g2 = MUL(g2, m);
        }
        grad[3 * i] = g0; grad[3 * i + 1] = g1; grad[3 * i + 2] = g2;
    }
}

template <bool FWD, bool BWD>
static int launch_dfloss(const float* V, int64_t n, const float* grid, int N, int layout, float* loss,
                         float* grad, int use_mask, float mask_thresh, cudaStream_t s) {
    MO_CHECK_ARG(n >= 0, "negative vertex count");
    MO_CHECK_ARG(N >= 2, "grid resolution must be >= 2 (got %d)", N);
    MO_CHECK_ARG(layout == MO_LAYOUT_LINEAR || layout == MO_LAYOUT_CELL || layout == MO_LAYOUT_BRICK4,
                 "unknown grid layout %d", layout);
    MO_CHECK_ARG(n == 0 || (V && grid), "null vertex or grid pointer");
    MO_CHECK_ARG(!BWD || n == 0 || grad, "null gradient pointer");
    MO_CHECK_ARG(layout != MO_LAYOUT_CELL || aligned(grid, 16), "cell-layout grid must be 16-byte aligned");
    MO_CHECK_ARG(layout != MO_LAYOUT_BRICK4 || N <= 1280, "brick layout supports N <= 1280");
    if (n == 0) return MO_OK;
    const int threads = 256;
    const int blocks = ceil_div(n, threads);
    const float Nf = (float)N, Cf = far_offset(N);
    if (layout == MO_LAYOUT_CELL) {
        k_dfloss<MO_LAYOUT_CELL, FWD, BWD><<<blocks, threads, 0, s>>>(V, n, grid, N, Nf, Cf, loss, grad,
                                                                      use_mask, mask_thresh);
    } else if (layout == MO_LAYOUT_BRICK4) {
        k_dfloss<MO_LAYOUT_BRICK4, FWD, BWD><<<blocks, threads, 0, s>>>(V, n, grid, N, Nf, Cf, loss, grad,
                                                                        use_mask, mask_thresh);
    } else {
        k_dfloss<MO_LAYOUT_LINEAR, FWD, BWD><<<blocks, threads, 0, s>>>(V, n, grid, N, Nf, Cf, loss, grad,
                                                                        use_mask, mask_thresh);
    }
    ::mo::note_launch();
    MO_LAUNCH_CHECK("k_dfloss");
    return MO_OK;
}

// Linear [z][y][x] -> 4x4x4 bricks (padding voxels hold 0; they are never read).
__global__ void __launch_bounds__(256) k_relayout_brick4(const float* __restrict__ g, int N, float* __restrict__ out) {
    const int nb = (N + 3) >> 2, P = nb * 4;
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= (int64_t)P * P * P) return;
    const int x = (int)(v % P), y = (int)((v / P) % P), z = (int)(v / ((int64_t)P * P));
    const int64_t b = ((int64_t)(z >> 2) * nb + (y >> 2)) * nb + (x >> 2);
    const float val = (x < N && y < N && z < N) ? g[((int64_t)z * N + y) * N + x] : 0.f;
    out[b * 64 + (((z & 3) * 4 + (y & 3)) * 4 + (x & 3))] = val;
}

// Linear [z][y][x] -> per-cell 8 corners (k = (bz<<2)|(by<<1)|bx).
__global__ void __launch_bounds__(256) k_relayout_cell(const float* __restrict__ g, int N,
                                                       float4* __restrict__ out) {
    const int M = N - 1;
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (int64_t)M * M * M) return;
    const int x = (int)(c % M), y = (int)((c / M) % M), z = (int)(c / ((int64_t)M * M));
    const int64_t b = ((int64_t)z * N + y) * N + x, sy = N, sz = (int64_t)N * N;
    out[2 * c] = make_float4(g[b], g[b + 1], g[b + sy], g[b + sy + 1]);
    out[2 * c + 1] = make_float4(g[b + sz], g[b + sz + 1], g[b + sz + sy], g[b + sz + sy + 1]);
}

}  // namespace mo

using namespace mo;

extern "C" int mo_dfloss_forward(const float* V, int64_t n, const float* grid, int N, int layout,
                                 float* loss_out, void* stream) {
    MO_CHECK_ARG(n == 0 || loss_out, "null loss pointer");
    return launch_dfloss<true, false>(V, n, grid, N, layout, loss_out, nullptr, 0, 0.f, as_stream(stream));
}

extern "C" int mo_dfloss_backward(const float* V, int64_t n, const float* grid, int N, int layout,
                                  float* grad_out, void* stream) {
    return launch_dfloss<false, true>(V, n, grid, N, layout, nullptr, grad_out, 0, 0.f, as_stream(stream));
}

extern "C" int mo_dfloss_fwd_bwd(const float* V, int64_t n, const float* grid, int N, int layout,
                                 float* loss_out, float* grad_out, int use_mask, float mask_thresh,
                                 void* stream) {
    return launch_dfloss<true, true>(V, n, grid, N, layout, loss_out, grad_out, use_mask, mask_thresh,
                                     as_stream(stream));
}

extern "C" size_t mo_grid_bytes(int N, int layout) {
    if (N < 2) return 0;
    if (layout == MO_LAYOUT_LINEAR) return (size_t)N * N * N * sizeof(float);
    if (layout == MO_LAYOUT_CELL) return (size_t)(N - 1) * (N - 1) * (N - 1) * 8 * sizeof(float);
    if (layout == MO_LAYOUT_BRICK4) {
        const size_t nb = (size_t)(N + 3) / 4;
        return nb * nb * nb * 64 * sizeof(float);
    }
    return 0;
}

extern "C" int mo_grid_relayout(const float* grid_linear, int N, int layout, float* out, void* stream) {
    MO_CHECK_ARG(N >= 2, "grid resolution must be >= 2 (got %d)", N);
    MO_CHECK_ARG(grid_linear && out, "null grid pointer");
    cudaStream_t s = as_stream(stream);
    if (layout == MO_LAYOUT_LINEAR) {
        MO_CUDA(cudaMemcpyAsync(out, grid_linear, mo_grid_bytes(N, layout), cudaMemcpyDeviceToDevice, s));
        return MO_OK;
    }
    if (layout == MO_LAYOUT_BRICK4) {
        const int64_t P = (int64_t)((N + 3) / 4) * 4;
        k_relayout_brick4<<<ceil_div(P * P * P, 256), 256, 0, s>>>(grid_linear, N, out); ::mo::note_launch();
        MO_LAUNCH_CHECK("k_relayout_brick4");
        return MO_OK;
    }
    MO_CHECK_ARG(layout == MO_LAYOUT_CELL, "unknown grid layout %d", layout);
    MO_CHECK_ARG(aligned(out, 16), "cell-layout output must be 16-byte aligned");
    const int64_t M = N - 1, cells = M * M * M;
    k_relayout_cell<<<ceil_div(cells, 256), 256, 0, s>>>(grid_linear, N, reinterpret_cast<float4*>(out)); ::mo::note_launch();
    MO_LAUNCH_CHECK("k_relayout_cell");
    return MO_OK;
}
