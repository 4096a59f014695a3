// Kernels of the velocity-field ODE deformation (the NeuralODE variant of
// src/python/layers/neuralode_fast.py:7-64, with a 3 -> m -> m -> m -> 3
// softplus MLP and fixed-step RK4).  The two m x m layers are plain GEMMs
// (cuBLAS through the caller); these kernels are everything around them:
// the 3-wide input layer with its bias and softplus, the bias + softplus
// epilogue, the 3-wide output layer fused with the RK4 stage update, and the
// matching backward pieces (softplus' = sigmoid).
#include "mo_common.cuh"

namespace mo {

// torch.nn.functional.softplus with beta = 1, threshold = 20.
__device__ __forceinline__ float softplus(float z) { return z > 20.f ? z : log1pf(expf(z)); }
__device__ __forceinline__ float sigmoid(float z) { return 1.f / (1.f + expf(-z)); }

// z = x W1^T + b1, h = softplus(z); one thread per (row, unit).
__global__ void k_mlp_in(const float* __restrict__ x, int64_t n, const float* __restrict__ W1,
                         const float* __restrict__ b1, int m, float* __restrict__ z, float* __restrict__ h) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * m) return;
    const int64_t r = i / m;
    const int j = (int)(i - r * m);
    const float v = fmaf(x[3 * r + 2], W1[3 * j + 2], fmaf(x[3 * r + 1], W1[3 * j + 1], fmaf(x[3 * r], W1[3 * j], b1[j])));
    if (z) z[i] = v;
    h[i] = softplus(v);
}

__global__ void k_bias_softplus(float* __restrict__ z, int64_t count, int m, const float* __restrict__ b,
                                float* __restrict__ h) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float v = z[i] + b[i % m];
    z[i] = v;
    h[i] = softplus(v);
}

// k = h W4^T + b4 (one warp per row, lanes over m); then
// u = x + a*k (next stage input) and acc = (init ? x : acc) + w*k.
__global__ void __launch_bounds__(256) k_mlp_out_rk4(const float* __restrict__ h, int64_t n, int m,
                                                     const float* __restrict__ W4, const float* __restrict__ b4,
                                                     const float* __restrict__ x, float a, float w, int init_acc,
                                                     float* __restrict__ k, float* __restrict__ u,
                                                     float* __restrict__ acc) {
    const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= n) return;
    const float* hr = h + r * m;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f;
    for (int j = lane; j < m; j += 32) {
        const float v = hr[j];
        s0 = fmaf(v, W4[j], s0);
        s1 = fmaf(v, W4[m + j], s1);
        s2 = fmaf(v, W4[2 * m + j], s2);
    }
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if (lane < 3) {
        const float kv = (lane == 0 ? s0 : lane == 1 ? s1 : s2) + b4[lane];
        const int64_t q = 3 * r + lane;
        if (k) k[q] = kv;
        if (u) u[q] = fmaf(a, kv, x[q]);
        if (acc) acc[q] = fmaf(w, kv, init_acc ? x[q] : acc[q]);
    }
}

// g_z = (g_out W4) * sigmoid(z); one thread per (row, unit).
__global__ void k_mlp_out_bwd(const float* __restrict__ g_out, int64_t n, int m, const float* __restrict__ W4,
                              const float* __restrict__ z, float* __restrict__ g_z) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * m) return;
    const int64_t r = i / m;
    const int j = (int)(i - r * m);
    const float g = fmaf(g_out[3 * r + 2], W4[2 * m + j], fmaf(g_out[3 * r + 1], W4[m + j], g_out[3 * r] * W4[j]));
    g_z[i] = g * sigmoid(z[i]);
}

__global__ void k_softplus_bwd(float* __restrict__ g, const float* __restrict__ z, int64_t count) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) g[i] *= sigmoid(z[i]);
}

// g_x (+)= g_z W1 (g_z [n,m], W1 [m,3]); one warp per row.
__global__ void __launch_bounds__(256) k_mlp_in_bwd(const float* __restrict__ g_z, int64_t n, int m,
                                                    const float* __restrict__ W1, float* __restrict__ g_x,
                                                    int accumulate) {
    const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= n) return;
    const float* gr = g_z + r * m;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f;
    for (int j = lane; j < m; j += 32) {
        const float v = gr[j];
        s0 = fmaf(v, W1[3 * j], s0);
        s1 = fmaf(v, W1[3 * j + 1], s1);
        s2 = fmaf(v, W1[3 * j + 2], s2);
    }
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if (lane < 3) {
        const float v = lane == 0 ? s0 : lane == 1 ? s1 : s2;
        g_x[3 * r + lane] = accumulate ? g_x[3 * r + lane] + v : v;
    }
}

}  // namespace mo

using namespace mo;

static int check_mlp(int64_t n, int m) {
    MO_CHECK_ARG(n >= 0 && m > 0, "bad MLP sizes (n=%lld, m=%d)", (long long)n, m);
    MO_CHECK_ARG(n * (int64_t)m < ((int64_t)1 << 40), "MLP activation too large");
    return MO_OK;
}

extern "C" int mo_mlp_in(const float* x, int64_t n, const float* W1, const float* b1, int m, float* z, float* h,
                         void* stream) {
    int rc = check_mlp(n, m);
    if (rc) return rc;
    if (n == 0) return MO_OK;
    MO_CHECK_ARG(x && W1 && b1 && h, "null pointer");
    k_mlp_in<<<ceil_div(n * m, 256), 256, 0, as_stream(stream)>>>(x, n, W1, b1, m, z, h); ::mo::note_launch();
    MO_LAUNCH_CHECK("k_mlp_in");
    return MO_OK;
}

extern "C" int mo_bias_softplus(float* z, int64_t n, int m, const float* b, float* h, void* stream) {
    int rc = check_mlp(n, m);
    if (rc) return rc;
    if (n == 0) return MO_OK;
    MO_CHECK_ARG(z && b && h, "null pointer");
    k_bias_softplus<<<ceil_div(n * m, 256), 256, 0, as_stream(stream)>>>(z, n * m, m, b, h); ::mo::note_launch();
    MO_LAUNCH_CHECK("k_bias_softplus");
    return MO_OK;
}

extern "C" int mo_mlp_out_rk4(const float* h, int64_t n, int m, const float* W4, const float* b4, const float* x,
                              float a, float w, int init_acc, float* k, float* u, float* acc, void* stream) {
    int rc = check_mlp(n, m);
    if (rc) return rc;
    if (n == 0) return MO_OK;
    MO_CHECK_ARG(h && W4 && b4, "null pointer");
    MO_CHECK_ARG((!u && !acc) || x, "x needed for the stage update");
    k_mlp_out_rk4<<<ceil_div(n * 32, 256), 256, 0, as_stream(stream)>>>(h, n, m, W4, b4, x, a, w, init_acc, k, u,
                                                                      acc); ::mo::note_launch();
    MO_LAUNCH_CHECK("k_mlp_out_rk4");
    return MO_OK;
}

extern "C" int mo_mlp_out_bwd(const float* g_out, int64_t n, int m, const float* W4, const float* z, float* g_z,
                              void* stream) {
    int rc = check_mlp(n, m);
    if (rc) return rc;
    if (n == 0) return MO_OK;
    MO_CHECK_ARG(g_out && W4 && z && g_z, "null pointer");
    k_mlp_out_bwd<<<ceil_div(n * m, 256), 256, 0, as_stream(stream)>>>(g_out, n, m, W4, z, g_z); ::mo::note_launch();
    MO_LAUNCH_CHECK("k_mlp_out_bwd");
    return MO_OK;
}

extern "C" int mo_softplus_bwd(float* g, const float* z, int64_t count, void* stream) {
    MO_CHECK_ARG(count >= 0, "negative size");
    if (count == 0) return MO_OK;
    MO_CHECK_ARG(g && z, "null pointer");
    k_softplus_bwd<<<ceil_div(count, 256), 256, 0, as_stream(stream)>>>(g, z, count); ::mo::note_launch();
    MO_LAUNCH_CHECK("k_softplus_bwd");
    return MO_OK;
}

extern "C" int mo_mlp_in_bwd(const float* g_z, int64_t n, int m, const float* W1, float* g_x, int accumulate,
                             void* stream) {
    int rc = check_mlp(n, m);
    if (rc) return rc;
    if (n == 0) return MO_OK;
    MO_CHECK_ARG(g_z && W1 && g_x, "null pointer");
    k_mlp_in_bwd<<<ceil_div(n * 32, 256), 256, 0, as_stream(stream)>>>(g_z, n, m, W1, g_x, accumulate);
    ::mo::note_launch();
    MO_LAUNCH_CHECK("k_mlp_in_bwd");
    return MO_OK;
}
