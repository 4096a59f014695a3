// Edge (rigidity) losses: rest offsets, per-half-edge residuals, and the
// deterministic vertex->half-edge CSR used for the gradient scatter.
// Reference: src/interface/rigid_layer.cc:11-133, graph_layer.cc:11-135.
//
// CSR buffer layout (int32 words):
//   row_ptr[nv+1] | key[2H] | other[2H] | cursor[nv] | status[1] | pad
// key = 2*h + role, role 0 when the vertex is the half-edge's v0 (the
// reference's `g[v0] -= r`), 1 when it is v1 (`g[v1] += r`).  Rows are sorted
// by key, i.e. in the order the reference's serial loop touches the vertex.
#include <climits>

#include "mo_common.cuh"

namespace mo {

struct CsrView {
    int* row_ptr;
    int* key;
    int* other;
    int* cursor;
    int* status;
};

static inline CsrView csr_view(void* base, int64_t nv, int64_t nh) {
    CsrView v;
    int* p = reinterpret_cast<int*>(base);
    v.row_ptr = p;
    v.key = p + (nv + 1);
    v.other = v.key + 2 * nh;
    v.cursor = v.other + 2 * nh;
    v.status = v.cursor + nv;
    return v;
}

__device__ __forceinline__ void he_ends(const int32_t* __restrict__ idx, int kind, int64_t h, int& v0, int& v1) {
    if (kind == MO_EDGES_FACES) {
        const int64_t f = h / 3;
        const int j = (int)(h - 3 * f);
        v0 = idx[3 * f + j];
        v1 = idx[3 * f + (j == 2 ? 0 : j + 1)];
    } else {
        v0 = idx[2 * h];
        v1 = idx[2 * h + 1];
    }
}

__device__ __forceinline__ bool in_range(int v, int64_t nv) { return v >= 0 && (int64_t)v < nv; }

__global__ void k_edge_offsets(const float* __restrict__ V, int64_t nv, const int32_t* __restrict__ idx,
                               int64_t nh, int kind, float* __restrict__ off) {
    const int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= nh) return;
    int v0, v1;
    he_ends(idx, kind, h, v0, v1);
    if (!in_range(v0, nv) || !in_range(v1, nv)) {
        off[3 * h] = off[3 * h + 1] = off[3 * h + 2] = __int_as_float(0x7fc00000);
        return;
    }
    for (int c = 0; c < 3; ++c) off[3 * h + c] = SUB(V[3 * (int64_t)v1 + c], V[3 * (int64_t)v0 + c]);
}

__global__ void k_edge_forward(const float* __restrict__ V, int64_t nv, const int32_t* __restrict__ idx,
                               int64_t nh, int kind, const float* __restrict__ off, float* __restrict__ L) {
    const int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= nh) return;
    int v0, v1;
    he_ends(idx, kind, h, v0, v1);
    if (!in_range(v0, nv) || !in_range(v1, nv)) {
        L[3 * h] = L[3 * h + 1] = L[3 * h + 2] = __int_as_float(0x7fc00000);
        return;
    }
    for (int c = 0; c < 3; ++c) {
        const float r = SUB(SUB(V[3 * (int64_t)v1 + c], V[3 * (int64_t)v0 + c]), off[3 * h + c]);
        L[3 * h + c] = MUL(r, r);
    }
}

__global__ void k_csr_count(const int32_t* __restrict__ idx, int64_t nh, int kind, int64_t nv,
                            int* __restrict__ cnt, int* __restrict__ status) {
    const int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= nh) return;
    int v0, v1;
    he_ends(idx, kind, h, v0, v1);
    if (!in_range(v0, nv) || !in_range(v1, nv)) {
        atomicOr(status, 1);
        return;
    }
    atomicAdd(&cnt[v0], 1);
    atomicAdd(&cnt[v1], 1);
}

__global__ void k_csr_fill(const int32_t* __restrict__ idx, int64_t nh, int kind, int64_t nv,
                           const int* __restrict__ row_ptr, int* __restrict__ cursor, int* __restrict__ key,
                           int* __restrict__ other) {
    const int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= nh) return;
    int v0, v1;
    he_ends(idx, kind, h, v0, v1);
    if (!in_range(v0, nv) || !in_range(v1, nv)) return;
    int p0 = row_ptr[v0] + atomicAdd(&cursor[v0], 1);
    key[p0] = (int)(2 * h);
    other[p0] = v1;
    int p1 = row_ptr[v1] + atomicAdd(&cursor[v1], 1);
    key[p1] = (int)(2 * h + 1);
    other[p1] = v0;
}

// Rows are short (vertex degree); sorting each by key makes the order
// independent of the atomic fill order.  Keys are distinct (2h for the v0
// role of half-edge h, 2h+1 for v1, also when v0 == v1), so any sort gives
// the same row: rows of up to 16 go through a bitonic network in registers,
// longer ones an insertion sort in place.
constexpr int ROW_NET = 16;

__global__ void k_csr_sort_rows(int64_t nv, const int* __restrict__ row_ptr, int* __restrict__ key,
                                int* __restrict__ other) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    const int b = row_ptr[v], e = row_ptr[v + 1];
    if (e - b <= ROW_NET) {
        const int len = e - b;
        int k[ROW_NET], o[ROW_NET];
#pragma unroll
        for (int i = 0; i < ROW_NET; ++i) {
            k[i] = i < len ? key[b + i] : INT_MAX;  // padding sorts last
            o[i] = i < len ? other[b + i] : 0;
        }
#pragma unroll
        for (int w = 2; w <= ROW_NET; w <<= 1)
#pragma unroll
            for (int j = w >> 1; j > 0; j >>= 1)
#pragma unroll
                for (int i = 0; i < ROW_NET; ++i) {
                    const int l = i ^ j;
                    if (l > i) {
                        const bool up = (i & w) == 0;
                        if ((k[i] > k[l]) == up) {
                            const int tk = k[i], to = o[i];
                            k[i] = k[l]; o[i] = o[l];
                            k[l] = tk; o[l] = to;
                        }
                    }
                }
#pragma unroll
        for (int i = 0; i < ROW_NET; ++i)
            if (i < len) {
                key[b + i] = k[i];
                other[b + i] = o[i];
            }
        return;
    }
    for (int i = b + 1; i < e; ++i) {
        const int k = key[i], o = other[i];
        int j = i - 1;
        while (j >= b && key[j] > k) {
            key[j + 1] = key[j];
            other[j + 1] = other[j];
            --j;
        }
        key[j + 1] = k;
        other[j + 1] = o;
    }
}

// Per-vertex gradient in the reference's serial scatter order.
__global__ void __launch_bounds__(256) k_edge_backward(const float* __restrict__ V, int64_t nv,
                                                       const int* __restrict__ row_ptr,
                                                       const int* __restrict__ key,
                                                       const int* __restrict__ other,
                                                       const float* __restrict__ off, float* __restrict__ G) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const float px = V[3 * i], py = V[3 * i + 1], pz = V[3 * i + 2];
    float gx = 0.0f, gy = 0.0f, gz = 0.0f;
    const int b = row_ptr[i], e = row_ptr[i + 1];
    for (int k = b; k < e; ++k) {
        const int kk = key[k];
        const int64_t h = kk >> 1;
        const int64_t o = other[k];
        const float qx = V[3 * o], qy = V[3 * o + 1], qz = V[3 * o + 2];
        const float ox = off[3 * h], oy = off[3 * h + 1], oz = off[3 * h + 2];
        if ((kk & 1) == 0) {  // this vertex is v0: g[v0] -= (v1 - v0 - off)
            gx = SUB(gx, SUB(SUB(qx, px), ox));
            gy = SUB(gy, SUB(SUB(qy, py), oy));
            gz = SUB(gz, SUB(SUB(qz, pz), oz));
        } else {              // this vertex is v1: g[v1] += (v1 - v0 - off)
            gx = ADD(gx, SUB(SUB(px, qx), ox));
            gy = ADD(gy, SUB(SUB(py, qy), oy));
            gz = ADD(gz, SUB(SUB(pz, qz), oz));
        }
    }
    G[3 * i] = gx; G[3 * i + 1] = gy; G[3 * i + 2] = gz;
}

// ---------------------------------------------------------------------------
// Weighted edges (CadEdgeLoss, src/interface/cad_layer.cc:11-223).
//
// The CAD loss's edge set is E's edges followed by F's half-edges
// (cad_layer.cc:33-67, 108-143, 178-219), one rest offset and one weight
// lambda_e = 2e-2 / (|off_e| + 1e-8) each (:48-49, :71-72).  The forward is
// ((v1 - v0 - off) * lambda)^2 per component (:114-122); the backward
// scatters (v1 - v0 - off) * (lambda * lambda) (:195-202) in the same serial
// order as the unweighted loss.
// ---------------------------------------------------------------------------
__global__ void k_edge_cad_list(const int32_t* __restrict__ E, int64_t ne, const int32_t* __restrict__ F,
                                int64_t nf, int32_t* __restrict__ out) {
    const int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= ne + 3 * nf) return;
    int v0, v1;
    if (h < ne) {
        v0 = E[2 * h];
        v1 = E[2 * h + 1];
    } else {
        he_ends(F, MO_EDGES_FACES, h - ne, v0, v1);
    }
    out[2 * h] = v0;
    out[2 * h + 1] = v1;
}

// |off| is Eigen's float norm: sqrt of x*x + (y*y + z*z) (its unrolled
// pairwise sum of three terms); the +1e-8 and the quotient are double (the
// literals are double), rounded to float on the store.
__global__ void k_edge_cad_weights(const float* __restrict__ off, int64_t nh, float* __restrict__ lam) {
    const int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= nh) return;
    const float x = off[3 * h], y = off[3 * h + 1], z = off[3 * h + 2];
    const float n = __fsqrt_rn(ADD(MUL(x, x), ADD(MUL(y, y), MUL(z, z))));
    lam[h] = __double2float_rn(__ddiv_rn(2e-2, __dadd_rn((double)n, 1e-8)));
}

__global__ void k_edge_forward_w(const float* __restrict__ V, int64_t nv, const int32_t* __restrict__ idx,
                                 int64_t nh, int kind, const float* __restrict__ off, const float* __restrict__ w,
                                 float* __restrict__ L) {
    const int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= nh) return;
    int v0, v1;
    he_ends(idx, kind, h, v0, v1);
    if (!in_range(v0, nv) || !in_range(v1, nv)) {
        L[3 * h] = L[3 * h + 1] = L[3 * h + 2] = __int_as_float(0x7fc00000);
        return;
    }
    const float lam = w[h];
    for (int c = 0; c < 3; ++c) {
        const float r = MUL(SUB(SUB(V[3 * (int64_t)v1 + c], V[3 * (int64_t)v0 + c]), off[3 * h + c]), lam);
        L[3 * h + c] = MUL(r, r);
    }
}

__global__ void __launch_bounds__(256) k_edge_backward_w(const float* __restrict__ V, int64_t nv,
                                                         const int* __restrict__ row_ptr,
                                                         const int* __restrict__ key,
                                                         const int* __restrict__ other,
                                                         const float* __restrict__ off,
                                                         const float* __restrict__ w, float* __restrict__ G) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const float px = V[3 * i], py = V[3 * i + 1], pz = V[3 * i + 2];
    float gx = 0.0f, gy = 0.0f, gz = 0.0f;
    const int b = row_ptr[i], e = row_ptr[i + 1];
    for (int k = b; k < e; ++k) {
        const int kk = key[k];
        const int64_t h = kk >> 1;
        const int64_t o = other[k];
        const float qx = V[3 * o], qy = V[3 * o + 1], qz = V[3 * o + 2];
        const float ox = off[3 * h], oy = off[3 * h + 1], oz = off[3 * h + 2];
        const float l2 = MUL(w[h], w[h]);
        if ((kk & 1) == 0) {  // v0: g[v0] -= (v1 - v0 - off) * lambda^2
            gx = SUB(gx, MUL(SUB(SUB(qx, px), ox), l2));
            gy = SUB(gy, MUL(SUB(SUB(qy, py), oy), l2));
            gz = SUB(gz, MUL(SUB(SUB(qz, pz), oz), l2));
        } else {              // v1: g[v1] += (v1 - v0 - off) * lambda^2
            gx = ADD(gx, MUL(SUB(SUB(px, qx), ox), l2));
            gy = ADD(gy, MUL(SUB(SUB(py, qy), oy), l2));
            gz = ADD(gz, MUL(SUB(SUB(pz, qz), oz), l2));
        }
    }
    G[3 * i] = gx; G[3 * i + 1] = gy; G[3 * i + 2] = gz;
}

// Slice widths (max row length over 32 consecutive vertices), x32.
__global__ void k_sell_width(int64_t nv, int64_t nslices, const int* __restrict__ row_ptr,
                             int* __restrict__ slice_ptr) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t s = t >> 5;
    const int lane = threadIdx.x & 31;
    if (s >= nslices) return;  // whole warp exits together (blockDim multiple of 32)
    const int64_t v = s * 32 + lane;
    int deg = v < nv ? row_ptr[v + 1] - row_ptr[v] : 0;
    for (int o = 16; o > 0; o >>= 1) deg = max(deg, __shfl_xor_sync(0xffffffffu, deg, o));
    if (lane == 0) slice_ptr[s] = deg * 32;
}

__global__ void k_sell_fill(int64_t nv, int64_t nslices, const int* __restrict__ row_ptr,
                            const int* __restrict__ key, const int* __restrict__ other,
                            const int* __restrict__ slice_ptr, int* __restrict__ rec) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t s = t >> 5;
    const int lane = threadIdx.x & 31;
    if (s >= nslices) return;
    const int64_t v = s * 32 + lane;
    const int base = slice_ptr[s];
    const int w = (slice_ptr[s + 1] - base) >> 5;
    const int b = v < nv ? row_ptr[v] : 0;
    const int deg = v < nv ? row_ptr[v + 1] - b : 0;
    for (int k = 0; k < w; ++k)
        rec[base + (int64_t)k * 32 + lane] = (k < deg) ? (other[b + k] | ((key[b + k] & 1) << 31)) : -1;
}

// The weight of every sliced-ELL record (w[h] of the record's half-edge h),
// in the records' layout; padding 0.
__global__ void k_sell_fill_w(int64_t nv, int64_t nslices, const int* __restrict__ row_ptr,
                              const int* __restrict__ key, const int* __restrict__ slice_ptr,
                              const float* __restrict__ w, float* __restrict__ rec_w) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t s = t >> 5;
    const int lane = threadIdx.x & 31;
    if (s >= nslices) return;
    const int64_t v = s * 32 + lane;
    const int base = slice_ptr[s];
    const int width = (slice_ptr[s + 1] - base) >> 5;
    const int b = v < nv ? row_ptr[v] : 0;
    const int deg = v < nv ? row_ptr[v + 1] - b : 0;
    for (int k = 0; k < width; ++k) rec_w[base + (int64_t)k * 32 + lane] = (k < deg) ? w[key[b + k] >> 1] : 0.f;
}

}  // namespace mo

using namespace mo;

extern "C" int64_t mo_edge_count(int64_t n_items, int kind) {
    if (n_items < 0) return -1;
    if (kind == MO_EDGES_FACES) return 3 * n_items;
    if (kind == MO_EDGES_LIST) return n_items;
    return -1;
}

static int check_edges(const float* V, int64_t nv, const int32_t* idx, int64_t n_items, int kind,
                       int64_t* nh) {
    MO_CHECK_ARG(kind == MO_EDGES_FACES || kind == MO_EDGES_LIST, "unknown edge kind %d", kind);
    MO_CHECK_ARG(nv >= 0 && n_items >= 0, "negative size");
    MO_CHECK_ARG(nv < (int64_t)INT_MAX, "too many vertices (%lld)", (long long)nv);
    *nh = mo_edge_count(n_items, kind);
    MO_CHECK_ARG(*nh < ((int64_t)1 << 30), "too many half-edges (%lld)", (long long)*nh);
    MO_CHECK_ARG(*nh == 0 || (idx && V), "null vertex or index pointer");
    return MO_OK;
}

extern "C" int mo_edge_offsets(const float* V, int64_t nv, const int32_t* idx, int64_t n_items, int kind,
                               float* off_out, void* stream) {
    int64_t nh;
    int rc = check_edges(V, nv, idx, n_items, kind, &nh);
    if (rc) return rc;
    if (nh == 0) return MO_OK;
    MO_CHECK_ARG(off_out, "null output pointer");
    k_edge_offsets<<<ceil_div(nh, 256), 256, 0, as_stream(stream)>>>(V, nv, idx, nh, kind, off_out); ::mo::note_launch();
    MO_LAUNCH_CHECK("k_edge_offsets");
    return MO_OK;
}

extern "C" int mo_edge_forward(const float* V, int64_t nv, const int32_t* idx, int64_t n_items, int kind,
                               const float* off, float* loss_out, void* stream) {
    int64_t nh;
    int rc = check_edges(V, nv, idx, n_items, kind, &nh);
    if (rc) return rc;
    if (nh == 0) return MO_OK;
    MO_CHECK_ARG(off && loss_out, "null offset or output pointer");
    k_edge_forward<<<ceil_div(nh, 256), 256, 0, as_stream(stream)>>>(V, nv, idx, nh, kind, off, loss_out); ::mo::note_launch();
    MO_LAUNCH_CHECK("k_edge_forward");
    return MO_OK;
}

extern "C" size_t mo_edge_csr_bytes(int64_t nv, int64_t n_items, int kind) {
    const int64_t nh = mo_edge_count(n_items, kind);
    if (nh < 0 || nv < 0) return 0;
    return sizeof(int) * (size_t)((nv + 1) + 4 * nh + nv + 4);
}

extern "C" int mo_edge_csr_build(const int32_t* idx, int64_t n_items, int kind, int64_t nv, void* csr,
                                 size_t csr_bytes, int32_t* status_out, void* stream) {
    int64_t nh;
    int rc = check_edges(reinterpret_cast<const float*>(idx), nv, idx, n_items, kind, &nh);
    if (rc) return rc;
    MO_CHECK_ARG(csr, "null CSR buffer");
    if (csr_bytes < mo_edge_csr_bytes(nv, n_items, kind)) {
        set_error("CSR buffer too small: %zu < %zu", csr_bytes, mo_edge_csr_bytes(nv, n_items, kind));
        return MO_ERR_SCRATCH;
    }
    cudaStream_t s = as_stream(stream);
    CsrView c = csr_view(csr, nv, nh);
    MO_CUDA(cudaMemsetAsync(c.row_ptr, 0, sizeof(int) * (nv + 1), s));
    MO_CUDA(cudaMemsetAsync(c.cursor, 0, sizeof(int) * (nv + 1), s));  // cursor[nv] + status
    int* st = status_out ? reinterpret_cast<int*>(status_out) : c.status;
    if (nh > 0) {
        k_csr_count<<<ceil_div(nh, 256), 256, 0, s>>>(idx, nh, kind, nv, c.row_ptr, st); ::mo::note_launch();
        MO_LAUNCH_CHECK("k_csr_count");
    }
    MO_CUDA(exclusive_scan_i32(c.row_ptr, (int)(nv + 1), nullptr, s));
    if (nh > 0) {
        k_csr_fill<<<ceil_div(nh, 256), 256, 0, s>>>(idx, nh, kind, nv, c.row_ptr, c.cursor, c.key, c.other); ::mo::note_launch();
        MO_LAUNCH_CHECK("k_csr_fill");
    }
    if (nv > 0) {
        k_csr_sort_rows<<<ceil_div(nv, 256), 256, 0, s>>>(nv, c.row_ptr, c.key, c.other); ::mo::note_launch();
        MO_LAUNCH_CHECK("k_csr_sort_rows");
    }
    if (status_out) return MO_OK;
    int status = 0;
    MO_CUDA(cudaMemcpyAsync(&status, c.status, sizeof(int), cudaMemcpyDeviceToHost, s));
    MO_CUDA(cudaStreamSynchronize(s));
    if (status) {
        set_error("edge index out of range [0, %lld)", (long long)nv);
        return MO_ERR_DEVICE;
    }
    return MO_OK;
}

extern "C" int mo_edge_backward(const float* V, int64_t nv, const void* csr, int64_t nh, const float* off,
                                float* grad_out, void* stream) {
    MO_CHECK_ARG(nv >= 0 && nh >= 0, "negative size");
    if (nv == 0) return MO_OK;
    MO_CHECK_ARG(V && csr && grad_out && (nh == 0 || off), "null pointer");
    CsrView c = csr_view(const_cast<void*>(csr), nv, nh);
    k_edge_backward<<<ceil_div(nv, 256), 256, 0, as_stream(stream)>>>(V, nv, c.row_ptr, c.key, c.other, off,
                                                                      grad_out); ::mo::note_launch();
    MO_LAUNCH_CHECK("k_edge_backward");
    return MO_OK;
}

extern "C" int mo_edge_cad_list(const int32_t* E, int64_t ne, const int32_t* F, int64_t nf, int32_t* list_out,
                                void* stream) {
    MO_CHECK_ARG(ne >= 0 && nf >= 0, "negative size");
    const int64_t nh = ne + 3 * nf;
    MO_CHECK_ARG(nh < ((int64_t)1 << 30), "too many edges (%lld)", (long long)nh);
    if (nh == 0) return MO_OK;
    MO_CHECK_ARG((ne == 0 || E) && (nf == 0 || F) && list_out, "null pointer");
    k_edge_cad_list<<<ceil_div(nh, 256), 256, 0, as_stream(stream)>>>(E, ne, F, nf, list_out); ::mo::note_launch();
    MO_LAUNCH_CHECK("k_edge_cad_list");
    return MO_OK;
}

extern "C" int mo_edge_cad_weights(const float* off, int64_t nh, float* lambda_out, void* stream) {
    MO_CHECK_ARG(nh >= 0 && nh < ((int64_t)1 << 30), "bad edge count (%lld)", (long long)nh);
    if (nh == 0) return MO_OK;
    MO_CHECK_ARG(off && lambda_out, "null pointer");
    k_edge_cad_weights<<<ceil_div(nh, 256), 256, 0, as_stream(stream)>>>(off, nh, lambda_out); ::mo::note_launch();
    MO_LAUNCH_CHECK("k_edge_cad_weights");
    return MO_OK;
}

extern "C" int mo_edge_forward_w(const float* V, int64_t nv, const int32_t* idx, int64_t n_items, int kind,
                                 const float* off, const float* w, float* loss_out, void* stream) {
    if (!w) return mo_edge_forward(V, nv, idx, n_items, kind, off, loss_out, stream);
    int64_t nh;
    int rc = check_edges(V, nv, idx, n_items, kind, &nh);
    if (rc) return rc;
    if (nh == 0) return MO_OK;
    MO_CHECK_ARG(off && loss_out, "null offset or output pointer");
    k_edge_forward_w<<<ceil_div(nh, 256), 256, 0, as_stream(stream)>>>(V, nv, idx, nh, kind, off, w, loss_out); ::mo::note_launch();
    MO_LAUNCH_CHECK("k_edge_forward_w");
    return MO_OK;
}

extern "C" int mo_edge_backward_w(const float* V, int64_t nv, const void* csr, int64_t nh, const float* off,
                                  const float* w, float* grad_out, void* stream) {
    if (!w) return mo_edge_backward(V, nv, csr, nh, off, grad_out, stream);
    MO_CHECK_ARG(nv >= 0 && nh >= 0, "negative size");
    if (nv == 0) return MO_OK;
    MO_CHECK_ARG(V && csr && grad_out && (nh == 0 || off), "null pointer");
    CsrView c = csr_view(const_cast<void*>(csr), nv, nh);
    k_edge_backward_w<<<ceil_div(nv, 256), 256, 0, as_stream(stream)>>>(V, nv, c.row_ptr, c.key, c.other, off, w,
                                                                        grad_out); ::mo::note_launch();
    MO_LAUNCH_CHECK("k_edge_backward_w");
    return MO_OK;
}

extern "C" int mo_edge_fwd_bwd(const float* V, int64_t nv, const int32_t* idx, int64_t n_items, int kind,
                               const void* csr, const float* off, const float* w, float* loss_out,
                               float* grad_out, void* stream) {
    int64_t nh;
    int rc = check_edges(V, nv, idx, n_items, kind, &nh);
    if (rc) return rc;
    MO_CHECK_ARG(grad_out && (nv == 0 || csr), "null gradient or CSR pointer");
    if (loss_out) {
        rc = mo_edge_forward_w(V, nv, idx, n_items, kind, off, w, loss_out, stream);
        if (rc) return rc;
    }
    return mo_edge_backward_w(V, nv, csr, nh, off, w, grad_out, stream);
}

extern "C" int mo_sell_plan(const void* csr, int64_t nv, int64_t nh, int32_t* slice_ptr, void* stream) {
    MO_CHECK_ARG(nv >= 0 && nh >= 0, "negative size");
    MO_CHECK_ARG(csr && slice_ptr, "null pointer");
    cudaStream_t s = as_stream(stream);
    const int64_t nslices = (nv + 31) / 32;
    CsrView c = csr_view(const_cast<void*>(csr), nv, nh);
    MO_CUDA(cudaMemsetAsync(slice_ptr, 0, sizeof(int) * (nslices + 1), s));
    if (nslices > 0) {
        k_sell_width<<<ceil_div(nslices * 32, 256), 256, 0, s>>>(nv, nslices, c.row_ptr, slice_ptr); ::mo::note_launch();
        MO_LAUNCH_CHECK("k_sell_width");
    }
    MO_CUDA(exclusive_scan_i32(slice_ptr, (int)(nslices + 1), nullptr, s));
    return MO_OK;
}

extern "C" int mo_sell_fill(const void* csr, int64_t nv, int64_t nh, const int32_t* slice_ptr, int32_t* records,
                            void* stream) {
    MO_CHECK_ARG(nv >= 0 && nh >= 0, "negative size");
    if (nv == 0) return MO_OK;
    MO_CHECK_ARG(csr && slice_ptr && records, "null pointer");
    const int64_t nslices = (nv + 31) / 32;
    CsrView c = csr_view(const_cast<void*>(csr), nv, nh);
    k_sell_fill<<<ceil_div(nslices * 32, 256), 256, 0, as_stream(stream)>>>(nv, nslices, c.row_ptr, c.key, c.other,
                                                                           slice_ptr, records); ::mo::note_launch();
    MO_LAUNCH_CHECK("k_sell_fill");
    return MO_OK;
}

extern "C" int mo_sell_fill_w(const void* csr, int64_t nv, int64_t nh, const int32_t* slice_ptr, const float* w,
                              float* record_w, void* stream) {
    MO_CHECK_ARG(nv >= 0 && nh >= 0, "negative size");
    if (nv == 0) return MO_OK;
    MO_CHECK_ARG(csr && slice_ptr && w && record_w, "null pointer");
    const int64_t nslices = (nv + 31) / 32;
    CsrView c = csr_view(const_cast<void*>(csr), nv, nh);
    k_sell_fill_w<<<ceil_div(nslices * 32, 256), 256, 0, as_stream(stream)>>>(nv, nslices, c.row_ptr, c.key,
                                                                             slice_ptr, w, record_w);
    ::mo::note_launch();
    MO_LAUNCH_CHECK("k_sell_fill_w");
    return MO_OK;
}
