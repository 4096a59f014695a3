// Nearest source vertex of every target vertex, and the reverse
// (target -> source) loss of src/python/layers/reverse_loss_layer.py:14-25:
//   ii = cKDTree(src).query(tar, k=1);  loss = 0.5 * sum |src[ii] - tar|^2.
//
// The query builds an LBVH over the source points (Morton codes in the points'
// bounding cube, stable radix sort, Karras tree, refit: the same stages as the
// distance-field build) and walks it once per target point, one thread per
// query, queries taken in Morton order so a warp's queries are neighbours.
// Distances are squared Euclidean in double, summed x, y, z like cKDTree's
// (src/scipy cKDTree evaluates them in float64 from the float32 input);
// among exactly equal distances the lowest source index wins.
#include <cfloat>

#include "mo_common.cuh"
#include "mo_lbvh.cuh"

namespace mo {
namespace {

constexpr int NN_STACK = 64;

struct NnScratch {
    int* bbox;        // 6 ordered ints
    float4* cube;     // lo.xyz, 1/extent
    int* status;
    uint32_t* codes_a;
    uint32_t* codes_b;
    int* ids_a;
    int* ids_b;
    float4* nodes;
    float4* boxes;
    int* parent;
    int* flags;
    int* hist;
    float* rootbox;
    uint32_t* qcodes_a;
    uint32_t* qcodes_b;
    int* qids_a;
    int* qids_b;
    int* qhist;
    size_t bytes;
};

size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

NnScratch plan(char* base, int64_t np, int64_t nq) {
    NnScratch s;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        char* p = base ? base + o : nullptr;
        o += a256(bytes);
        return p;
    };
    s.bbox = reinterpret_cast<int*>(take(32));
    s.cube = reinterpret_cast<float4*>(take(16));
    s.status = reinterpret_cast<int*>(take(16));
    s.rootbox = reinterpret_cast<float*>(take(32));
    s.codes_a = reinterpret_cast<uint32_t*>(take(4 * (size_t)np));
    s.codes_b = reinterpret_cast<uint32_t*>(take(4 * (size_t)np));
    s.ids_a = reinterpret_cast<int*>(take(4 * (size_t)np));
    s.ids_b = reinterpret_cast<int*>(take(4 * (size_t)np));
    s.nodes = reinterpret_cast<float4*>(take(64 * (size_t)(np > 1 ? np - 1 : 1)));
    s.boxes = reinterpret_cast<float4*>(take(32 * (size_t)np));
    s.parent = reinterpret_cast<int*>(take(8 * (size_t)np));
    s.flags = reinterpret_cast<int*>(take(4 * (size_t)np));
    s.hist = reinterpret_cast<int*>(take(4 * radix_hist_ints((int)np)));
    s.qcodes_a = reinterpret_cast<uint32_t*>(take(4 * (size_t)nq));
    s.qcodes_b = reinterpret_cast<uint32_t*>(take(4 * (size_t)nq));
    s.qids_a = reinterpret_cast<int*>(take(4 * (size_t)nq));
    s.qids_b = reinterpret_cast<int*>(take(4 * (size_t)nq));
    s.qhist = reinterpret_cast<int*>(take(4 * radix_hist_ints((int)nq)));
    s.bytes = o;
    return s;
}

__global__ void k_pt_bbox_init(int* bb) {
    if (threadIdx.x < 3) bb[threadIdx.x] = INT_MAX;
    else if (threadIdx.x < 6) bb[threadIdx.x] = INT_MIN;
}

// Exact per-axis extremes of the finite coordinates (ordered-int encoding).
__global__ void __launch_bounds__(256) k_pt_bbox(const float* __restrict__ P, int64_t n, int* __restrict__ bb) {
    int lo[3] = {INT_MAX, INT_MAX, INT_MAX}, hi[3] = {INT_MIN, INT_MIN, INT_MIN};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        for (int c = 0; c < 3; ++c) {
            const float f = P[3 * i + c];
            if (!isfinite(f)) continue;
            const int k = float_to_ordered(f);
            lo[c] = min(lo[c], k);
            hi[c] = max(hi[c], k);
        }
    }
    for (int c = 0; c < 3; ++c) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[c] = min(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], o));
            hi[c] = max(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], o));
        }
    }
    if ((threadIdx.x & 31) == 0) {
        for (int c = 0; c < 3; ++c) {
            atomicMin(&bb[c], lo[c]);
            atomicMax(&bb[3 + c], hi[c]);
        }
    }
}

// The cube the Morton codes quantise: lower corner and 1/longest extent.
__global__ void k_pt_cube(const int* __restrict__ bb, float4* __restrict__ cube) {
    float lo[3], ext = 0.f;
    for (int c = 0; c < 3; ++c) {
        lo[c] = bb[c] == INT_MAX ? 0.f : ordered_to_float(bb[c]);
        const float h = bb[3 + c] == INT_MIN ? 0.f : ordered_to_float(bb[3 + c]);
        ext = fmaxf(ext, h - lo[c]);
    }
    *cube = make_float4(lo[0], lo[1], lo[2], ext > 0.f && isfinite(ext) ? 1.0f / ext : 0.f);
}

__device__ __forceinline__ uint32_t pt_code(const float* __restrict__ p, float4 cube) {
    return morton30((p[0] - cube.x) * cube.w, (p[1] - cube.y) * cube.w, (p[2] - cube.z) * cube.w);
}

__global__ void k_pt_morton(const float* __restrict__ P, int64_t n, const float4* __restrict__ cube,
                            uint32_t* __restrict__ codes, int* __restrict__ ids) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    codes[i] = pt_code(P + 3 * i, *cube);
    ids[i] = (int)i;
}

// Leaf k's box is its point (NaN coordinates give an empty box, never nearest).
__global__ void k_pt_leaves(const float* __restrict__ P, const int* __restrict__ order, int n,
                            float4* __restrict__ boxes) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float* p = P + 3 * (int64_t)order[k];
    boxes[2 * (int64_t)k] = make_float4(p[0], p[1], p[2], 0.f);
    boxes[2 * (int64_t)k + 1] = make_float4(p[0], p[1], p[2], 0.f);
}

// Squared distance from q to a box, per axis max(lo - q, q - hi, 0), summed
// x, y, z in double.  For a point box it is cKDTree's (p - q)^2 sum exactly,
// and a box's value never exceeds that of a point inside it.
// Every product and sum rounded on its own (no fused multiply-add), the
// plain evaluation order.
__device__ __forceinline__ double sum_sq(double dx, double dy, double dz) {
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

__device__ __forceinline__ double box_d2(double qx, double qy, double qz, float4 lo, float4 hi) {
    const double dx = fmax(fmax(__dsub_rn((double)lo.x, qx), __dsub_rn(qx, (double)hi.x)), 0.0);
    const double dy = fmax(fmax(__dsub_rn((double)lo.y, qy), __dsub_rn(qy, (double)hi.y)), 0.0);
    const double dz = fmax(fmax(__dsub_rn((double)lo.z, qz), __dsub_rn(qz, (double)hi.z)), 0.0);
    return sum_sq(dx, dy, dz);
}

__device__ __forceinline__ double pt_d2(double qx, double qy, double qz, const float* __restrict__ p) {
    return sum_sq(__dsub_rn((double)__ldg(p), qx), __dsub_rn((double)__ldg(p + 1), qy),
                  __dsub_rn((double)__ldg(p + 2), qz));
}

__device__ __forceinline__ void take(double d, int id, double& best, int& best_id) {
    if (d < best || (d == best && id < best_id)) {
        best = d;
        best_id = id;
    }
}

__global__ void __launch_bounds__(128) k_nn(const float4* __restrict__ nodes, const int* __restrict__ order,
                                            const float* __restrict__ P, int np, const float* __restrict__ Q,
                                            const int* __restrict__ qorder, int nq, int32_t* __restrict__ idx_out,
                                            double* __restrict__ d2_out, int* __restrict__ status) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nq) return;
    const int q = qorder[t];
    const double qx = Q[3 * (int64_t)q], qy = Q[3 * (int64_t)q + 1], qz = Q[3 * (int64_t)q + 2];
    double best = DBL_MAX;  // a point at DBL_MAX or NaN distance is never taken
    int best_id = -1;
    if (!isfinite(qx) || !isfinite(qy) || !isfinite(qz)) {
        atomicOr(status, 16);
        idx_out[q] = 0;
        if (d2_out) d2_out[q] = DBL_MAX;
        return;
    }
    if (np == 1) {
        take(pt_d2(qx, qy, qz, P), 0, best, best_id);
    } else {
        int stack[NN_STACK];
        int sp = 0, node = 0;
        const int max_iter = 2 * np + 64;  // each node is entered at most once
        for (int iter = 0;; ++iter) {
            if (iter > max_iter) {
                atomicOr(status, 4);
                break;
            }
            const float4* nd = nodes + 4 * (int64_t)node;
            const float4 a = __ldg(nd), b = __ldg(nd + 1), c = __ldg(nd + 2), d = __ldg(nd + 3);
            const int L = __float_as_int(a.w), R = __float_as_int(b.w);
            double dl = box_d2(qx, qy, qz, a, b), dr = box_d2(qx, qy, qz, c, d);
            // boxes at exactly the best distance are opened too: a lower index
            // may tie
            bool wl = dl <= best, wr = dr <= best;
            if (wl && L < 0) {
                const int id = order[~L];
                take(pt_d2(qx, qy, qz, P + 3 * (int64_t)id), id, best, best_id);
                wl = false;
            }
            if (wr && R < 0) {
                const int id = order[~R];
                take(pt_d2(qx, qy, qz, P + 3 * (int64_t)id), id, best, best_id);
                wr = false;
            }
            wl = wl && dl <= best;
            wr = wr && dr <= best;
            if (wl && wr) {
                if (sp >= NN_STACK) {  // cannot happen for trees of depth <= 64
                    atomicOr(status, 2);
                    break;
                }
                const bool lfirst = dl <= dr;
                stack[sp++] = lfirst ? R : L;
                node = lfirst ? L : R;
            } else if (wl) {
                node = L;
            } else if (wr) {
                node = R;
            } else {
                if (sp == 0) break;
                node = stack[--sp];
            }
        }
    }
    if (best_id < 0) atomicOr(status, 8);  // every source coordinate non-finite
    idx_out[q] = best_id < 0 ? 0 : best_id;
    if (d2_out) d2_out[q] = best;
}

// ---- reverse loss ----------------------------------------------------------
constexpr int RL_THREADS = 256;

// Block b sums 0.5*|src[idx[t]] - tar[t]|^2 (float differences and squares
// as the reference's tensors compute them, accumulated in double) over its
// chunk in a fixed tree order.
__global__ void __launch_bounds__(RL_THREADS) k_rev_partial(const float* __restrict__ src, int64_t ns,
                                                           const float* __restrict__ tar,
                                                           const int32_t* __restrict__ idx, int64_t nt,
                                                           double* __restrict__ partial, int* __restrict__ status) {
    __shared__ double sh[RL_THREADS];
    double acc = 0.0;
    for (int64_t t = (int64_t)blockIdx.x * RL_THREADS + threadIdx.x; t < nt; t += (int64_t)gridDim.x * RL_THREADS) {
        const int64_t i = idx[t];
        if (i < 0 || i >= ns) {  // skipped and reported
            atomicOr(status, 1);
            continue;
        }
        for (int c = 0; c < 3; ++c) {
            const float l = SUB(src[3 * i + c], tar[3 * t + c]);
            acc += (double)MUL(l, l);
        }
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int o = RL_THREADS / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(RL_THREADS) k_rev_total(const double* __restrict__ partial, int n,
                                                         double* __restrict__ loss) {
    __shared__ double sh[RL_THREADS];
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += RL_THREADS) acc += partial[i];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int o = RL_THREADS / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *loss = 0.5 * sh[0];
}

// Segment bounds of the targets grouped by their nearest source vertex.
__global__ void k_rev_segments(const uint32_t* __restrict__ keys, int nt, int64_t ns, int* __restrict__ seg_begin,
                               int* __restrict__ seg_end, int* __restrict__ status) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nt) return;
    const uint32_t key = keys[k];
    if ((int64_t)key >= ns) {  // out-of-range (or negative) index: skipped and reported
        atomicOr(status, 1);
        return;
    }
    if (k == 0 || keys[k - 1] != key) seg_begin[key] = k;
    if (k == nt - 1 || keys[k + 1] != key) seg_end[key] = k + 1;
}

// grad_src[i] = sum over the targets t matched to i, in increasing t, of
// (g*l + g*l) with l = src[i] - tar[t] and g = 0.5 * grad_out: torch's
// backward of 0.5*(l*l).sum() through src_V[ii], whose index_put_
// accumulation adds the matched rows in order, from zero.
__global__ void k_rev_grad(const float* __restrict__ src, const float* __restrict__ tar,
                           const int* __restrict__ sorted_t, const int* __restrict__ seg_begin,
                           const int* __restrict__ seg_end, int64_t ns, const float* __restrict__ grad_out,
                           float* __restrict__ grad_src) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ns) return;
    const float g = MUL(0.5f, *grad_out);
    float a0 = 0.f, a1 = 0.f, a2 = 0.f;
    const int b = seg_begin[i], e = seg_end[i];
    for (int k = b; k < e; ++k) {
        const int64_t t = sorted_t[k];
        const float l0 = SUB(src[3 * i], tar[3 * t]), l1 = SUB(src[3 * i + 1], tar[3 * t + 1]);
        const float l2 = SUB(src[3 * i + 2], tar[3 * t + 2]);
        const float g0 = MUL(g, l0), g1 = MUL(g, l1), g2 = MUL(g, l2);
        a0 = ADD(a0, ADD(g0, g0));
        a1 = ADD(a1, ADD(g1, g1));
        a2 = ADD(a2, ADD(g2, g2));
    }
    grad_src[3 * i] = a0;
    grad_src[3 * i + 1] = a1;
    grad_src[3 * i + 2] = a2;
}

struct RevScratch {
    int* status;
    double* partial;
    uint32_t* keys_a;
    uint32_t* keys_b;
    int* vals_a;
    int* vals_b;
    int* hist;
    int* seg_begin;
    int* seg_end;
    size_t bytes;
};

constexpr int RL_BLOCKS = 1024;

RevScratch plan_rev(char* base, int64_t ns, int64_t nt) {
    RevScratch s;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        char* p = base ? base + o : nullptr;
        o += a256(bytes);
        return p;
    };
    s.status = reinterpret_cast<int*>(take(16));
    s.partial = reinterpret_cast<double*>(take(8 * RL_BLOCKS));
    s.keys_a = reinterpret_cast<uint32_t*>(take(4 * (size_t)nt));
    s.keys_b = reinterpret_cast<uint32_t*>(take(4 * (size_t)nt));
    s.vals_a = reinterpret_cast<int*>(take(4 * (size_t)nt));
    s.vals_b = reinterpret_cast<int*>(take(4 * (size_t)nt));
    s.hist = reinterpret_cast<int*>(take(4 * radix_hist_ints((int)nt)));
    s.seg_begin = reinterpret_cast<int*>(take(4 * (size_t)ns));
    s.seg_end = reinterpret_cast<int*>(take(4 * (size_t)ns));
    s.bytes = o;
    return s;
}

__global__ void k_rev_keys(const int32_t* __restrict__ idx, int64_t nt, uint32_t* __restrict__ keys,
                           int* __restrict__ vals) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    keys[t] = (uint32_t)idx[t];
    vals[t] = (int)t;
}

int bits_for(int64_t n) {
    int b = 1;
    while (b < 32 && ((int64_t)1 << b) < n) ++b;
    return b;
}

// status_out given: OR the index error into it; else synchronise and report.
int finish_status(RevScratch& S, int32_t* status_out, cudaStream_t s) {
    if (status_out) return MO_OK;
    int status = 0;
    cudaError_t e = cudaMemcpyAsync(&status, S.status, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_status(e, "reverse loss status");
    if (status & 1) {
        set_error("nearest-point index out of range");
        return MO_ERR_DEVICE;
    }
    return MO_OK;
}

}  // namespace
}  // namespace mo

using namespace mo;

extern "C" size_t mo_nn_scratch_bytes(int64_t np, int64_t nq) {
    if (np < 0 || nq < 0) return 0;
    return plan(nullptr, np, nq).bytes;
}

extern "C" int mo_nn_query(const float* P, int64_t np, const float* Q, int64_t nq, int32_t* idx_out,
                           double* d2_out, void* scratch, size_t scratch_bytes, void* stream) {
    MO_CHECK_ARG(np > 0 && nq >= 0, "need at least one source point (np=%lld)", (long long)np);
    MO_CHECK_ARG(np < ((int64_t)1 << 30) && nq < ((int64_t)1 << 31), "too many points");
    if (nq == 0) return MO_OK;
    MO_CHECK_ARG(P && Q && idx_out, "null pointer");
    cudaStream_t s = as_stream(stream);
    const size_t need = plan(nullptr, np, nq).bytes;
    void* owned = nullptr;
    if (!scratch) {
        MO_CUDA(cudaMallocAsync(&owned, need, s));
        scratch = owned;
    } else if (scratch_bytes < need) {
        set_error("NN query scratch too small: %zu < %zu", scratch_bytes, need);
        return MO_ERR_SCRATCH;
    }
    NnScratch S = plan(reinterpret_cast<char*>(scratch), np, nq);
    int rc = MO_OK;
    do {
        cudaError_t e = cudaMemsetAsync(S.status, 0, 16, s);
        if (e != cudaSuccess) { rc = cuda_status(e, "memset"); break; }
        k_pt_bbox_init<<<1, 32, 0, s>>>(S.bbox); ::mo::note_launch();
        k_pt_bbox<<<std::min(ceil_div(np, 256), 4 * device_sm_count()), 256, 0, s>>>(P, np, S.bbox);
        ::mo::note_launch();
        k_pt_cube<<<1, 1, 0, s>>>(S.bbox, S.cube); ::mo::note_launch();
        k_pt_morton<<<ceil_div(np, 256), 256, 0, s>>>(P, np, S.cube, S.codes_a, S.ids_a); ::mo::note_launch();
        e = radix_sort_pairs(S.codes_a, S.ids_a, S.codes_b, S.ids_b, (int)np, 30, S.hist, s);
        if (e != cudaSuccess) { rc = cuda_status(e, "radix_sort_pairs"); break; }
        // queries in Morton order of the same cube
        k_pt_morton<<<ceil_div(nq, 256), 256, 0, s>>>(Q, nq, S.cube, S.qcodes_a, S.qids_a); ::mo::note_launch();
        e = radix_sort_pairs(S.qcodes_a, S.qids_a, S.qcodes_b, S.qids_b, (int)nq, 30, S.qhist, s);
        if (e != cudaSuccess) { rc = cuda_status(e, "radix_sort_pairs"); break; }
        if (np > 1) {
            k_pt_leaves<<<ceil_div(np, 256), 256, 0, s>>>(P, S.ids_a, (int)np, S.boxes); ::mo::note_launch();
            k_karras<<<ceil_div(np - 1, 256), 256, 0, s>>>(S.codes_a, (int)np, S.nodes, S.parent, S.flags,
                                                           nullptr);
            ::mo::note_launch();
            k_refit<<<ceil_div(np, 256), 256, 0, s>>>(S.boxes, (int)np, S.nodes, S.parent, S.flags, S.rootbox,
                                                       S.status);
            ::mo::note_launch();
        }
        k_nn<<<ceil_div(nq, 128), 128, 0, s>>>(S.nodes, S.ids_a, P, (int)np, Q, S.qids_a, (int)nq, idx_out, d2_out,
                                               S.status);
        ::mo::note_launch();
        e = cudaGetLastError();
        if (e != cudaSuccess) { rc = cuda_status(e, "nn kernels"); break; }
        int status = 0;
        e = cudaMemcpyAsync(&status, S.status, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) { rc = cuda_status(e, "nn status"); break; }
        if (status & 16) { set_error("a query point has non-finite coordinates"); rc = MO_ERR_DEVICE; }
        else if (status & 8) { set_error("no source point has finite coordinates"); rc = MO_ERR_DEVICE; }
        else if (status & 6) { set_error("point LBVH is malformed (status %d)", status); rc = MO_ERR_DEVICE; }
    } while (0);
    if (owned) cudaFreeAsync(owned, s);
    return rc;
}

extern "C" size_t mo_reverse_loss_scratch_bytes(int64_t ns, int64_t nt) {
    if (ns < 0 || nt < 0) return 0;
    return plan_rev(nullptr, ns, nt).bytes;
}

extern "C" int mo_reverse_loss_forward(const float* src, int64_t ns, const float* tar, int64_t nt,
                                       const int32_t* idx, double* loss_out, void* scratch, size_t scratch_bytes,
                                       int32_t* status_out, void* stream) {
    MO_CHECK_ARG(ns > 0 && nt >= 0 && nt < ((int64_t)1 << 31), "bad sizes");
    MO_CHECK_ARG(src && loss_out && (nt == 0 || (tar && idx)), "null pointer");
    MO_CHECK_ARG(scratch && scratch_bytes >= plan_rev(nullptr, ns, nt).bytes, "reverse loss scratch too small");
    cudaStream_t s = as_stream(stream);
    RevScratch S = plan_rev(reinterpret_cast<char*>(scratch), ns, nt);
    int* st = status_out ? reinterpret_cast<int*>(status_out) : S.status;
    if (!status_out) MO_CUDA(cudaMemsetAsync(S.status, 0, 16, s));
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(RL_BLOCKS, (nt + RL_THREADS - 1) / RL_THREADS));
    k_rev_partial<<<blocks, RL_THREADS, 0, s>>>(src, ns, tar, idx, nt, S.partial, st); ::mo::note_launch();
    k_rev_total<<<1, RL_THREADS, 0, s>>>(S.partial, blocks, loss_out); ::mo::note_launch();
    MO_LAUNCH_CHECK("reverse loss forward");
    return finish_status(S, status_out, s);
}

extern "C" int mo_reverse_loss_backward(const float* src, int64_t ns, const float* tar, int64_t nt,
                                        const int32_t* idx, const float* grad_out, float* grad_src, void* scratch,
                                        size_t scratch_bytes, int32_t* status_out, void* stream) {
    MO_CHECK_ARG(ns > 0 && nt >= 0 && nt < ((int64_t)1 << 31) && ns < ((int64_t)1 << 31), "bad sizes");
    MO_CHECK_ARG(src && grad_out && grad_src && (nt == 0 || (tar && idx)), "null pointer");
    MO_CHECK_ARG(scratch && scratch_bytes >= plan_rev(nullptr, ns, nt).bytes, "reverse loss scratch too small");
    cudaStream_t s = as_stream(stream);
    RevScratch S = plan_rev(reinterpret_cast<char*>(scratch), ns, nt);
    int* st = status_out ? reinterpret_cast<int*>(status_out) : S.status;
    if (!status_out) MO_CUDA(cudaMemsetAsync(S.status, 0, 16, s));
    MO_CUDA(cudaMemsetAsync(S.seg_begin, 0, 4 * (size_t)ns, s));
    MO_CUDA(cudaMemsetAsync(S.seg_end, 0, 4 * (size_t)ns, s));
    if (nt > 0) {
        k_rev_keys<<<ceil_div(nt, 256), 256, 0, s>>>(idx, nt, S.keys_a, S.vals_a); ::mo::note_launch();
        MO_CUDA(radix_sort_pairs(S.keys_a, S.vals_a, S.keys_b, S.vals_b, (int)nt, bits_for(ns), S.hist, s));
        k_rev_segments<<<ceil_div(nt, 256), 256, 0, s>>>(S.keys_a, (int)nt, ns, S.seg_begin, S.seg_end, st);
        ::mo::note_launch();
    }
    k_rev_grad<<<ceil_div(ns, 256), 256, 0, s>>>(src, tar, S.vals_a, S.seg_begin, S.seg_end, ns, grad_out, grad_src);
    ::mo::note_launch();
    MO_LAUNCH_CHECK("reverse loss backward");
    return finish_status(S, status_out, s);
}
