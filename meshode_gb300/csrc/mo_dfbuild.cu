// Distance-field build: normalisation, triangle records, Morton codes, stable
// radix sort, Karras LBVH, bottom-up refit, warp-packet nearest-triangle
// traversal, and a shared-memory-tiled brute force for small targets.
// Reference: Mesh::Normalize (src/lib/mesh.cc:66-96) and
// Mesh::ConstructDistanceField (mesh.cc:106-152), whose
// igl::point_mesh_squared_distance query (mesh.cc:140) returns the exact
// squared distance to the nearest triangle; the grid stores its sqrt.
#include <cfloat>
#include <cmath>
#include <cstring>
#include <mutex>

#include "mo_common.cuh"
#include "mo_df_trav.cuh"
#include "mo_lbvh.cuh"

namespace mo {

// ---------------------------------------------------------------------------
// Normalisation
// ---------------------------------------------------------------------------
__global__ void k_bbox_init(int* bb) {
    if (threadIdx.x < 3) bb[threadIdx.x] = INT_MAX;
    else if (threadIdx.x < 6) bb[threadIdx.x] = INT_MIN;
}

__global__ void __launch_bounds__(256) k_bbox(const float* __restrict__ V, int64_t n, int* __restrict__ bb) {
    int lo[3] = {INT_MAX, INT_MAX, INT_MAX}, hi[3] = {INT_MIN, INT_MIN, INT_MIN};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        for (int c = 0; c < 3; ++c) {
            const float f = V[3 * i + c];
            if (f != f) continue;  // NaN never wins a comparison in the reference
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

// mesh.cc:79-82 in double from the exact float extremes.
__global__ void k_norm_params(const int* __restrict__ bb, double* __restrict__ prm) {
    double mn[3], mx[3];
    for (int c = 0; c < 3; ++c) {
        mn[c] = (bb[c] == INT_MAX) ? 1e30 : (double)ordered_to_float(bb[c]);
        mx[c] = (bb[3 + c] == INT_MIN) ? -1e30 : (double)ordered_to_float(bb[3 + c]);
    }
    const double e0 = mx[0] - mn[0], e1 = mx[1] - mn[1], e2 = mx[2] - mn[2];
    const double m12 = (e1 < e2) ? e2 : e1;
    const double m = (e0 < m12) ? m12 : e0;
    const double scale = m * 1.1;
    prm[0] = scale;
    for (int c = 0; c < 3; ++c) prm[1 + c] = mn[c] - 0.05 * scale;
}

// normalize.cc:21 / :42, evaluated in double (the reference's FT) once per
// vertex, rounded to float.
__global__ void k_normalize(float* __restrict__ V, int64_t n, const double* __restrict__ prm, int inverse) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * n) return;
    const int c = (int)(i % 3);
    const double s = prm[0], t = prm[1 + c];
    const double v = (double)V[i];
    V[i] = inverse ? (float)__dadd_rn(__dmul_rn(v, s), t) : (float)__ddiv_rn(__dsub_rn(v, t), s);
}

__global__ void k_normalize_copy(const float* __restrict__ V, int64_t n, const double* __restrict__ prm,
                                 float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * n) return;
    const int c = (int)(i % 3);
    out[i] = (float)__ddiv_rn(__dsub_rn((double)V[i], prm[1 + c]), prm[0]);
}

// Triangle records (the layout is described in mo_df_trav.cuh).

__device__ __forceinline__ float dot3(float ax, float ay, float az, float bx, float by, float bz) {
    return ax * bx + ay * by + az * bz;
}

__device__ Tri make_tri(const float* __restrict__ Vn, int i0, int i1, int i2, float4* lo, float4* hi) {
    const float ax = Vn[3 * (int64_t)i0], ay = Vn[3 * (int64_t)i0 + 1], az = Vn[3 * (int64_t)i0 + 2];
    const float bx = Vn[3 * (int64_t)i1], by = Vn[3 * (int64_t)i1 + 1], bz = Vn[3 * (int64_t)i1 + 2];
    const float cx = Vn[3 * (int64_t)i2], cy = Vn[3 * (int64_t)i2 + 1], cz = Vn[3 * (int64_t)i2 + 2];
    *lo = make_float4(fminf(fminf(ax, bx), cx), fminf(fminf(ay, by), cy), fminf(fminf(az, bz), cz), 0.f);
    *hi = make_float4(fmaxf(fmaxf(ax, bx), cx), fmaxf(fmaxf(ay, by), cy), fmaxf(fmaxf(az, bz), cz), 0.f);
    const float abx = bx - ax, aby = by - ay, abz = bz - az;
    const float acx = cx - ax, acy = cy - ay, acz = cz - az;
    const float lab = dot3(abx, aby, abz, abx, aby, abz);
    float nx = aby * acz - abz * acy, ny = abz * acx - abx * acz, nz = abx * acy - aby * acx;
    const float nn = dot3(nx, ny, nz, nx, ny, nz);
    Tri t;
    if (nn > 0.f && isfinite(nn) && lab > 0.f) {
        const float inn = rsqrtf(nn);
        nx *= inn; ny *= inn; nz *= inn;
        const float len = sqrtf(lab), il = 1.0f / len;
        const float ex = abx * il, ey = aby * il, ez = abz * il;
        const float yx = ny * ez - nz * ey, yy = nz * ex - nx * ez, yz = nx * ey - ny * ex;  // n x ex
        const float c2x = dot3(acx, acy, acz, ex, ey, ez), c2y = dot3(acx, acy, acz, yx, yy, yz);
        const float ebx = c2x - len;
        const float lac = c2x * c2x + c2y * c2y, lbc = ebx * ebx + c2y * c2y;
        t.r0 = make_float4(ax, ay, az, len);
        t.r1 = make_float4(ex, ey, ez, c2x);
        t.r2 = make_float4(yx, yy, yz, c2y);
        t.r3 = make_float4(nx, ny, nz, 1.f);
        t.r4 = make_float4(1.0f / len, lac > 0.f ? 1.0f / lac : 0.f, lbc > 0.f ? 1.0f / lbc : 0.f, ebx);
    } else {
        const float bcx = cx - bx, bcy = cy - by, bcz = cz - bz;
        const float lbc = dot3(bcx, bcy, bcz, bcx, bcy, bcz);
        const float lca = dot3(acx, acy, acz, acx, acy, acz);
        t.r0 = make_float4(ax, ay, az, 0.f);
        t.r1 = make_float4(bx, by, bz, 0.f);
        t.r2 = make_float4(cx, cy, cz, 0.f);
        t.r3 = make_float4(0.f, 0.f, 0.f, 0.f);
        t.r4 = make_float4(lab > 0.f ? 1.0f / lab : 0.f, lbc > 0.f ? 1.0f / lbc : 0.f, lca > 0.f ? 1.0f / lca : 0.f,
                           0.f);
    }
    return t;
}

__device__ __forceinline__ void store_tri(float4* __restrict__ tris, int i, const Tri& t) {
    float4* p = tris + TRI_F4 * (int64_t)i;
    p[0] = t.r0; p[1] = t.r1; p[2] = t.r2; p[3] = t.r3; p[4] = t.r4;
}

// ---------------------------------------------------------------------------
// Morton codes (identical float operations to the oracle's restatement).
// ---------------------------------------------------------------------------
__global__ void k_morton(const float* __restrict__ Vn, const int32_t* __restrict__ F, int64_t nf, int64_t nv,
                         uint32_t* __restrict__ codes, int* __restrict__ ids, int* __restrict__ status) {
    const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const int i0 = F[3 * f], i1 = F[3 * f + 1], i2 = F[3 * f + 2];
    ids[f] = (int)f;
    if (i0 < 0 || i1 < 0 || i2 < 0 || i0 >= nv || i1 >= nv || i2 >= nv) {
        atomicOr(status, 1);
        codes[f] = 0;
        return;
    }
    float c[3];
    for (int k = 0; k < 3; ++k) {
        float s = ADD(Vn[3 * (int64_t)i0 + k], Vn[3 * (int64_t)i1 + k]);
        s = ADD(s, Vn[3 * (int64_t)i2 + k]);
        c[k] = __fdiv_rn(s, 3.0f);
    }
    codes[f] = (spread10(quant10(c[0])) << 2) | (spread10(quant10(c[1])) << 1) | spread10(quant10(c[2]));
}

__global__ void k_check_faces(const int32_t* __restrict__ F, int64_t nf, int64_t nv, int* __restrict__ status) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * nf) return;
    const int v = F[i];
    if (v < 0 || v >= nv) atomicOr(status, 1);
}

// Sorted triangle records (leaf order) from the sorted ids.
__global__ void k_tri_records(const float* __restrict__ Vn, const int32_t* __restrict__ F, int64_t nf,
                              int64_t nv, const int* __restrict__ order, float4* __restrict__ tris,
                              float4* __restrict__ boxes) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nf) return;
    const int64_t f = order ? order[i] : i;
    int i0 = F[3 * f], i1 = F[3 * f + 1], i2 = F[3 * f + 2];
    if (i0 < 0 || i1 < 0 || i2 < 0 || i0 >= nv || i1 >= nv || i2 >= nv) i0 = i1 = i2 = 0;  // flagged earlier
    float4 lo, hi;
    store_tri(tris, (int)i, make_tri(Vn, i0, i1, i2, &lo, &hi));
    if (boxes) {
        boxes[2 * i] = lo;
        boxes[2 * i + 1] = hi;
    }
}

// ---------------------------------------------------------------------------
// Karras (2012) binary radix tree over sorted codes.  Node record (64 B):
//   [0] = (left box lo xyz, left child), [1] = (left box hi xyz, right child),
//   [2] = (right box lo xyz, -), [3] = (right box hi xyz, -).
// Children >= 0 are internal nodes, ~i encodes leaf i.  parent[] slots:
// internal i -> i, leaf j -> (n-1)+j; value = 2*parent + side.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int kdelta(const uint32_t* __restrict__ k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const uint32_t a = k[i], b = k[j];
    if (a != b) return __clz(a ^ b);
    return 32 + __clz((uint32_t)i ^ (uint32_t)j);
}

__global__ void k_karras(const uint32_t* __restrict__ k, int n, float4* __restrict__ nodes,
                         int* __restrict__ parent, int* __restrict__ flags, int2* __restrict__ range) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (kdelta(k, n, i, i + 1) - kdelta(k, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = kdelta(k, n, i, i - d);
    int lmax = 2;
    while (kdelta(k, n, i, i + lmax * d) > dmin) lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
        if (kdelta(k, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = kdelta(k, n, i, j);
    int s = 0, t = l;
    do {
        t = (t + 1) / 2;
        if (kdelta(k, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int gamma = i + s * d + (d < 0 ? -1 : 0);
    const int lo = min(i, j), hi = max(i, j);
    if (range) range[i] = make_int2(lo, hi);
    const int left = (lo == gamma) ? ~gamma : gamma;
    const int right = (hi == gamma + 1) ? ~(gamma + 1) : gamma + 1;
    nodes[4 * (int64_t)i].w = __int_as_float(left);
    nodes[4 * (int64_t)i + 1].w = __int_as_float(right);
    parent[left >= 0 ? left : (n - 1) + ~left] = 2 * i;
    parent[right >= 0 ? right : (n - 1) + ~right] = 2 * i + 1;
    flags[i] = 0;
    if (i == 0) parent[0] = -1;
}

__device__ __forceinline__ void write_child_box(float4* nodes, int p, int side, const float lo[3],
                                                const float hi[3]) {
    float* r = reinterpret_cast<float*>(nodes + 4 * (int64_t)p + 2 * side);
    r[0] = lo[0]; r[1] = lo[1]; r[2] = lo[2];
    r[4] = hi[0]; r[5] = hi[1]; r[6] = hi[2];
}

// Bottom-up refit: the second thread to reach a node merges its children.
__global__ void k_refit(const float4* __restrict__ boxes, int n, float4* nodes, const int* __restrict__ parent,
                        int* flags, float* rootbox, int* status) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const float4 blo = boxes[2 * (int64_t)j], bhi = boxes[2 * (int64_t)j + 1];
    float lo[3] = {blo.x, blo.y, blo.z};
    float hi[3] = {bhi.x, bhi.y, bhi.z};
    int slot = (n - 1) + j;
    // A Karras tree over distinct (code, index) keys is at most 64 levels
    // deep; the bound only guards against a corrupted parent array.
    for (int level = 0;; ++level) {
        if (level > 128) {
            atomicOr(status, 4);
            return;
        }
        const int ps = parent[slot];
        if (ps < 0) break;  // root
        const int p = ps >> 1, side = ps & 1;
        write_child_box(nodes, p, side, lo, hi);
        __threadfence();
        if (atomicAdd(&flags[p], 1) == 0) return;
        __threadfence();
        const float* r = reinterpret_cast<const float*>(nodes + 4 * (int64_t)p);
        for (int c = 0; c < 3; ++c) {
            lo[c] = fminf(__ldcg(r + c), __ldcg(r + 8 + c));
            hi[c] = fmaxf(__ldcg(r + 4 + c), __ldcg(r + 12 + c));
        }
        slot = p;
    }
    for (int c = 0; c < 3; ++c) {
        rootbox[c] = lo[c];
        rootbox[3 + c] = hi[c];
    }
}

// Leaf buckets: a child whose subtree holds at most DF_BUCKET triangles is a
// bucket -- its record holds ~first leaf and the count (a single triangle:
// count 1; an internal child: 0) -- and the traversal tests the bucket's
// contiguous sorted triangles directly instead of descending the bottom
// levels of the tree.
constexpr int DF_BUCKET = 6;

// ---------------------------------------------------------------------------
// Oriented bounding boxes.  Every child of a node is bounded, for the
// traversal, by a box aligned with its surface patch: axis a3 along the sum
// of the patch's area-weighted normals, a1 in the patch's plane (a single
// triangle: along its first edge; otherwise the x or y axis projected on the
// plane), a2 = a3 x a1, extents measured from an origin corner.  A near-planar
// patch's box is thin along its normal, so it reaches toward a query point
// only by the patch's curvature, where an axis-aligned box reaches by the
// patch's size; far fewer boxes come within a voxel's distance.
// Subtrees of at most OBB_EXACT triangles get extents from their own
// vertices; larger ones from the eight corners of their two children's boxes.
// Every extent is widened by OBB_INFL on both sides, more than the float
// rounding of the projections at build and query time, so the box contains
// its triangles' computed points and the distance bound stays below every
// triangle's computed distance by less than the traversal's slack.
// ---------------------------------------------------------------------------
constexpr int OBB_EXACT = 4096;
constexpr float OBB_INFL = 2e-6f;

struct Obb {
    float3 o, a1, a2, e;  // origin, axes (a3 = a1 x a2), extents
};

__device__ __forceinline__ float3 unit3f(float3 v, float3 fallback) {
    const float n2 = v.x * v.x + v.y * v.y + v.z * v.z;
    if (!(n2 > 1e-30f) || !isfinite(n2)) return fallback;
    const float r = 1.0f / sqrtf(n2);
    return make_float3(v.x * r, v.y * r, v.z * r);
}

// Frame from a normal sum and an in-plane hint (NaN hint: project x or y).
__device__ void obb_frame(float3 nsum, float3 hint, float3& a1, float3& a2) {
    const float3 a3 = unit3f(nsum, make_float3(0.f, 0.f, 1.f));
    float3 h = hint;
    if (!(h.x == h.x)) h = fabsf(a3.x) < 0.9f ? make_float3(1.f, 0.f, 0.f) : make_float3(0.f, 1.f, 0.f);
    const float d = h.x * a3.x + h.y * a3.y + h.z * a3.z;
    float3 t = make_float3(h.x - d * a3.x, h.y - d * a3.y, h.z - d * a3.z);
    const float3 alt = fabsf(a3.x) < 0.9f ? make_float3(1.f - a3.x * a3.x, -a3.x * a3.y, -a3.x * a3.z)
                                          : make_float3(-a3.y * a3.x, 1.f - a3.y * a3.y, -a3.y * a3.z);
    a1 = unit3f(t, unit3f(alt, make_float3(1.f, 0.f, 0.f)));
    a2 = unit3f(make_float3(a3.y * a1.z - a3.z * a1.y, a3.z * a1.x - a3.x * a1.z, a3.x * a1.y - a3.y * a1.x),
                make_float3(0.f, 1.f, 0.f));
}

// Running extents of points projected on (a1, a2, a3) relative to r.
struct Ext {
    float lo[3], hi[3];
    __device__ void init() {
        for (int k = 0; k < 3; ++k) { lo[k] = FLT_MAX; hi[k] = -FLT_MAX; }
    }
    __device__ void add(float3 a1, float3 a2, float3 a3, float3 r, float x, float y, float z) {
        const float qx = __fsub_rn(x, r.x), qy = __fsub_rn(y, r.y), qz = __fsub_rn(z, r.z);
        const float t[3] = {dotf3(a1, qx, qy, qz), dotf3(a2, qx, qy, qz), dotf3(a3, qx, qy, qz)};
        for (int k = 0; k < 3; ++k) { lo[k] = fminf(lo[k], t[k]); hi[k] = fmaxf(hi[k], t[k]); }
    }
    __device__ Obb finish(float3 a1, float3 a2, float3 a3, float3 r) const {
        Obb b;
        b.a1 = a1; b.a2 = a2;
        float l[3];
        for (int k = 0; k < 3; ++k) l[k] = lo[k] - OBB_INFL;
        b.o = make_float3(r.x + l[0] * a1.x + l[1] * a2.x + l[2] * a3.x, r.y + l[0] * a1.y + l[1] * a2.y + l[2] * a3.y,
                          r.z + l[0] * a1.z + l[1] * a2.z + l[2] * a3.z);
        b.e = make_float3(hi[0] - lo[0] + 2.f * OBB_INFL, hi[1] - lo[1] + 2.f * OBB_INFL,
                          hi[2] - lo[2] + 2.f * OBB_INFL);
        return b;
    }
};

// The vertices of sorted triangle k from its record (non-degenerate: a, a +
// bx ex, a + cx ex + cy ey, within rounding of the input vertices) and its
// normal scaled by twice its area (zero for a degenerate record).
__device__ __forceinline__ void rec_tri(const float4* __restrict__ tris, int k, float3 v[3], float3* n,
                                        float3* edge) {
    const float4* r = tris + TRI_F4 * (int64_t)k;
    const float4 r0 = __ldg(r), r1 = __ldg(r + 1), r2 = __ldg(r + 2), r3 = __ldg(r + 3);
    v[0] = make_float3(r0.x, r0.y, r0.z);
    if (r3.w != 0.f) {
        v[1] = make_float3(fmaf(r0.w, r1.x, r0.x), fmaf(r0.w, r1.y, r0.y), fmaf(r0.w, r1.z, r0.z));
        v[2] = make_float3(fmaf(r2.w, r2.x, fmaf(r1.w, r1.x, r0.x)), fmaf(r2.w, r2.y, fmaf(r1.w, r1.y, r0.y)),
                           fmaf(r2.w, r2.z, fmaf(r1.w, r1.z, r0.z)));
        const float w = r0.w * r2.w;
        *n = make_float3(r3.x * w, r3.y * w, r3.z * w);
        *edge = make_float3(r1.x, r1.y, r1.z);
    } else {
        v[1] = make_float3(r1.x, r1.y, r1.z);
        v[2] = make_float3(r2.x, r2.y, r2.z);
        *n = make_float3(0.f, 0.f, 0.f);
        *edge = make_float3(r1.x - r0.x, r1.y - r0.y, r1.z - r0.z);
    }
}

// The box of one sorted triangle (a1 along its first edge).
__device__ Obb obb_of_tri(const float4* __restrict__ tris, int k, float3* nsum_out) {
    float3 v[3], n, edge;
    rec_tri(tris, k, v, &n, &edge);
    float3 a1, a2;
    obb_frame(n, edge, a1, a2);
    const float3 a3 = obb_a3(a1, a2);
    Ext x;
    x.init();
    for (int c = 0; c < 3; ++c) x.add(a1, a2, a3, v[0], v[c].x, v[c].y, v[c].z);
    *nsum_out = n;
    return x.finish(a1, a2, a3, v[0]);
}

// obb[4*i] = (o, nsum.x) (a1, nsum.y) (a2, nsum.z) (e, -) of internal node i.
__device__ __forceinline__ void store_obb(float4* __restrict__ obb, int i, const Obb& b, float3 ns) {
    obb[4 * (int64_t)i] = make_float4(b.o.x, b.o.y, b.o.z, ns.x);
    obb[4 * (int64_t)i + 1] = make_float4(b.a1.x, b.a1.y, b.a1.z, ns.y);
    obb[4 * (int64_t)i + 2] = make_float4(b.a2.x, b.a2.y, b.a2.z, ns.z);
    obb[4 * (int64_t)i + 3] = make_float4(b.e.x, b.e.y, b.e.z, 0.f);
}

__device__ __forceinline__ Obb load_obb(const float4* obb, int i, float3* ns) {
    const float4 p = __ldcg(obb + 4 * (int64_t)i), q = __ldcg(obb + 4 * (int64_t)i + 1);
    const float4 u = __ldcg(obb + 4 * (int64_t)i + 2), w = __ldcg(obb + 4 * (int64_t)i + 3);
    Obb b;
    b.o = make_float3(p.x, p.y, p.z);
    b.a1 = make_float3(q.x, q.y, q.z);
    b.a2 = make_float3(u.x, u.y, u.z);
    b.e = make_float3(w.x, w.y, w.z);
    *ns = make_float3(p.w, q.w, u.w);
    return b;
}

// Boxes of the internal nodes whose subtree holds at most OBB_EXACT
// triangles, one warp per node: the lanes stride over the node's sorted
// triangles for the normal sum, then for the extents (butterfly reductions,
// so every lane holds the same frame).
constexpr int OBB_WARPS = 4;

// A node of at most DF_BUCKET triangles under a parent of at most DF_BUCKET
// lies inside a bucket: the walk tests the bucket's triangles and never reads
// its box (nor visits its parent), so none is made.
__device__ __forceinline__ bool inside_bucket(const int2* __restrict__ range, const int* __restrict__ parent, int i) {
    const int2 r = range[i];
    if (i == 0 || r.y - r.x + 1 > DF_BUCKET) return false;
    const int2 pr = range[parent[i] >> 1];
    return pr.y - pr.x + 1 <= DF_BUCKET;
}

__global__ void __launch_bounds__(OBB_WARPS * 32) k_obb_exact(const int2* __restrict__ range, int n,
                                                              const int* __restrict__ parent,
                                                              const float4* __restrict__ tris,
                                                              float4* __restrict__ obb) {
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * OBB_WARPS + (threadIdx.x >> 5);
    if (i >= n - 1) return;  // warp-uniform
    const int2 r = range[i];
    if (r.y - r.x + 1 > OBB_EXACT || inside_bucket(range, parent, i)) return;
    const unsigned FULL = 0xffffffffu;
    float3 ns = make_float3(0.f, 0.f, 0.f), v[3], nn, edge;
    for (int k = r.x + lane; k <= r.y; k += 32) {
        rec_tri(tris, k, v, &nn, &edge);
        ns.x += nn.x; ns.y += nn.y; ns.z += nn.z;
    }
    for (int o = 16; o > 0; o >>= 1) {
        ns.x += __shfl_xor_sync(FULL, ns.x, o);
        ns.y += __shfl_xor_sync(FULL, ns.y, o);
        ns.z += __shfl_xor_sync(FULL, ns.z, o);
    }
    float3 a1, a2;
    obb_frame(ns, make_float3(NAN, NAN, NAN), a1, a2);
    const float3 a3 = obb_a3(a1, a2);
    rec_tri(tris, r.x, v, &nn, &edge);
    const float3 ref = v[0];
    Ext x;
    x.init();
    for (int k = r.x + lane; k <= r.y; k += 32) {
        rec_tri(tris, k, v, &nn, &edge);
        for (int c = 0; c < 3; ++c) x.add(a1, a2, a3, ref, v[c].x, v[c].y, v[c].z);
    }
    for (int o = 16; o > 0; o >>= 1)
        for (int d = 0; d < 3; ++d) {
            x.lo[d] = fminf(x.lo[d], __shfl_xor_sync(FULL, x.lo[d], o));
            x.hi[d] = fmaxf(x.hi[d], __shfl_xor_sync(FULL, x.hi[d], o));
        }
    if (lane == 0) store_obb(obb, i, x.finish(a1, a2, a3, ref), ns);
}

__device__ void add_corners(Ext& x, float3 a1, float3 a2, float3 a3, float3 r, const Obb& c) {
    const float3 c3 = obb_a3(c.a1, c.a2);
    for (int m = 0; m < 8; ++m) {
        const float t1 = (m & 1) ? c.e.x : 0.f, t2 = (m & 2) ? c.e.y : 0.f, t3 = (m & 4) ? c.e.z : 0.f;
        x.add(a1, a2, a3, r, c.o.x + t1 * c.a1.x + t2 * c.a2.x + t3 * c3.x,
              c.o.y + t1 * c.a1.y + t2 * c.a2.y + t3 * c3.y, c.o.z + t1 * c.a1.z + t2 * c.a2.z + t3 * c3.z);
    }
}

// Boxes of the larger nodes, bottom-up: the second thread to reach a node
// merges its children (normal sums; extents from the children's corners).
// The walks start at the tree's slots (leaves and internal nodes) of at most
// OBB_EXACT triangles whose parent holds more, so each larger node is
// reached once from each child, and no thread climbs the levels below.
__global__ void k_obb_walk(const float4* __restrict__ nodes, const int2* __restrict__ range, int n,
                           const int* __restrict__ parent, int* flags, const float4* __restrict__ tris,
                           float4* obb, int* status) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= 2 * n - 1) return;
    int slot = j;  // internal node j (j < n-1) or leaf j-(n-1)
    {
        const int ps = parent[slot];
        if (ps < 0) return;  // the root
        const int2 pr = range[ps >> 1];
        if (pr.y - pr.x + 1 <= OBB_EXACT) return;  // the parent's box is exact
        if (slot < n - 1) {
            const int2 r = range[slot];
            if (r.y - r.x + 1 > OBB_EXACT) return;  // reached by the walks below it
        }
    }
    for (int level = 0;; ++level) {
        if (level > 128) {
            atomicOr(status, 4);
            return;
        }
        const int ps = parent[slot];
        if (ps < 0) return;  // root done
        const int p = ps >> 1;
        __threadfence();
        if (atomicAdd(&flags[p], 1) == 0) return;
        __threadfence();
        const int2 r = range[p];
        if (r.y - r.x + 1 > OBB_EXACT) {
            Obb cb[2];
            float3 cn[2];
            for (int side = 0; side < 2; ++side) {
                const int c = __float_as_int(__ldcg(&nodes[4 * (int64_t)p + side].w));
                if (c < 0) cb[side] = obb_of_tri(tris, ~c, &cn[side]);
                else cb[side] = load_obb(obb, c, &cn[side]);
            }
            const float3 ns = make_float3(cn[0].x + cn[1].x, cn[0].y + cn[1].y, cn[0].z + cn[1].z);
            float3 a1, a2;
            obb_frame(ns, make_float3(NAN, NAN, NAN), a1, a2);
            const float3 a3 = obb_a3(a1, a2);
            Ext x;
            x.init();
            add_corners(x, a1, a2, a3, cb[0].o, cb[0]);
            add_corners(x, a1, a2, a3, cb[0].o, cb[1]);
            store_obb(obb, p, x.finish(a1, a2, a3, cb[0].o), ns);
        }
        slot = p;
    }
}

// Traversal records (layout at NODE_F4 in mo_df_trav.cuh).
__global__ void k_obb_nodes(const float4* __restrict__ nodes, const int2* __restrict__ range, int n,
                            const int* __restrict__ parent, const float4* __restrict__ tris,
                            const float4* __restrict__ obb, float4* __restrict__ tnodes) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    // a node of at most DF_BUCKET triangles other than the root is never
    // visited (it is its parent's bucket, or inside one)
    if (i != 0 && range[i].y - range[i].x + 1 <= DF_BUCKET) return;
    int cnts[2], ids[2];
    Obb bs[2];
    float3 a3s[2];
    for (int side = 0; side < 2; ++side) {
        const int c = __float_as_int(nodes[4 * (int64_t)i + side].w);
        int id = c, cnt = 0;
        Obb b;
        float3 ns;
        if (c < 0) {
            cnt = 1;
            b = obb_of_tri(tris, ~c, &ns);
        } else {
            const int2 r = range[c];
            b = load_obb(obb, c, &ns);
            if (r.y - r.x + 1 <= DF_BUCKET) {
                id = ~r.x;
                cnt = r.y - r.x + 1;
            }
        }
        bs[side] = b;
        a3s[side] = obb_a3(b.a1, b.a2);
        ids[side] = id;
        cnts[side] = cnt;
    }
    // the two children interleaved (left, right) per float2, origin and
    // extents negated (see NODE_F4)
    const Obb& L = bs[0];
    const Obb& R = bs[1];
    float4* t = tnodes + NODE_F4 * (int64_t)i;
    t[0] = make_float4(-L.o.x, -R.o.x, -L.o.y, -R.o.y);
    t[1] = make_float4(-L.o.z, -R.o.z, -L.e.x, -R.e.x);
    t[2] = make_float4(L.a1.x, R.a1.x, L.a1.y, R.a1.y);
    t[3] = make_float4(L.a1.z, R.a1.z, -L.e.y, -R.e.y);
    t[4] = make_float4(L.a2.x, R.a2.x, L.a2.y, R.a2.y);
    t[5] = make_float4(L.a2.z, R.a2.z, -L.e.z, -R.e.z);
    t[6] = make_float4(a3s[0].x, a3s[1].x, a3s[0].y, a3s[1].y);
    // ids: a node index, or ~first triangle of a bucket (count > 0)
    t[7] = make_float4(a3s[0].z, a3s[1].z, __int_as_float(pack_child(cnts[0] ? ~ids[0] : ids[0], cnts[0])),
                       __int_as_float(pack_child(cnts[1] ? ~ids[1] : ids[1], cnts[1])));
}

// The full grid: one warp per packet of PX x PY x PZ voxels.
template <int PX, int PY, int PZ, bool PAIR_TRIS, bool COUNT = false>
__global__ void __launch_bounds__(TRAV_WARPS * 32) k_df_lbvh(const float4* __restrict__ nodes,
                                                             const float4* __restrict__ tris, int ntri, int N,
                                                             float band, float band2, float* __restrict__ grid,
                                                             int* __restrict__ status,
                                                             unsigned long long* __restrict__ counts) {
    __shared__ int stack[TRAV_WARPS][TRAV_STACK];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    static_assert(PX * PY * PZ == 32, "a packet is one warp");
    const int bx = (N + PX - 1) / PX, by = (N + PY - 1) / PY, bz = (N + PZ - 1) / PZ;
    const int64_t brick = (int64_t)blockIdx.x * TRAV_WARPS + w;
    if (brick >= (int64_t)bx * by * bz) return;  // warp-uniform
    const int ix = (int)(brick % bx), iy = (int)((brick / bx) % by), iz = (int)(brick / ((int64_t)bx * by));
    const int x = ix * PX + (lane % PX), y = iy * PY + ((lane / PX) % PY), z = iz * PZ + lane / (PX * PY);
    const bool valid = x < N && y < N && z < N;
    const float v = df_voxel_value<PAIR_TRIS, COUNT>(nodes, tris, ntri, N, band, band2, x, y, z, valid, stack[w],
                                                     status, counts);
    if (valid) grid[((int64_t)z * N + y) * N + x] = v;
}

// Two voxels per lane: the base packet PX x PY x PZ and the one PZ above it.
template <int PX, int PY, int PZ, bool COUNT = false>
__global__ void __launch_bounds__(TRAV_WARPS * 32) k_df_lbvh2(const float4* __restrict__ nodes,
                                                              const float4* __restrict__ tris, int ntri, int N,
                                                              float band, float band2, float* __restrict__ grid,
                                                              int* __restrict__ status,
                                                              unsigned long long* __restrict__ counts) {
    __shared__ int stack[TRAV_WARPS][TRAV_STACK];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    static_assert(PX * PY * PZ == 32, "a packet is one warp");
    const int bx = (N + PX - 1) / PX, by = (N + PY - 1) / PY, bz = (N + 2 * PZ - 1) / (2 * PZ);
    const int64_t brick = (int64_t)blockIdx.x * TRAV_WARPS + w;
    if (brick >= (int64_t)bx * by * bz) return;  // warp-uniform
    const int ix = (int)(brick % bx), iy = (int)((brick / bx) % by), iz = (int)(brick / ((int64_t)bx * by));
    const int x = ix * PX + (lane % PX), y = iy * PY + ((lane / PX) % PY);
    const int za = iz * 2 * PZ + lane / (PX * PY), zb = za + PZ;
    const bool va = x < N && y < N && za < N, vb = x < N && y < N && zb < N;
    const float2 v = df_voxel_value2<COUNT>(nodes, tris, ntri, N, band, band2, x, y, za, zb, va, vb, stack[w],
                                            status, counts);
    if (va) grid[((int64_t)za * N + y) * N + x] = v.x;
    if (vb) grid[((int64_t)zb * N + y) * N + x] = v.y;
}

template <int PX, int PY, int PZ>
static void launch_df_lbvh2_shape(const float4* nodes, const float4* tris, int ntri, int N, float band, float band2,
                                  float* grid, int* status, unsigned long long* counts, cudaStream_t s) {
    const int64_t bricks = (int64_t)((N + PX - 1) / PX) * ((N + PY - 1) / PY) * ((N + 2 * PZ - 1) / (2 * PZ));
    if (counts)
        k_df_lbvh2<PX, PY, PZ, true><<<ceil_div(bricks, TRAV_WARPS), TRAV_WARPS * 32, 0, s>>>(
            nodes, tris, ntri, N, band, band2, grid, status, counts);
    else
        k_df_lbvh2<PX, PY, PZ><<<ceil_div(bricks, TRAV_WARPS), TRAV_WARPS * 32, 0, s>>>(
            nodes, tris, ntri, N, band, band2, grid, status, nullptr);
    ::mo::note_launch();
}

template <int PX, int PY, int PZ, bool PAIR_TRIS = false>
static void launch_df_lbvh_shape(const float4* nodes, const float4* tris, int ntri, int N, float band, float band2,
                                 float* grid, int* status, unsigned long long* counts, cudaStream_t s) {
    const int64_t bricks = (int64_t)((N + PX - 1) / PX) * ((N + PY - 1) / PY) * ((N + PZ - 1) / PZ);
    if (counts)
        k_df_lbvh<PX, PY, PZ, PAIR_TRIS, true><<<ceil_div(bricks, TRAV_WARPS), TRAV_WARPS * 32, 0, s>>>(
            nodes, tris, ntri, N, band, band2, grid, status, counts);
    else
        k_df_lbvh<PX, PY, PZ, PAIR_TRIS><<<ceil_div(bricks, TRAV_WARPS), TRAV_WARPS * 32, 0, s>>>(
            nodes, tris, ntri, N, band, band2, grid, status, nullptr);
    ::mo::note_launch();
}

// counts != NULL: the counting instantiation (node visits and triangle tests
// per voxel into counts[0], counts[1]); it computes the same grid.
static void launch_df_lbvh(int packet, const float4* nodes, const float4* tris, int ntri, int N, float band,
                           float band2, float* grid, int* status, unsigned long long* counts, cudaStream_t s) {
#define MO_ARGS nodes, tris, ntri, N, band, band2, grid, status, counts, s
    switch (packet) {
        case MO_PACKET_8x4x1: launch_df_lbvh_shape<8, 4, 1>(MO_ARGS); break;
        case MO_PACKET_4x2x4: launch_df_lbvh_shape<4, 2, 4>(MO_ARGS); break;
        case MO_PACKET_2x4x4: launch_df_lbvh_shape<2, 4, 4>(MO_ARGS); break;
        case MO_PACKET_8x2x2: launch_df_lbvh_shape<8, 2, 2>(MO_ARGS); break;
        case MO_PACKET_4x4x4: launch_df_lbvh2_shape<4, 4, 2>(MO_ARGS); break;
        case MO_PACKET_2x4x8: launch_df_lbvh2_shape<2, 4, 4>(MO_ARGS); break;
        case MO_PACKET_8x4x2: launch_df_lbvh2_shape<8, 4, 1>(MO_ARGS); break;
        case MO_PACKET_4x4x2_TRI2: launch_df_lbvh_shape<4, 4, 2, true>(MO_ARGS); break;
        case MO_PACKET_2x4x4_TRI2: launch_df_lbvh_shape<2, 4, 4, true>(MO_ARGS); break;
        default: launch_df_lbvh_shape<4, 4, 2>(MO_ARGS); break;
    }
#undef MO_ARGS
}

// Brute force: one warp per packet of 4 x 4 x 2 voxels with two voxels per
// lane (the packet and the one 2 above it in z, so a warp covers 4 x 4 x 4),
// triangles staged through shared memory in chunks and each tested against
// both voxels of a lane at once on the packed FP32 pipe (tri_d2_2, the same
// IEEE operations per voxel as tri_d2).  A compact packet lets the
// warp-wide plane-distance cull skip most tests; a skipped test could not
// have lowered any lane's best, so every voxel gets the minimum over all
// triangles, as a test of every pair would.
constexpr int BF_THREADS = 256, BF_CHUNK = 128;
constexpr int BF_PX = 4, BF_PY = 4, BF_PZ = 2;

__host__ __device__ __forceinline__ int64_t bf_bricks(int N) {
    return (int64_t)((N + BF_PX - 1) / BF_PX) * ((N + BF_PY - 1) / BF_PY) * ((N + 2 * BF_PZ - 1) / (2 * BF_PZ));
}

__global__ void __launch_bounds__(BF_THREADS) k_df_brute(const float4* __restrict__ tris, int ntri, int N,
                                                         float band, float band2, float* __restrict__ grid) {
    __shared__ float4 sh[BF_CHUNK * TRI_F4];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int bx = (N + BF_PX - 1) / BF_PX, by = (N + BF_PY - 1) / BF_PY;
    const int64_t brick = (int64_t)blockIdx.x * (BF_THREADS / 32) + w;
    // a warp past the last packet still stages triangles with its block
    const bool live = brick < bf_bricks(N);
    const int64_t b = live ? brick : 0;
    const int ix = (int)(b % bx), iy = (int)((b / bx) % by), iz = (int)(b / ((int64_t)bx * by));
    const int x = ix * BF_PX + (lane % BF_PX), y = iy * BF_PY + ((lane / BF_PX) % BF_PY);
    const int za = iz * 2 * BF_PZ + lane / (BF_PX * BF_PY), zb = za + BF_PZ;
    const bool va = live && x < N && y < N && za < N, vb = live && x < N && y < N && zb < N;
    const float Nf = (float)N;
    const float fx = __fdiv_rn((float)x, Nf), fy = __fdiv_rn((float)y, Nf);
    const float2 px = bc2(fx), py = bc2(fy);
    const float2 pz = make_float2(__fdiv_rn((float)za, Nf), __fdiv_rn((float)zb, Nf));
    const VoxelBand ba = voxel_band(x, y, za, N, band, band2), bb = voxel_band(x, y, zb, N, band, band2);
    float2 best = make_float2(ba.bound2, bb.bound2);
    for (int base = 0; base < ntri; base += BF_CHUNK) {
        const int cnt = min(BF_CHUNK, ntri - base);
        __syncthreads();
        for (int k = threadIdx.x; k < cnt * TRI_F4; k += BF_THREADS) sh[k] = tris[TRI_F4 * (int64_t)base + k];
        __syncthreads();
        for (int t = 0; t < cnt; ++t) {
            Tri T;
            T.r0 = sh[TRI_F4 * t]; T.r1 = sh[TRI_F4 * t + 1]; T.r2 = sh[TRI_F4 * t + 2];
            T.r3 = sh[TRI_F4 * t + 3]; T.r4 = sh[TRI_F4 * t + 4];
            const float2 d = tri_d2_2(px, py, pz, T, make_float2(va ? best.x : -1.0f, vb ? best.y : -1.0f));
            best.x = fminf(best.x, d.x);
            best.y = fminf(best.y, d.y);
        }
    }
    if (va) grid[((int64_t)za * N + y) * N + x] = best.x < ba.bound2 ? __fsqrt_rn(best.x) : ba.value;
    if (vb) grid[((int64_t)zb * N + y) * N + x] = best.y < bb.bound2 ? __fsqrt_rn(best.y) : bb.value;
}

// ---------------------------------------------------------------------------
// Scratch layout
// ---------------------------------------------------------------------------
struct BuildScratch {
    float* Vn;
    float4* tris;
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
    int* status;
    int2* range;    // leaves [first, last] of every internal node
    float4* obb;    // 4 float4 per internal node: its oriented box and normal sum
    float4* tnodes; // NODE_F4 float4 per internal node: the traversal records
    size_t bytes;
};

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

static BuildScratch plan_scratch(char* base, int64_t nv, int64_t nf, int method) {
    BuildScratch s;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        char* p = base ? base + o : nullptr;
        o += align256(bytes);
        return p;
    };
    s.status = reinterpret_cast<int*>(take(sizeof(int) * 4));
    s.rootbox = reinterpret_cast<float*>(take(sizeof(float) * 8));
    s.Vn = reinterpret_cast<float*>(take(sizeof(float) * 3 * (size_t)nv));
    s.tris = reinterpret_cast<float4*>(take(sizeof(float4) * TRI_F4 * (size_t)nf));
    if (method == MO_DF_LBVH) {
        s.codes_a = reinterpret_cast<uint32_t*>(take(sizeof(uint32_t) * (size_t)nf));
        s.codes_b = reinterpret_cast<uint32_t*>(take(sizeof(uint32_t) * (size_t)nf));
        s.ids_a = reinterpret_cast<int*>(take(sizeof(int) * (size_t)nf));
        s.ids_b = reinterpret_cast<int*>(take(sizeof(int) * (size_t)nf));
        s.nodes = reinterpret_cast<float4*>(take(sizeof(float4) * 4 * (size_t)(nf > 1 ? nf - 1 : 1)));
        s.boxes = reinterpret_cast<float4*>(take(sizeof(float4) * 2 * (size_t)nf));
        s.parent = reinterpret_cast<int*>(take(sizeof(int) * (size_t)(2 * nf)));
        s.flags = reinterpret_cast<int*>(take(sizeof(int) * (size_t)nf));
        s.hist = reinterpret_cast<int*>(take(sizeof(int) * radix_hist_ints((int)nf)));
        s.range = reinterpret_cast<int2*>(take(sizeof(int2) * (size_t)(nf > 1 ? nf - 1 : 1)));
        s.obb = reinterpret_cast<float4*>(take(sizeof(float4) * 4 * (size_t)(nf > 1 ? nf - 1 : 1)));
        s.tnodes = reinterpret_cast<float4*>(take(sizeof(float4) * NODE_F4 * (size_t)(nf > 1 ? nf - 1 : 1)));
    } else {
        s.codes_a = s.codes_b = nullptr;
        s.ids_a = s.ids_b = nullptr;
        s.nodes = nullptr;
        s.boxes = nullptr;
        s.parent = s.flags = s.hist = nullptr;
        s.range = nullptr;
        s.obb = s.tnodes = nullptr;
    }
    s.bytes = o;
    return s;
}

// The LBVH build up to the traversal inputs (S.tris: sorted triangle
// records, S.tnodes: node records) from the normalised vertices S.Vn.
static cudaError_t issue_tree(const BuildScratch& S, const int32_t* F, int64_t nv, int64_t nf, int* st,
                              cudaStream_t s) {
    k_morton<<<ceil_div(nf, 256), 256, 0, s>>>(S.Vn, F, nf, nv, S.codes_a, S.ids_a, st); ::mo::note_launch();
    cudaError_t e = radix_sort_pairs(S.codes_a, S.ids_a, S.codes_b, S.ids_b, (int)nf, 30, S.hist, s);
    if (e != cudaSuccess) return e;
    k_tri_records<<<ceil_div(nf, 256), 256, 0, s>>>(S.Vn, F, nf, nv, S.ids_a, S.tris, S.boxes); ::mo::note_launch();
    if (nf > 1) {
        k_karras<<<ceil_div(nf - 1, 256), 256, 0, s>>>(S.codes_a, (int)nf, S.nodes, S.parent, S.flags, S.range);
        ::mo::note_launch();
        k_obb_exact<<<ceil_div(nf - 1, OBB_WARPS), OBB_WARPS * 32, 0, s>>>(S.range, (int)nf, S.parent, S.tris,
                                                                           S.obb);
        ::mo::note_launch();
        k_obb_walk<<<ceil_div(2 * nf - 1, 256), 256, 0, s>>>(S.nodes, S.range, (int)nf, S.parent, S.flags, S.tris,
                                                             S.obb,
                                                     st);
        ::mo::note_launch();
        k_obb_nodes<<<ceil_div(nf - 1, 256), 256, 0, s>>>(S.nodes, S.range, (int)nf, S.parent, S.tris, S.obb,
                                                          S.tnodes);
        ::mo::note_launch();
    }
    return cudaGetLastError();
}

}  // namespace mo

using namespace mo;

extern "C" size_t mo_df_tree_bytes(int64_t nf) {
    if (nf <= 0) return 0;
    return sizeof(float4) * ((size_t)tree_nodes_offset_f4(nf) + NODE_F4 * (size_t)(nf > 1 ? nf - 1 : 1));
}

extern "C" size_t mo_df_tree_scratch_bytes(int64_t nv, int64_t nf) {
    if (nv < 0 || nf < 0) return 0;
    return plan_scratch(nullptr, nv, nf, MO_DF_LBVH).bytes;
}

extern "C" int mo_df_tree_build(const float* V, int64_t nv, const int32_t* F, int64_t nf, const double* params4,
                                void* scratch, size_t scratch_bytes, void* tree_out, int32_t* status_out,
                                void* stream) {
    MO_CHECK_ARG(nv > 0 && nf > 0, "target mesh must have vertices and faces (nv=%lld nf=%lld)", (long long)nv,
                 (long long)nf);
    MO_CHECK_ARG(nf <= MAX_TREE_TRIANGLES && nv < ((int64_t)1 << 31), "target mesh too large for the tree");
    MO_CHECK_ARG(V && F && params4 && scratch && tree_out && status_out, "null pointer");
    MO_CHECK_ARG((reinterpret_cast<uintptr_t>(tree_out) & 15) == 0, "tree_out must be 16-byte aligned");
    const size_t need = plan_scratch(nullptr, nv, nf, MO_DF_LBVH).bytes;
    if (scratch_bytes < need) {
        set_error("tree build scratch too small: %zu < %zu", scratch_bytes, need);
        return MO_ERR_SCRATCH;
    }
    cudaStream_t s = as_stream(stream);
    BuildScratch S = plan_scratch(reinterpret_cast<char*>(scratch), nv, nf, MO_DF_LBVH);
    float4* out = reinterpret_cast<float4*>(tree_out);
    // the records are written straight into the output
    S.tris = out;
    S.tnodes = out + tree_nodes_offset_f4(nf);
    k_normalize_copy<<<ceil_div(3 * nv, 256), 256, 0, s>>>(V, nv, params4, S.Vn); ::mo::note_launch();
    cudaError_t e = issue_tree(S, F, nv, nf, reinterpret_cast<int*>(status_out), s);
    if (e != cudaSuccess) return cuda_status(e, "mo_df_tree_build");
    return MO_OK;
}

extern "C" int mo_bbox(const float* V, int64_t n, int32_t* bbox6, void* stream) {
    MO_CHECK_ARG(n >= 0, "negative vertex count");
    MO_CHECK_ARG(bbox6 && (n == 0 || V), "null pointer");
    cudaStream_t s = as_stream(stream);
    k_bbox_init<<<1, 32, 0, s>>>(bbox6); ::mo::note_launch();
    if (n > 0) {
        const int blocks = std::min(ceil_div(n, 256), 4 * device_sm_count());
        k_bbox<<<blocks, 256, 0, s>>>(V, n, bbox6); ::mo::note_launch();
    }
    MO_LAUNCH_CHECK("k_bbox");
    return MO_OK;
}

extern "C" int mo_norm_params(const int32_t* bbox6, double* params4, void* stream) {
    MO_CHECK_ARG(bbox6 && params4, "null pointer");
    k_norm_params<<<1, 1, 0, as_stream(stream)>>>(bbox6, params4); ::mo::note_launch();
    MO_LAUNCH_CHECK("k_norm_params");
    return MO_OK;
}

extern "C" int mo_normalize(float* V, int64_t n, const double* params4, int inverse, void* stream) {
    MO_CHECK_ARG(n >= 0, "negative vertex count");
    if (n == 0) return MO_OK;
    MO_CHECK_ARG(V && params4, "null pointer");
    k_normalize<<<ceil_div(3 * n, 256), 256, 0, as_stream(stream)>>>(V, n, params4, inverse); ::mo::note_launch();
    MO_LAUNCH_CHECK("k_normalize");
    return MO_OK;
}

extern "C" float mo_df_loss_band(int N) {
    if (N < 2) return 0.0f;
    return (float)(0.2 + std::sqrt(3.0) / (double)N + 1e-3);
}

extern "C" int mo_df_method_for(int64_t nf, int N) {
    // Brute force tests every voxel against every triangle; below ~3e8 pair
    // tests it beats building and walking the tree.
    const double pairs = (double)nf * (double)N * N * N;
    return (nf <= 64 || pairs <= 3.0e8) ? MO_DF_BRUTE : MO_DF_LBVH;
}

extern "C" size_t mo_df_build_scratch_bytes(int64_t nv, int64_t nf, int N, int method) {
    if (nv < 0 || nf < 0) return 0;
    if (method == MO_DF_AUTO) method = mo_df_method_for(nf, N);
    return plan_scratch(nullptr, nv, nf, method).bytes;
}

__global__ void k_add_u64(unsigned long long* __restrict__ c, unsigned long long v) { atomicAdd(c, v); }

static int df_build_impl(const float* V, int64_t nv, const int32_t* F, int64_t nf, int N, const double* params4,
                         const MoDfOptions* opt, void* scratch, size_t scratch_bytes, float* grid_out,
                         int32_t* status_out, unsigned long long* counts, void* stream) {
    int method = opt ? opt->method : MO_DF_AUTO;
    const int packet = opt ? opt->packet : MO_PACKET_4x4x2;
    const float band = opt ? opt->band : 0.0f;
    MO_CHECK_ARG(packet >= MO_PACKET_4x4x2 && packet <= MO_PACKET_LAST, "unknown packet shape %d", packet);
    MO_CHECK_ARG(band >= 0.0f && band <= 4.0f, "band must be in [0, 4] (0: exact grid), got %g", (double)band);
    const float band2 = band > 0.0f ? band * band : FLT_MAX;
    MO_CHECK_ARG(nv > 0 && nf > 0, "target mesh must have vertices and faces (nv=%lld nf=%lld)", (long long)nv,
                 (long long)nf);
    MO_CHECK_ARG(nf < ((int64_t)1 << 30) && nv < ((int64_t)1 << 31), "target mesh too large");
    MO_CHECK_ARG(N >= 2 && N <= 2048, "grid resolution out of range (%d)", N);
    MO_CHECK_ARG(V && F && params4 && grid_out, "null pointer");
    MO_CHECK_ARG(method == MO_DF_AUTO || method == MO_DF_BRUTE || method == MO_DF_LBVH, "unknown method %d", method);
    if (method == MO_DF_AUTO) method = mo_df_method_for(nf, N);
    MO_CHECK_ARG(method != MO_DF_LBVH || nf <= MAX_TREE_TRIANGLES, "target mesh too large for the LBVH (%lld > %lld)",
                 (long long)nf, (long long)MAX_TREE_TRIANGLES);
    cudaStream_t s = as_stream(stream);
    const size_t need = plan_scratch(nullptr, nv, nf, method).bytes;
    void* owned = nullptr;
    if (!scratch) {
        MO_CUDA(cudaMallocAsync(&owned, need, s));
        scratch = owned;
    } else if (scratch_bytes < need) {
        set_error("DF build scratch too small: %zu < %zu", scratch_bytes, need);
        return MO_ERR_SCRATCH;
    }
    BuildScratch S = plan_scratch(reinterpret_cast<char*>(scratch), nv, nf, method);
    int rc = MO_OK;
    auto fail = [&](cudaError_t e, const char* where) {
        rc = cuda_status(e, where);
    };
    int* st = status_out ? reinterpret_cast<int*>(status_out) : S.status;
    do {
        cudaError_t e = cudaSuccess;
        if (!status_out) {
            e = cudaMemsetAsync(S.status, 0, sizeof(int) * 4, s);
            if (e != cudaSuccess) { fail(e, "memset"); break; }
        }
        k_normalize_copy<<<ceil_div(3 * nv, 256), 256, 0, s>>>(V, nv, params4, S.Vn); ::mo::note_launch();
        if (method == MO_DF_BRUTE) {
            k_check_faces<<<ceil_div(nf, 256), 256, 0, s>>>(F, nf, nv, st); ::mo::note_launch();
            k_tri_records<<<ceil_div(nf, 256), 256, 0, s>>>(S.Vn, F, nf, nv, nullptr, S.tris, nullptr); ::mo::note_launch();
            const int64_t nvox = (int64_t)N * N * N;
            k_df_brute<<<ceil_div(bf_bricks(N), BF_THREADS / 32), BF_THREADS, 0, s>>>(S.tris, (int)nf, N, band,
                                                                                   band2, grid_out);
            ::mo::note_launch();
            if (counts) {  // every voxel tests every triangle
                k_add_u64<<<1, 1, 0, s>>>(counts + 1, (unsigned long long)nvox * (unsigned long long)nf);
                ::mo::note_launch();
            }
        } else {
            e = issue_tree(S, F, nv, nf, st, s);
            if (e != cudaSuccess) { fail(e, "LBVH build"); break; }
            launch_df_lbvh(packet, S.tnodes, S.tris, (int)nf, N, band, band2, grid_out, st, counts, s);
        }
        e = cudaGetLastError();
        if (e != cudaSuccess) { fail(e, "df build kernels"); break; }
    } while (0);
    if (rc == MO_OK && !status_out) {
        int status = 0;
        cudaError_t e = cudaMemcpyAsync(&status, S.status, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = cuda_status(e, "df build status");
        else if (status & 1) { set_error("face index out of range [0, %lld)", (long long)nv); rc = MO_ERR_DEVICE; }
        else if (status & 2) { set_error("LBVH traversal stack overflow"); rc = MO_ERR_DEVICE; }
        else if (status & 4) { set_error("LBVH is malformed (refit or traversal bound exceeded)"); rc = MO_ERR_DEVICE; }
    }
    if (owned) cudaFreeAsync(owned, s);
    return rc;
}

extern "C" int mo_df_build_ex(const float* V, int64_t nv, const int32_t* F, int64_t nf, int N,
                              const double* params4, const MoDfOptions* opt, void* scratch, size_t scratch_bytes,
                              float* grid_out, int32_t* status_out, void* stream) {
    return df_build_impl(V, nv, F, nf, N, params4, opt, scratch, scratch_bytes, grid_out, status_out, nullptr,
                         stream);
}

extern "C" int mo_df_build_count(const float* V, int64_t nv, const int32_t* F, int64_t nf, int N,
                                 const double* params4, const MoDfOptions* opt, void* scratch, size_t scratch_bytes,
                                 float* grid_out, int32_t* status_out, uint64_t* counts, void* stream) {
    MO_CHECK_ARG(counts, "null counts pointer");
    return df_build_impl(V, nv, F, nf, N, params4, opt, scratch, scratch_bytes, grid_out, status_out,
                         reinterpret_cast<unsigned long long*>(counts), stream);
}

extern "C" int mo_df_build(const float* V, int64_t nv, const int32_t* F, int64_t nf, int N, const double* params4,
                           int method, void* scratch, size_t scratch_bytes, float* grid_out, int32_t* status_out,
                           void* stream) {
    MoDfOptions opt;
    std::memset(&opt, 0, sizeof(opt));
    opt.method = method;
    opt.packet = MO_PACKET_4x4x2;
    return mo_df_build_ex(V, nv, F, nf, N, params4, &opt, scratch, scratch_bytes, grid_out, status_out, stream);
}

extern "C" int mo_lbvh_build(const float* V, int64_t nv, const int32_t* F, int64_t nf, const double* params4,
                             void* scratch, size_t scratch_bytes, uint32_t* sorted_codes, int32_t* order,
                             int32_t* left, int32_t* right, float* root_box, void* stream) {
    MO_CHECK_ARG(nv > 0 && nf > 0, "empty mesh");
    MO_CHECK_ARG(nf < ((int64_t)1 << 30) && nv < ((int64_t)1 << 31), "mesh too large");
    MO_CHECK_ARG(V && F && params4 && sorted_codes && order, "null pointer");
    MO_CHECK_ARG(nf == 1 || (left && right), "null child arrays");
    cudaStream_t s = as_stream(stream);
    const size_t need = plan_scratch(nullptr, nv, nf, MO_DF_LBVH).bytes;
    void* owned = nullptr;
    if (!scratch) {
        MO_CUDA(cudaMallocAsync(&owned, need, s));
        scratch = owned;
    } else if (scratch_bytes < need) {
        set_error("LBVH scratch too small: %zu < %zu", scratch_bytes, need);
        return MO_ERR_SCRATCH;
    }
    BuildScratch S = plan_scratch(reinterpret_cast<char*>(scratch), nv, nf, MO_DF_LBVH);
    int rc = MO_OK;
    cudaError_t e = cudaMemsetAsync(S.status, 0, sizeof(int) * 4, s);
    if (e == cudaSuccess) {
        k_normalize_copy<<<ceil_div(3 * nv, 256), 256, 0, s>>>(V, nv, params4, S.Vn); ::mo::note_launch();
        k_morton<<<ceil_div(nf, 256), 256, 0, s>>>(S.Vn, F, nf, nv, S.codes_a, S.ids_a, S.status); ::mo::note_launch();
        e = radix_sort_pairs(S.codes_a, S.ids_a, S.codes_b, S.ids_b, (int)nf, 30, S.hist, s);
    }
    if (e == cudaSuccess) {
        k_tri_records<<<ceil_div(nf, 256), 256, 0, s>>>(S.Vn, F, nf, nv, S.ids_a, S.tris, S.boxes); ::mo::note_launch();
        if (nf > 1) {
            k_karras<<<ceil_div(nf - 1, 256), 256, 0, s>>>(S.codes_a, (int)nf, S.nodes, S.parent, S.flags, nullptr);
            ::mo::note_launch();
            k_refit<<<ceil_div(nf, 256), 256, 0, s>>>(S.boxes, (int)nf, S.nodes, S.parent, S.flags, S.rootbox,
                                                      S.status); ::mo::note_launch();
        }
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(sorted_codes, S.codes_a, 4 * nf, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(order, S.ids_a, 4 * nf, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && nf > 1) {
        // child indices live in the .w lanes of node words 0 and 1
        e = cudaMemcpy2DAsync(left, sizeof(int32_t), reinterpret_cast<const char*>(S.nodes) + 12, 64, sizeof(int32_t),
                              (size_t)(nf - 1), cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpy2DAsync(right, sizeof(int32_t), reinterpret_cast<const char*>(S.nodes) + 28, 64,
                                  sizeof(int32_t), (size_t)(nf - 1), cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess && root_box)
            e = cudaMemcpyAsync(root_box, S.rootbox, 6 * sizeof(float), cudaMemcpyDeviceToDevice, s);
    }
    if (e != cudaSuccess) rc = cuda_status(e, "mo_lbvh_build");
    if (rc == MO_OK) {
        int status = 0;
        e = cudaMemcpyAsync(&status, S.status, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = cuda_status(e, "mo_lbvh_build status");
        else if (status & 1) { set_error("face index out of range [0, %lld)", (long long)nv); rc = MO_ERR_DEVICE; }
    }
    if (owned) cudaFreeAsync(owned, s);
    return rc;
}

// ---------------------------------------------------------------------------
// Allocation-free distance-field build.
//
// Some callers cannot allocate device memory while they run: code executing
// inside another runtime or plugin host that owns the whole device memory
// pool, or a real-time loop whose policy forbids allocation after start-up.
// For them the build's scratch lives in one fixed, file-scope device array
// that every GPU loading this library holds until the process exits.
// In host code the array's name is only a host-side stand-in; its device
// address is looked up once per device with cudaGetSymbolAddress.
// ---------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_df_noalloc_scratch[MO_DF_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_addr[kMaxDevices] = {};
}  // namespace

// Device address of the fixed scratch on the current device, looked up on the
// first call made with that device current and cached for the process: the
// cached address is not valid across a cudaDeviceReset of that device.
static int noalloc_scratch_address(void** out) {
    int dev = 0;
    MO_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("device ordinal %d is outside the %d devices this library tracks", dev, kMaxDevices);
        return MO_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_df_noalloc_scratch);
        if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(g_df_noalloc_scratch)");
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return MO_OK;
}

extern "C" size_t mo_df_noalloc_scratch_capacity(void) { return MO_DF_NOALLOC_SCRATCH_BYTES; }

extern "C" int mo_df_build_noalloc(const float* V, int64_t nv, const int32_t* F, int64_t nf, int N,
                                   const double* params4, float* grid_linear_out, void* stream) {
    MO_CHECK_ARG(nv > 0 && nf > 0, "target mesh must have vertices and faces (nv=%lld nf=%lld)", (long long)nv,
                 (long long)nf);
    MO_CHECK_ARG(nf < ((int64_t)1 << 30) && nv < ((int64_t)1 << 31), "target mesh too large");
    MO_CHECK_ARG(N >= 2 && N <= 2048, "grid resolution out of range (%d)", N);
    const int method = mo_df_method_for(nf, N);
    const size_t need = plan_scratch(nullptr, nv, nf, method).bytes;
    if (need > (size_t)MO_DF_NOALLOC_SCRATCH_BYTES) {
        set_error("mo_df_build_noalloc: a target with %lld vertices and %lld faces needs %zu bytes of scratch, "
                  "more than the fixed %zu-byte array; use mo_df_build with caller scratch",
                  (long long)nv, (long long)nf, need, (size_t)MO_DF_NOALLOC_SCRATCH_BYTES);
        return MO_ERR_SCRATCH;
    }
    void* scratch = nullptr;
    const int rc = noalloc_scratch_address(&scratch);
    if (rc != MO_OK) return rc;
    // status_out == NULL: the build reads its status word from the fixed
    // array (zeroed at the start of every call) and synchronises `stream`.
    return mo_df_build(V, nv, F, nf, N, params4, method, scratch, (size_t)MO_DF_NOALLOC_SCRATCH_BYTES,
                       grid_linear_out, nullptr, stream);
}
