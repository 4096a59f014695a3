// Nearest-triangle queries of the distance-field build, shared by the
// full-grid build (mo_dfbuild.cu) and the on-demand cell fills
// (mo_lazydf.cu): the triangle records and their exact squared-distance
// query, the oriented-box bound of a tree child, and the warp-packet walk
// of the tree that gives one voxel's stored value.
// Reference: igl::point_mesh_squared_distance as called by
// Mesh::ConstructDistanceField (src/lib/mesh.cc:106-152).
#pragma once

#include <cfloat>

#include "mo_common.cuh"

namespace mo {

// ---------------------------------------------------------------------------
// Triangle records, 5 float4 (80 B), in a per-triangle 2D frame so a query
// costs a projection and three 2D segment distances:
//   r0 = (a, bx)  r1 = (ex, cx)  r2 = (ey, cy)  r3 = (n, 1)
//   r4 = (1/bx, 1/|ac|^2, 1/|bc|^2, cx - bx)
// with ex = ab/|ab|, n the unit normal, ey = n x ex, and the triangle at
// A=(0,0), B=(bx,0), C=(cx,cy), cy > 0 in (ex, ey).  A degenerate triangle
// (zero area or zero-length ab) keeps its vertices instead and is measured
// by its three segments:
//   r0 = (a, 0)  r1 = (b, 0)  r2 = (c, 0)  r3 = (0, 0, 0, 0)
//   r4 = (1/|ab|^2, 1/|bc|^2, 1/|ca|^2, 0)   (0 for a zero-length segment)
// ---------------------------------------------------------------------------
struct Tri {
    float4 r0, r1, r2, r3, r4;
};
constexpr int TRI_F4 = 5;

// The query arithmetic is written with explicit fmaf / __fmul_rn / __fadd_rn
// so that every kernel that inlines it (LBVH traversal, brute force) rounds
// identically and the two build methods give the same grid bit for bit.
__device__ __forceinline__ float dot3e(float ax, float ay, float az, float bx, float by, float bz) {
    return fmaf(az, bz, fmaf(ay, by, __fmul_rn(ax, bx)));
}

__device__ __forceinline__ float seg3_d2(float px, float py, float pz, float4 a, float4 b, float inv_l2) {
    const float ex = __fsub_rn(b.x, a.x), ey = __fsub_rn(b.y, a.y), ez = __fsub_rn(b.z, a.z);
    const float apx = __fsub_rn(px, a.x), apy = __fsub_rn(py, a.y), apz = __fsub_rn(pz, a.z);
    float t = __fmul_rn(dot3e(apx, apy, apz, ex, ey, ez), inv_l2);
    t = fminf(fmaxf(t, 0.f), 1.f);
    const float qx = fmaf(-t, ex, apx), qy = fmaf(-t, ey, apy), qz = fmaf(-t, ez, apz);
    return dot3e(qx, qy, qz, qx, qy, qz);
}

// Squared distance from p to the triangle.  `cut` is this lane's current
// best: when no lane of the (converged) warp can beat its best because the
// plane distance alone is too large, the in-plane part is skipped and
// FLT_MAX returned.  The record is warp-uniform, so both branches are too.
__device__ __forceinline__ float tri_d2(float px, float py, float pz, const Tri& T, float cut) {
    if (T.r3.w != 0.f) {
        const float qx = __fsub_rn(px, T.r0.x), qy = __fsub_rn(py, T.r0.y), qz = __fsub_rn(pz, T.r0.z);
        const float h = dot3e(qx, qy, qz, T.r3.x, T.r3.y, T.r3.z);
        const float h2 = __fmul_rn(h, h);
        if (!__any_sync(0xffffffffu, h2 < cut)) return FLT_MAX;
        const float x = dot3e(qx, qy, qz, T.r1.x, T.r1.y, T.r1.z);
        const float y = dot3e(qx, qy, qz, T.r2.x, T.r2.y, T.r2.z);
        const float bx = T.r0.w, cx = T.r1.w, cy = T.r2.w, ebx = T.r4.w;
        const float y2 = __fmul_rn(y, y);
        // A-B along the x axis
        float t = fminf(fmaxf(__fmul_rn(x, T.r4.x), 0.f), 1.f);
        float dx = fmaf(-t, bx, x);
        float d = fmaf(dx, dx, y2);
        // A-C
        t = fminf(fmaxf(__fmul_rn(fmaf(x, cx, __fmul_rn(y, cy)), T.r4.y), 0.f), 1.f);
        dx = fmaf(-t, cx, x);
        float dy = fmaf(-t, cy, y);
        d = fminf(d, fmaf(dx, dx, __fmul_rn(dy, dy)));
        // B-C
        const float xb = __fsub_rn(x, bx);
        t = fminf(fmaxf(__fmul_rn(fmaf(xb, ebx, __fmul_rn(y, cy)), T.r4.z), 0.f), 1.f);
        dx = fmaf(-t, ebx, xb);
        dy = fmaf(-t, cy, y);
        d = fminf(d, fmaf(dx, dx, __fmul_rn(dy, dy)));
        // inside: left of A->B, B->C and C->A (counter-clockwise in the frame)
        const bool inside = (y >= 0.f) && (fmaf(ebx, y, -__fmul_rn(cy, xb)) >= 0.f) &&
                            (fmaf(cy, x, -__fmul_rn(cx, y)) >= 0.f);
        return inside ? h2 : __fadd_rn(h2, d);
    }
    float d = seg3_d2(px, py, pz, T.r0, T.r1, T.r4.x);
    d = fminf(d, seg3_d2(px, py, pz, T.r1, T.r2, T.r4.y));
    d = fminf(d, seg3_d2(px, py, pz, T.r2, T.r0, T.r4.z));
    return d;
}

__device__ __forceinline__ Tri load_tri(const float4* __restrict__ tris, int i) {
    const float4* p = tris + TRI_F4 * (int64_t)i;
    Tri t;
    t.r0 = __ldg(p); t.r1 = __ldg(p + 1); t.r2 = __ldg(p + 2); t.r3 = __ldg(p + 3); t.r4 = __ldg(p + 4);
    return t;
}

// a3 exactly as the traversal computes it
__device__ __forceinline__ float3 obb_a3(float3 a1, float3 a2) {
    return make_float3(__fsub_rn(__fmul_rn(a1.y, a2.z), __fmul_rn(a1.z, a2.y)),
                       __fsub_rn(__fmul_rn(a1.z, a2.x), __fmul_rn(a1.x, a2.z)),
                       __fsub_rn(__fmul_rn(a1.x, a2.y), __fmul_rn(a1.y, a2.x)));
}

__device__ __forceinline__ float dotf3(float3 a, float x, float y, float z) {
    return fmaf(a.z, z, fmaf(a.y, y, __fmul_rn(a.x, x)));
}

// Traversal record of an internal node: NODE_F4 float4 (128 bytes, one
// cache line when the record array is 128-byte aligned) holding both
// children's oriented boxes interleaved, each float2 (left, right), so that
// one packed FP32 pass (FFMA2 / FADD2) bounds both children:
//   w0 = (-o.x, -o.y)  w1 = (-o.z, -e.x)  w2 = (a1.x, a1.y)  w3 = (a1.z, -e.y)
//   w4 = (a2.x, a2.y)  w5 = (a2.z, -e.z)  w6 = (a3.x, a3.y)  w7 = (a3.z, id)
// where each named component is a (left, right) pair: w0 = (-oL.x, -oR.x,
// -oL.y, -oR.y) and so on.  o: a box's origin corner, a1..a3 its axes
// (a3 = obb_a3(a1, a2), stored so the walk does not recompute it), e its
// extents (origin and extents stored negated: the walk adds them); id (an
// int) = index << 3 | count: an internal node (count 0) and its index, or a
// bucket of `count` (1..DF_BUCKET) sorted triangles from triangle `index`.
constexpr int NODE_F4 = 8;
constexpr int64_t MAX_TREE_TRIANGLES = (int64_t)1 << 27;  // index << 3 stays an int

// a child's id: `index` is its node (count 0) or its bucket's first triangle
__host__ __device__ __forceinline__ int pack_child(int index, int count) { return (index << 3) | count; }
// bucket size of a packed child (0: internal node)
__device__ __forceinline__ int child_count(int packed) { return packed & 7; }
// the child's node index, or the first triangle of its bucket
__device__ __forceinline__ int child_index(int packed) { return packed >> 3; }

// Offset (float4) of the node records behind the triangle records in a
// traversal tree buffer (mo_df_tree_build): the triangles rounded up to 128
// bytes, so that a 128-byte aligned buffer aligns every node record.
__host__ __device__ __forceinline__ int64_t tree_nodes_offset_f4(int64_t ntri) {
    return (TRI_F4 * ntri + 7) & ~(int64_t)7;
}

__device__ __forceinline__ float2 lo2(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.z, v.w); }

// Squared distances from p (broadcast in Px, Py, Pz) to the left and right
// child's boxes of a record: the bound the traversal uses, both children in
// one packed pass (each half the one-box arithmetic in the same order).
__device__ __forceinline__ float2 obb_pair_d2(float2 Px, float2 Py, float2 Pz, float4 w0, float4 w1, float4 w2,
                                              float4 w3, float4 w4, float4 w5, float4 w6, float4 w7) {
    const float2 qx = __fadd2_rn(Px, lo2(w0)), qy = __fadd2_rn(Py, hi2(w0)), qz = __fadd2_rn(Pz, lo2(w1));
    const float2 t1 = __ffma2_rn(lo2(w3), qz, __ffma2_rn(hi2(w2), qy, __fmul2_rn(lo2(w2), qx)));
    const float2 t2 = __ffma2_rn(lo2(w5), qz, __ffma2_rn(hi2(w4), qy, __fmul2_rn(lo2(w4), qx)));
    const float2 t3 = __ffma2_rn(lo2(w7), qz, __ffma2_rn(hi2(w6), qy, __fmul2_rn(lo2(w6), qx)));
    const float2 u1 = __fadd2_rn(t1, hi2(w1)), u2 = __fadd2_rn(t2, hi2(w3)), u3 = __fadd2_rn(t3, hi2(w5));
    const float2 s1 = make_float2(fmaxf(fmaxf(-t1.x, u1.x), 0.f), fmaxf(fmaxf(-t1.y, u1.y), 0.f));
    const float2 s2 = make_float2(fmaxf(fmaxf(-t2.x, u2.x), 0.f), fmaxf(fmaxf(-t2.y, u2.y), 0.f));
    const float2 s3 = make_float2(fmaxf(fmaxf(-t3.x, u3.x), 0.f), fmaxf(fmaxf(-t3.y, u3.y), 0.f));
    return __ffma2_rn(s3, s3, __ffma2_rn(s2, s2, __fmul2_rn(s1, s1)));
}

// ---------------------------------------------------------------------------
// Warp-packet traversal: one warp = a 4x4x2 brick of voxels.  The warp walks
// the tree together (node and triangle loads are warp-uniform broadcasts);
// a child is visited when any lane's box distance beats that lane's best.
// ---------------------------------------------------------------------------
constexpr int TRAV_WARPS = 4;
constexpr float kSlack = 2e-6f;

// (sqrt(best) + kSlack)^2: the squared-distance bound a box must beat.
__device__ __forceinline__ float slack_bound(float best) { return best + kSlack * (2.f * sqrtf(best) + kSlack); }
constexpr int TRAV_STACK = 64;


// Packet shapes (voxels per warp along x, y, z; product 32), selectable per
// launch: MO_PACKET_4x4x2 (default), 8x4x1, 4x2x4, 2x4x4, 8x2x2.
// Band: with band > 0 a voxel whose distance is not below `band` stores
// `band` itself, except in the two lowest layers along each axis (x, y or
// z <= 1), where lookups just below the cube extrapolate: there the band is
// band + 13/N; band2 = band^2 (FLT_MAX for none).
struct VoxelBand {
    float bound2;  // squared distance a triangle must beat (FLT_MAX: none)
    float value;   // stored when none does
};

__device__ __forceinline__ VoxelBand voxel_band(int x, int y, int z, int N, float band, float band2) {
    VoxelBand b;
    if (band2 == FLT_MAX) {
        b.bound2 = FLT_MAX;
        b.value = 0.f;
    } else if (x <= 1 || y <= 1 || z <= 1) {
        b.value = __fadd_rn(band, __fdiv_rn(13.0f, (float)N));
        b.bound2 = __fmul_rn(b.value, b.value);
    } else {
        b.bound2 = band2;
        b.value = band;
    }
    return b;
}

// ---------------------------------------------------------------------------
// Two voxels per lane, on the packed FP32 pipe (FFMA2 / FADD2 / FMUL2 of
// sm_100+): one walk of the tree serves 64 voxels, the node and triangle
// loads, votes and stack are shared, and every per-voxel operation is the
// same IEEE operation as in the one-voxel code, in the same order, so each
// voxel gets the same value bit for bit.  Subtracting a uniform scalar is
// written as adding its negation (a - b == a + (-b) exactly), and
// fmaf(-t, b, x) as fma(t, -b, x) (the same exact product).
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 bc2(float s) { return make_float2(s, s); }

__device__ __forceinline__ float2 dot3e2(float2 ax, float2 ay, float2 az, float bx, float by, float bz) {
    return __ffma2_rn(az, bc2(bz), __ffma2_rn(ay, bc2(by), __fmul2_rn(ax, bc2(bx))));
}

__device__ __forceinline__ float2 dot3e2(float2 ax, float2 ay, float2 az) {
    return __ffma2_rn(az, az, __ffma2_rn(ay, ay, __fmul2_rn(ax, ax)));
}

__device__ __forceinline__ float2 clamp01_2(float2 t) {
    return make_float2(fminf(fmaxf(t.x, 0.f), 1.f), fminf(fmaxf(t.y, 0.f), 1.f));
}

__device__ __forceinline__ float2 fmin2(float2 a, float2 b) { return make_float2(fminf(a.x, b.x), fminf(a.y, b.y)); }

__device__ __forceinline__ float2 seg3_d2_2(float2 px, float2 py, float2 pz, float4 a, float4 b, float inv_l2) {
    const float ex = __fsub_rn(b.x, a.x), ey = __fsub_rn(b.y, a.y), ez = __fsub_rn(b.z, a.z);
    const float2 apx = __fadd2_rn(px, bc2(-a.x)), apy = __fadd2_rn(py, bc2(-a.y)), apz = __fadd2_rn(pz, bc2(-a.z));
    const float2 t = clamp01_2(__fmul2_rn(dot3e2(apx, apy, apz, ex, ey, ez), bc2(inv_l2)));
    const float2 qx = __ffma2_rn(t, bc2(-ex), apx), qy = __ffma2_rn(t, bc2(-ey), apy),
                 qz = __ffma2_rn(t, bc2(-ez), apz);
    return dot3e2(qx, qy, qz);
}

// tri_d2 for two points; the plane-distance cull skips the rest when no
// voxel of the warp can beat its best.
__device__ __forceinline__ float2 tri_d2_2(float2 px, float2 py, float2 pz, const Tri& T, float2 cut) {
    if (T.r3.w != 0.f) {
        const float2 qx = __fadd2_rn(px, bc2(-T.r0.x)), qy = __fadd2_rn(py, bc2(-T.r0.y)),
                     qz = __fadd2_rn(pz, bc2(-T.r0.z));
        const float2 h = dot3e2(qx, qy, qz, T.r3.x, T.r3.y, T.r3.z);
        const float2 h2 = __fmul2_rn(h, h);
        if (!__any_sync(0xffffffffu, h2.x < cut.x || h2.y < cut.y)) return bc2(FLT_MAX);
        const float2 x = dot3e2(qx, qy, qz, T.r1.x, T.r1.y, T.r1.z);
        const float2 y = dot3e2(qx, qy, qz, T.r2.x, T.r2.y, T.r2.z);
        const float bx = T.r0.w, cx = T.r1.w, cy = T.r2.w, ebx = T.r4.w;
        const float2 y2 = __fmul2_rn(y, y);
        // A-B along the x axis
        float2 t = clamp01_2(__fmul2_rn(x, bc2(T.r4.x)));
        float2 dx = __ffma2_rn(t, bc2(-bx), x);
        float2 d = __ffma2_rn(dx, dx, y2);
        // A-C
        t = clamp01_2(__fmul2_rn(__ffma2_rn(x, bc2(cx), __fmul2_rn(y, bc2(cy))), bc2(T.r4.y)));
        dx = __ffma2_rn(t, bc2(-cx), x);
        float2 dy = __ffma2_rn(t, bc2(-cy), y);
        d = fmin2(d, __ffma2_rn(dx, dx, __fmul2_rn(dy, dy)));
        // B-C
        const float2 xb = __fadd2_rn(x, bc2(-bx));
        t = clamp01_2(__fmul2_rn(__ffma2_rn(xb, bc2(ebx), __fmul2_rn(y, bc2(cy))), bc2(T.r4.z)));
        dx = __ffma2_rn(t, bc2(-ebx), xb);
        dy = __ffma2_rn(t, bc2(-cy), y);
        d = fmin2(d, __ffma2_rn(dx, dx, __fmul2_rn(dy, dy)));
        // inside: left of A->B, B->C and C->A
        const float2 sb = __ffma2_rn(bc2(ebx), y, __fmul2_rn(bc2(-cy), xb));
        const float2 sc = __ffma2_rn(bc2(cy), x, __fmul2_rn(bc2(-cx), y));
        const float2 hd = __fadd2_rn(h2, d);
        const bool inx = (y.x >= 0.f) && (sb.x >= 0.f) && (sc.x >= 0.f);
        const bool iny = (y.y >= 0.f) && (sb.y >= 0.f) && (sc.y >= 0.f);
        return make_float2(inx ? h2.x : hd.x, iny ? h2.y : hd.y);
    }
    float2 d = seg3_d2_2(px, py, pz, T.r0, T.r1, T.r4.x);
    d = fmin2(d, seg3_d2_2(px, py, pz, T.r1, T.r2, T.r4.y));
    d = fmin2(d, seg3_d2_2(px, py, pz, T.r2, T.r0, T.r4.z));
    return d;
}

// tri_d2 of one point against two triangles (both non-degenerate), each
// element the one-triangle code's operations in its order; the cull skips
// the rest when no lane can beat its best with either.
__device__ __forceinline__ float2 tri_d2_t2(float px, float py, float pz, const Tri& A, const Tri& B, float cut) {
    const float2 qx = __fadd2_rn(bc2(px), make_float2(-A.r0.x, -B.r0.x));
    const float2 qy = __fadd2_rn(bc2(py), make_float2(-A.r0.y, -B.r0.y));
    const float2 qz = __fadd2_rn(bc2(pz), make_float2(-A.r0.z, -B.r0.z));
    const float2 h = __ffma2_rn(make_float2(A.r3.z, B.r3.z), qz,
                                __ffma2_rn(make_float2(A.r3.y, B.r3.y), qy,
                                           __fmul2_rn(make_float2(A.r3.x, B.r3.x), qx)));
    const float2 h2 = __fmul2_rn(h, h);
    if (!__any_sync(0xffffffffu, fminf(h2.x, h2.y) < cut)) return bc2(FLT_MAX);
    const float2 x = __ffma2_rn(make_float2(A.r1.z, B.r1.z), qz,
                                __ffma2_rn(make_float2(A.r1.y, B.r1.y), qy,
                                           __fmul2_rn(make_float2(A.r1.x, B.r1.x), qx)));
    const float2 y = __ffma2_rn(make_float2(A.r2.z, B.r2.z), qz,
                                __ffma2_rn(make_float2(A.r2.y, B.r2.y), qy,
                                           __fmul2_rn(make_float2(A.r2.x, B.r2.x), qx)));
    const float2 bx = make_float2(A.r0.w, B.r0.w), cx = make_float2(A.r1.w, B.r1.w);
    const float2 cy = make_float2(A.r2.w, B.r2.w), ebx = make_float2(A.r4.w, B.r4.w);
    const float2 nbx = make_float2(-A.r0.w, -B.r0.w), ncx = make_float2(-A.r1.w, -B.r1.w);
    const float2 ncy = make_float2(-A.r2.w, -B.r2.w), nebx = make_float2(-A.r4.w, -B.r4.w);
    const float2 y2 = __fmul2_rn(y, y);
    // A-B along the x axis
    float2 t = clamp01_2(__fmul2_rn(x, make_float2(A.r4.x, B.r4.x)));
    float2 dx = __ffma2_rn(t, nbx, x);
    float2 d = __ffma2_rn(dx, dx, y2);
    // A-C
    t = clamp01_2(__fmul2_rn(__ffma2_rn(x, cx, __fmul2_rn(y, cy)), make_float2(A.r4.y, B.r4.y)));
    dx = __ffma2_rn(t, ncx, x);
    float2 dy = __ffma2_rn(t, ncy, y);
    d = fmin2(d, __ffma2_rn(dx, dx, __fmul2_rn(dy, dy)));
    // B-C
    const float2 xb = __fadd2_rn(x, nbx);
    t = clamp01_2(__fmul2_rn(__ffma2_rn(xb, ebx, __fmul2_rn(y, cy)), make_float2(A.r4.z, B.r4.z)));
    dx = __ffma2_rn(t, nebx, xb);
    dy = __ffma2_rn(t, ncy, y);
    d = fmin2(d, __ffma2_rn(dx, dx, __fmul2_rn(dy, dy)));
    const float2 sb = __ffma2_rn(ebx, y, __fmul2_rn(ncy, xb));
    const float2 sc = __ffma2_rn(cy, x, __fmul2_rn(ncx, y));
    const float2 hd = __fadd2_rn(h2, d);
    const bool ina = (y.x >= 0.f) && (sb.x >= 0.f) && (sc.x >= 0.f);
    const bool inb = (y.y >= 0.f) && (sb.y >= 0.f) && (sc.y >= 0.f);
    return make_float2(ina ? h2.x : hd.x, inb ? h2.y : hd.y);
}

// Component SIDE (0: left, 1: right) of the low (x, y) or high (z, w) pair
// of a record word.
template <int SIDE>
__device__ __forceinline__ float sel(float4 v, bool hi) {
    return hi ? (SIDE ? v.w : v.z) : (SIDE ? v.y : v.x);
}

// The box distance of one child (SIDE) of a record for two points (a bound
// only: its rounding may differ from the one-point form by a few ulps, far
// inside the traversal's slack).
template <int SIDE>
__device__ __forceinline__ float2 obb_d2_2(float2 px, float2 py, float2 pz, float4 w0, float4 w1, float4 w2,
                                           float4 w3, float4 w4, float4 w5, float4 w6, float4 w7) {
    const float2 qx = __fadd2_rn(px, bc2(sel<SIDE>(w0, false))), qy = __fadd2_rn(py, bc2(sel<SIDE>(w0, true))),
                 qz = __fadd2_rn(pz, bc2(sel<SIDE>(w1, false)));
    const float2 t1 = dot3e2(qx, qy, qz, sel<SIDE>(w2, false), sel<SIDE>(w2, true), sel<SIDE>(w3, false));
    const float2 t2 = dot3e2(qx, qy, qz, sel<SIDE>(w4, false), sel<SIDE>(w4, true), sel<SIDE>(w5, false));
    const float2 t3 = dot3e2(qx, qy, qz, sel<SIDE>(w6, false), sel<SIDE>(w6, true), sel<SIDE>(w7, false));
    const float2 u1 = __fadd2_rn(t1, bc2(sel<SIDE>(w1, true))), u2 = __fadd2_rn(t2, bc2(sel<SIDE>(w3, true))),
                 u3 = __fadd2_rn(t3, bc2(sel<SIDE>(w5, true)));
    const float2 s1 = make_float2(fmaxf(fmaxf(-t1.x, u1.x), 0.f), fmaxf(fmaxf(-t1.y, u1.y), 0.f));
    const float2 s2 = make_float2(fmaxf(fmaxf(-t2.x, u2.x), 0.f), fmaxf(fmaxf(-t2.y, u2.y), 0.f));
    const float2 s3 = make_float2(fmaxf(fmaxf(-t3.x, u3.x), 0.f), fmaxf(fmaxf(-t3.y, u3.y), 0.f));
    return dot3e2(s1, s2, s3);
}

// The value the voxel (x, y, z) of this lane stores (PAIR_TRIS: a bucket's
// triangles are tested two at a time on the packed FP32 pipe, which helps
// dense targets and costs registers elsewhere): its exact distance to
// the nearest triangle, or `band` when that is not below the band.  All 32
// lanes of the warp call it together and walk the tree jointly (node and
// triangle loads are warp-uniform broadcasts); lanes with valid == false
// only follow.  stack: this warp's TRAV_STACK ints of shared memory.
// COUNT: also add this warp's node visits and triangle tests, each times the
// warp's valid voxels, to counts[0] and counts[1] (the measurement build,
// mo_df_build_count; compiled out otherwise).
template <bool PAIR_TRIS = false, bool COUNT = false>
__device__ __forceinline__ float df_voxel_value(const float4* __restrict__ nodes, const float4* __restrict__ tris,
                                                int ntri, int N, float band, float band2, int x, int y, int z,
                                                bool valid, int* stack, int* __restrict__ status,
                                                unsigned long long* __restrict__ counts = nullptr) {
    const int lane = threadIdx.x & 31;
    const float Nf = (float)N;
    const float px = __fdiv_rn((float)x, Nf), py = __fdiv_rn((float)y, Nf), pz = __fdiv_rn((float)z, Nf);
    const VoxelBand vb = voxel_band(x, y, z, N, band, band2);
    const float init = vb.bound2;
    float best = valid ? init : -1.0f;
    // Boxes are visited while their fp32 distance is within kSlack (in
    // distance units) of the lane's best: the rounding of the box bound can
    // exceed a triangle's computed distance by far less than that, so no
    // triangle that could lower `best` is skipped and the result is the exact
    // minimum of the computed distances, whatever the visit order.  Starting
    // from band^2 instead of FLT_MAX skips what lies beyond the band and keeps
    // every distance below it.
    float lim = valid ? (init == FLT_MAX ? FLT_MAX : slack_bound(init)) : -1.0f;
    const unsigned FULL = 0xffffffffu;
    const float2 P2x = make_float2(px, px), P2y = make_float2(py, py), P2z = make_float2(pz, pz);
    unsigned long long n_visit = 0, n_test = 0;  // warp-uniform (COUNT only)
    if (ntri == 1) {
        const float t = tri_d2(px, py, pz, load_tri(tris, 0), best);
        if (valid && t < best) best = t;
        if (COUNT) n_test = 1;
    } else {
        int sp = 0;
        int node = 0;
        // each node is entered at most once per traversal; the cap only
        // guards against a corrupted tree
        const int64_t max_iter = 2 * (int64_t)ntri + 64;
        for (int64_t iter = 0;; ++iter) {
            if (iter > max_iter) {
                if (lane == 0) atomicOr(status, 4);
                break;
            }
            if (COUNT) ++n_visit;
            const float4* nd = nodes + NODE_F4 * (int64_t)node;
            const float4 w0 = __ldg(nd), w1 = __ldg(nd + 1), w2 = __ldg(nd + 2), w3 = __ldg(nd + 3);
            const float4 w4 = __ldg(nd + 4), w5 = __ldg(nd + 5), w6 = __ldg(nd + 6), w7 = __ldg(nd + 7);
            const int Lp = __float_as_int(w7.z), Rp = __float_as_int(w7.w);
            const int L = child_index(Lp), R = child_index(Rp);
            const int cl = child_count(Lp), cr = child_count(Rp);  // bucket sizes (0: internal)
            const float2 dlr = obb_pair_d2(P2x, P2y, P2z, w0, w1, w2, w3, w4, w5, w6, w7);
            const float dl = dlr.x, dr = dlr.y;
            bool wl = __any_sync(FULL, dl < lim);
            bool wr = __any_sync(FULL, dr < lim);
            // the opened buckets' triangles, left then right, one test body
            const int nl = wl ? cl : 0, nr = wr ? cr : 0;
            if (COUNT) n_test += (unsigned long long)(nl + nr);
            // two triangles per test where both are non-degenerate
#pragma unroll 1
            for (int k = 0; PAIR_TRIS && k < nl + nr; k += 2) {
                const int ta = k < nl ? L + k : R + (k - nl);
                const Tri A = load_tri(tris, ta);
                if (k + 1 < nl + nr) {
                    const int tb = k + 1 < nl ? L + k + 1 : R + (k + 1 - nl);
                    const Tri B = load_tri(tris, tb);
                    if (A.r3.w != 0.f && B.r3.w != 0.f) {  // warp-uniform
                        const float2 t = tri_d2_t2(px, py, pz, A, B, best);
                        if (valid && t.x < best) { best = t.x; lim = slack_bound(best); }
                        if (valid && t.y < best) { best = t.y; lim = slack_bound(best); }
                        continue;
                    }
                    const float t = tri_d2(px, py, pz, A, best);
                    if (valid && t < best) { best = t; lim = slack_bound(best); }
                    const float u = tri_d2(px, py, pz, B, best);
                    if (valid && u < best) { best = u; lim = slack_bound(best); }
                    continue;
                }
                const float t = tri_d2(px, py, pz, A, best);
                if (valid && t < best) { best = t; lim = slack_bound(best); }
            }
#pragma unroll 1
            for (int k = 0; !PAIR_TRIS && k < nl + nr; ++k) {
                const int tri = k < nl ? L + k : R + (k - nl);
                const float t = tri_d2(px, py, pz, load_tri(tris, tri), best);
                if (valid && t < best) { best = t; lim = slack_bound(best); }
            }
            if (cl > 0) wl = false;
            if (cr > 0) wr = false;
            if (wl && wr) {
                const unsigned nearer_l = __ballot_sync(FULL, valid && dl <= dr);
                const unsigned act = __ballot_sync(FULL, valid);
                const bool lfirst = 2 * __popc(nearer_l) >= __popc(act);
                if (sp >= TRAV_STACK) {  // cannot happen for trees of depth <= 64
                    if (lane == 0) atomicOr(status, 2);
                    break;
                }
                if (lane == 0) stack[sp] = lfirst ? R : L;
                ++sp;
                node = lfirst ? L : R;
            } else if (wl) {
                node = L;
            } else if (wr) {
                node = R;
            } else {
                if (sp == 0) break;
                __syncwarp();
                node = stack[--sp];
            }
            __syncwarp();
        }
    }
    if (COUNT) {
        const unsigned long long nvalid = (unsigned long long)__popc(__ballot_sync(FULL, valid));
        if (lane == 0) {
            atomicAdd(&counts[0], n_visit * nvalid);
            atomicAdd(&counts[1], n_test * nvalid);
        }
    }
    return best < init ? __fsqrt_rn(best) : vb.value;
}

// The values of voxels (x, y, za) and (x, y, zb) of this lane, by one joint
// walk of the warp (see df_voxel_value).
template <bool COUNT = false>
__device__ __forceinline__ float2 df_voxel_value2(const float4* __restrict__ nodes,
                                                  const float4* __restrict__ tris, int ntri, int N, float band,
                                                  float band2, int x, int y, int za, int zb, bool va, bool vb,
                                                  int* stack, int* __restrict__ status,
                                                  unsigned long long* __restrict__ counts = nullptr) {
    const int lane = threadIdx.x & 31;
    const float Nf = (float)N;
    const float fx = __fdiv_rn((float)x, Nf), fy = __fdiv_rn((float)y, Nf);
    const float2 px = bc2(fx), py = bc2(fy);
    const float2 pz = make_float2(__fdiv_rn((float)za, Nf), __fdiv_rn((float)zb, Nf));
    const VoxelBand ba = voxel_band(x, y, za, N, band, band2), bb = voxel_band(x, y, zb, N, band, band2);
    const float2 init = make_float2(ba.bound2, bb.bound2);
    float2 best = make_float2(va ? init.x : -1.0f, vb ? init.y : -1.0f);
    float2 lim = make_float2(va ? (init.x == FLT_MAX ? FLT_MAX : slack_bound(init.x)) : -1.0f,
                             vb ? (init.y == FLT_MAX ? FLT_MAX : slack_bound(init.y)) : -1.0f);
    const unsigned FULL = 0xffffffffu;
    unsigned long long n_visit = 0, n_test = 0;  // warp-uniform (COUNT only)
    if (ntri == 1) {
        const float2 t = tri_d2_2(px, py, pz, load_tri(tris, 0), best);
        if (va && t.x < best.x) best.x = t.x;
        if (vb && t.y < best.y) best.y = t.y;
        if (COUNT) n_test = 1;
    } else {
        int sp = 0;
        int node = 0;
        const int64_t max_iter = 2 * (int64_t)ntri + 64;
        for (int64_t iter = 0;; ++iter) {
            if (iter > max_iter) {
                if (lane == 0) atomicOr(status, 4);
                break;
            }
            if (COUNT) ++n_visit;
            const float4* nd = nodes + NODE_F4 * (int64_t)node;
            const float4 w0 = __ldg(nd), w1 = __ldg(nd + 1), w2 = __ldg(nd + 2), w3 = __ldg(nd + 3);
            const float4 w4 = __ldg(nd + 4), w5 = __ldg(nd + 5), w6 = __ldg(nd + 6), w7 = __ldg(nd + 7);
            const int Lp = __float_as_int(w7.z), Rp = __float_as_int(w7.w);
            const int L = child_index(Lp), R = child_index(Rp);
            const int cl = child_count(Lp), cr = child_count(Rp);
            const float2 dl = obb_d2_2<0>(px, py, pz, w0, w1, w2, w3, w4, w5, w6, w7);
            const float2 dr = obb_d2_2<1>(px, py, pz, w0, w1, w2, w3, w4, w5, w6, w7);
            bool wl = __any_sync(FULL, dl.x < lim.x || dl.y < lim.y);
            bool wr = __any_sync(FULL, dr.x < lim.x || dr.y < lim.y);
            const int nl = wl ? cl : 0, nr = wr ? cr : 0;
            if (COUNT) n_test += (unsigned long long)(nl + nr);
#pragma unroll 1
            for (int k = 0; k < nl + nr; ++k) {
                const int tri = k < nl ? L + k : R + (k - nl);
                const float2 t = tri_d2_2(px, py, pz, load_tri(tris, tri), best);
                if (va && t.x < best.x) { best.x = t.x; lim.x = slack_bound(best.x); }
                if (vb && t.y < best.y) { best.y = t.y; lim.y = slack_bound(best.y); }
            }
            if (cl > 0) wl = false;
            if (cr > 0) wr = false;
            if (wl && wr) {
                // nearer child first by majority over the warp's voxels
                const unsigned na = __ballot_sync(FULL, va && dl.x <= dr.x);
                const unsigned nb = __ballot_sync(FULL, vb && dl.y <= dr.y);
                const unsigned aa = __ballot_sync(FULL, va), ab = __ballot_sync(FULL, vb);
                const bool lfirst = 2 * (__popc(na) + __popc(nb)) >= __popc(aa) + __popc(ab);
                if (sp >= TRAV_STACK) {
                    if (lane == 0) atomicOr(status, 2);
                    break;
                }
                if (lane == 0) stack[sp] = lfirst ? R : L;
                ++sp;
                node = lfirst ? L : R;
            } else if (wl) {
                node = L;
            } else if (wr) {
                node = R;
            } else {
                if (sp == 0) break;
                __syncwarp();
                node = stack[--sp];
            }
            __syncwarp();
        }
    }
    if (COUNT) {
        const unsigned long long nvalid =
            (unsigned long long)(__popc(__ballot_sync(FULL, va)) + __popc(__ballot_sync(FULL, vb)));
        if (lane == 0) {
            atomicAdd(&counts[0], n_visit * nvalid);
            atomicAdd(&counts[1], n_test * nvalid);
        }
    }
    return make_float2(best.x < init.x ? __fsqrt_rn(best.x) : ba.value, best.y < init.y ? __fsqrt_rn(best.y) : bb.value);
}

}  // namespace mo
