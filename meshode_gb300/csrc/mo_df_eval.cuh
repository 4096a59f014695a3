// Trilinear distance lookup with its forward-mode derivative, bit-identical to
// UniformGrid::DistanceFloat<ceres::Jet<float,3>> (src/lib/uniformgrid.cc:85-150)
// as evaluated by the reference for DistanceFieldLoss (distance_layer.cc:58-78).
//
// The jet arithmetic is specialised by hand: the seed derivatives of p are unit
// vectors, so every jet component is either an exact zero or one rounded
// product, and the surviving operations are kept in the reference's order
// with separate IEEE roundings (a*b = (a.a*b.a, a.a*b.v + a.v*b.a); adding an
// exact zero is the identity).
#pragma once

#include "mo_common.cuh"

namespace mo {

struct DFJet {
    float d;          // distance value
    float gx, gy, gz; // d(distance)/d(p)
};

// Corner fetch for the two layouts.  c[k] with k = (bz<<2)|(by<<1)|bx.
template <int LAYOUT>
__device__ __forceinline__ void df_corners(const float* __restrict__ grid, int N, int px, int py, int pz,
                                           float c[8]) {
    if (LAYOUT == MO_LAYOUT_BRICK4) {
        // 32-bit element offsets: grids up to 2^31 floats (N <= 1280)
        const int nb = (N + 3) >> 2;
        int ox[2], oy[2], oz[2];
#pragma unroll
        for (int d = 0; d < 2; ++d) {
            const int x = px + d, y = py + d, z = pz + d;
            ox[d] = (x >> 2) * 64 + (x & 3);
            oy[d] = (y >> 2) * nb * 64 + (y & 3) * 4;
            oz[d] = (z >> 2) * nb * nb * 64 + (z & 3) * 16;
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) c[k] = __ldg(grid + (oz[k >> 2] + oy[(k >> 1) & 1] + ox[k & 1]));
    } else if (LAYOUT == MO_LAYOUT_CELL) {
        const int64_t cell = ((int64_t)pz * (N - 1) + py) * (int64_t)(N - 1) + px;
        const float4* g4 = reinterpret_cast<const float4*>(grid) + 2 * cell;
        const float4 lo = __ldg(g4), hi = __ldg(g4 + 1);
        c[0] = lo.x; c[1] = lo.y; c[2] = lo.z; c[3] = lo.w;
        c[4] = hi.x; c[5] = hi.y; c[6] = hi.z; c[7] = hi.w;
    } else {
        const int64_t b = ((int64_t)pz * N + py) * (int64_t)N + px;
        const int64_t sy = N, sz = (int64_t)N * N;
        c[0] = __ldg(grid + b);
        c[1] = __ldg(grid + b + 1);
        c[2] = __ldg(grid + b + sy);
        c[3] = __ldg(grid + b + sy + 1);
        c[4] = __ldg(grid + b + sz);
        c[5] = __ldg(grid + b + sz + 1);
        c[6] = __ldg(grid + b + sz + sy);
        c[7] = __ldg(grid + b + sz + sy + 1);
    }
}

// Cf = (float)((double)(N - 1) - 1e-3), the far-side penalty offset.
template <int LAYOUT, bool GRAD>
__device__ __forceinline__ DFJet df_eval(const float* __restrict__ grid, int N, float Nf, float Cf,
                                         float x, float y, float z) {
    DFJet r;
    const float sx = MUL(x, Nf), sy = MUL(y, Nf), sz = MUL(z, Nf);
    const int px = trunc_i32_x86(sx), py = trunc_i32_x86(sy), pz = trunc_i32_x86(sz);
    if (px < 0 || py < 0 || pz < 0 || px >= N - 1 || py >= N - 1 || pz >= N - 1) {
        // Out-of-box linear penalty (uniformgrid.cc:90-115): no cutoff here,
        // and no term for an axis with p == N-1.
        float l = 0.0f, gx = 0.0f, gy = 0.0f, gz = 0.0f;
        if (px < 0) { l = ADD(l, -sx); gx = -Nf; }
        else if (px >= N) { l = ADD(l, SUB(sx, Cf)); gx = Nf; }
        if (py < 0) { l = ADD(l, -sy); gy = -Nf; }
        else if (py >= N) { l = ADD(l, SUB(sy, Cf)); gy = Nf; }
        if (pz < 0) { l = ADD(l, -sz); gz = -Nf; }
        else if (pz >= N) { l = ADD(l, SUB(sz, Cf)); gz = Nf; }
        r.d = l; r.gx = gx; r.gy = gy; r.gz = gz;
        return r;
    }
    const float wx = SUB(sx, (float)px), wy = SUB(sy, (float)py), wz = SUB(sz, (float)pz);
    const float ox = SUB(1.0f, wx), oy = SUB(1.0f, wy), oz = SUB(1.0f, wz);
    float c[8];
    df_corners<LAYOUT>(grid, N, px, py, pz, c);
    float ra = 0.0f, rx = 0.0f, ry = 0.0f, rz = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const bool bx = k & 1, by = (k >> 1) & 1, bz = (k >> 2) & 1;
        const float fx = bx ? wx : ox, fy = by ? wy : oy, fz = bz ? wz : oz;
        const float P = MUL(fx, fy);
        const float Q = MUL(P, fz);
        const float W = MUL(Q, c[k]);
        ra = (k == 0) ? W : ADD(ra, W);
        if (GRAD) {
            const float sfx = bx ? Nf : -Nf, sfy = by ? Nf : -Nf, sfz = bz ? Nf : -Nf;
            const float Px = MUL(sfx, fy), Py = MUL(fx, sfy);
            const float Qx = MUL(Px, fz), Qy = MUL(Py, fz), Qz = MUL(P, sfz);
            const float Wx = MUL(Qx, c[k]), Wy = MUL(Qy, c[k]), Wz = MUL(Qz, c[k]);
            rx = (k == 0) ? Wx : ADD(rx, Wx);
            ry = (k == 0) ? Wy : ADD(ry, Wy);
            rz = (k == 0) ? Wz : ADD(rz, Wz);
        }
    }
    if (ra > 0.2f) {  // uniformgrid.cc:147-148
        r.d = 0.0f; r.gx = 0.0f; r.gy = 0.0f; r.gz = 0.0f;
    } else {
        r.d = ra; r.gx = rx; r.gy = ry; r.gz = rz;
    }
    return r;
}

// 0.5 * d(d^2)/dp through the jet square, as distance_layer.cc:73-77:
// vd*vd has derivative d*g + g*d, then * 0.5.
__device__ __forceinline__ float df_grad_component(float d, float g) {
    return MUL(ADD(MUL(d, g), MUL(g, d)), 0.5f);
}

}  // namespace mo
