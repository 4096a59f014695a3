// LBVH pieces shared by the distance-field build (triangles) and the
// nearest-point queries (points): 30-bit Morton codes, the Karras (HPG 2012)
// radix tree over sorted codes, and the bottom-up box refit.  The kernels are
// defined in mo_dfbuild.cu.
//
// Node layout: internal node i (of n-1) is 4 float4 =
//   (left lo.xyz, left id) (left hi.xyz, right id) (right lo.xyz, -) (right hi.xyz, -)
// with ids >= 0 for internal nodes and ~k for leaf k (the k-th sorted item).
#pragma once

#include "mo_common.cuh"

namespace mo {

// The low 10 bits of x spread to every third bit.
__device__ __forceinline__ uint32_t spread10(uint32_t x) {
    x &= 0x3ffu;
    x = (x | (x << 16)) & 0x030000ffu;
    x = (x | (x << 8)) & 0x0300f00fu;
    x = (x | (x << 4)) & 0x030c30c3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

// A unit-cube coordinate quantised to 10 bits (clamped).
__device__ __forceinline__ uint32_t quant10(float c) {
    float q = MUL(c, 1024.0f);
    q = fmaxf(q, 0.0f);
    q = fminf(q, 1023.0f);
    return (uint32_t)q;
}

__device__ __forceinline__ uint32_t morton30(float x, float y, float z) {
    return (spread10(quant10(x)) << 2) | (spread10(quant10(y)) << 1) | spread10(quant10(z));
}

// Children of the n-1 internal nodes from n sorted codes (ties broken by
// index), parent links (parent[slot] = 2*node + side; leaf k has slot n-1+k)
// and zeroed refit flags; range (optional) gets each node's leaves
// [first, last] (a Karras subtree's leaves are contiguous).
__global__ void k_karras(const uint32_t* __restrict__ k, int n, float4* __restrict__ nodes,
                         int* __restrict__ parent, int* __restrict__ flags, int2* __restrict__ range);
// Boxes of every internal node from the n leaf boxes (2 float4 each, lo then
// hi, in sorted order); the root box goes to rootbox[6].  Bit 2 of status on
// a malformed parent array.
__global__ void k_refit(const float4* __restrict__ boxes, int n, float4* nodes, const int* __restrict__ parent,
                        int* flags, float* rootbox, int* status);

}  // namespace mo
