// Shared helpers for the MeshODE GB300 kernels: error reporting, IEEE
// arithmetic without contraction, x86-compatible float->int truncation.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <climits>
#include <cstdio>
#include <string>

#include "../../include/meshode.h"

namespace mo {

// Thread-local last-error message returned by mo_last_error().
void set_error(const char* fmt, ...);
int cuda_status(cudaError_t e, const char* where);

#define MO_CHECK_ARG(cond, ...)                 \
    do {                                        \
        if (!(cond)) {                          \
            ::mo::set_error(__VA_ARGS__);       \
            return MO_ERR_INVALID;              \
        }                                       \
    } while (0)

#define MO_CUDA(call)                                                    \
    do {                                                                 \
        cudaError_t _e = (call);                                         \
        if (_e != cudaSuccess) return ::mo::cuda_status(_e, #call);      \
    } while (0)

#define MO_LAUNCH_CHECK(name)                                            \
    do {                                                                 \
        cudaError_t _e = cudaGetLastError();                             \
        if (_e != cudaSuccess) return ::mo::cuda_status(_e, name);       \
    } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline bool aligned(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

// ---------------------------------------------------------------------------
// Arithmetic that must round exactly like the reference's separate IEEE
// operations (no FMA contraction).
// ---------------------------------------------------------------------------
__device__ __forceinline__ float MUL(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float ADD(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float SUB(float a, float b) { return __fsub_rn(a, b); }

// `int px = float_value` on x86-64: truncation toward zero, and the
// "integer indefinite" INT_MIN for NaN and values outside the int range.
__device__ __forceinline__ int trunc_i32_x86(float f) {
    return (f >= -2147483648.0f && f < 2147483648.0f) ? __float2int_rz(f) : INT_MIN;
}

// Ordered-int encoding of a float so that signed int order == float order
// (used for exact min/max with integer atomics).
__device__ __forceinline__ int float_to_ordered(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__host__ __device__ __forceinline__ float ordered_to_float(int i) {
#ifdef __CUDA_ARCH__
    return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff);
#else
    int j = i >= 0 ? i : i ^ 0x7fffffff;
    float f;
    memcpy(&f, &j, 4);
    return f;
#endif
}

inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

int device_sm_count();

// Counts kernel launches issued through this library (mo_launch_count()).
void note_launch(int n = 1);

// Exclusive scan of n ints in place (single CTA; used for one-shot set-up
// arrays).  If total != nullptr, the sum is stored there (device pointer).
cudaError_t exclusive_scan_i32(int* data, int n, int* total, cudaStream_t s);

// Stable LSD radix sort of (uint32 key, int32 value) pairs over the low
// `bits` bits.  Buffers *_a hold the input; the sorted result is returned in
// *_a as well (ping-pong through *_b).  hist must hold 256*ceil(n/2048) ints.
cudaError_t radix_sort_pairs(uint32_t* keys_a, int* vals_a, uint32_t* keys_b, int* vals_b,
                             int n, int bits, int* hist, cudaStream_t s);
size_t radix_hist_ints(int n);

}  // namespace mo
