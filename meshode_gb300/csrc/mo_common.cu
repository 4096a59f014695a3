// Error state, device queries and two set-up primitives shared by the
// builders: a single-CTA exclusive scan and a stable LSD radix sort.
#include <atomic>
#include <cstdarg>
#include <cstring>

#include "mo_common.cuh"

namespace mo {

static thread_local char g_err[512] = "";
static std::atomic<unsigned long long> g_launches{0};

void note_launch(int n) { g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed); }

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int cuda_status(cudaError_t e, const char* where) {
    set_error("CUDA error %d (%s) in %s", (int)e, cudaGetErrorString(e), where);
    return MO_ERR_CUDA;
}

int device_sm_count() {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 1;
    return sms > 0 ? sms : 1;
}

// ---------------------------------------------------------------------------
// Single-CTA exclusive scan, in tiles of 1024 x 8 ints: coalesced loads into
// shared memory, each thread scans 8 consecutive ints, a block scan of the
// thread sums, coalesced stores; a running carry joins the tiles.
// ---------------------------------------------------------------------------
constexpr int SCAN_THREADS = 1024, SCAN_PER = 8, SCAN_TILE = SCAN_THREADS * SCAN_PER;

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_1cta(int* a, int n, int* total) {
    __shared__ int tile[SCAN_TILE + SCAN_TILE / 32];  // one pad int per 32 breaks bank conflicts
    __shared__ int warp_sums[32];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    auto at = [](int i) { return i + (i >> 5); };
    int carry = 0;
    for (int base = 0; base < n; base += SCAN_TILE) {
#pragma unroll
        for (int k = 0; k < SCAN_PER; ++k) {
            const int i = k * SCAN_THREADS + tid;
            tile[at(i)] = base + i < n ? a[base + i] : 0;
        }
        __syncthreads();
        int v[SCAN_PER];
        int s = 0;
#pragma unroll
        for (int k = 0; k < SCAN_PER; ++k) {
            v[k] = s;
            s += tile[at(tid * SCAN_PER + k)];
        }
        int x = s;  // inclusive scan of the thread sums
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sums[w] = x;
        __syncthreads();
        if (w == 0) {
            int ws = warp_sums[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, ws, o);
                if (lane >= o) ws += y;
            }
            warp_sums[lane] = ws;
        }
        __syncthreads();
        const int pre = carry + x - s + (w > 0 ? warp_sums[w - 1] : 0);
#pragma unroll
        for (int k = 0; k < SCAN_PER; ++k) tile[at(tid * SCAN_PER + k)] = pre + v[k];
        const int tile_total = warp_sums[31];
        __syncthreads();
#pragma unroll
        for (int k = 0; k < SCAN_PER; ++k) {
            const int i = k * SCAN_THREADS + tid;
            if (base + i < n) a[base + i] = tile[at(i)];
        }
        carry += tile_total;
        __syncthreads();  // tile and warp_sums are rewritten next round
    }
    if (total && tid == 0) *total = carry;
}

cudaError_t exclusive_scan_i32(int* data, int n, int* total, cudaStream_t s) {
    if (n <= 0) {
        if (total) return cudaMemsetAsync(total, 0, sizeof(int), s);
        return cudaSuccess;
    }
    k_scan_1cta<<<1, 1024, 0, s>>>(data, n, total); ::mo::note_launch();
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Stable LSD radix sort, 8-bit digits.  Tile = 8 warps x 8 rounds x 32 keys.
// Pass: per-tile digit histogram -> exclusive scan over [digit][tile] ->
// stable scatter (per-warp ranks from __match_any_sync, warps in order).
// ---------------------------------------------------------------------------
constexpr int RS_WARPS = 8, RS_ROUNDS = 8, RS_TILE = RS_WARPS * RS_ROUNDS * 32;

size_t radix_hist_ints(int n) { return (size_t)256 * (size_t)ceil_div(n > 0 ? n : 1, RS_TILE); }

__global__ void __launch_bounds__(256) k_rs_hist(const uint32_t* __restrict__ keys, int n, int shift,
                                                 int* __restrict__ hist, int ntiles) {
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * RS_TILE;
    for (int j = 0; j < RS_TILE / 256; ++j) {
        int i = base + j * 256 + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1);
    }
    __syncthreads();
    hist[threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(256) k_rs_scatter(const uint32_t* __restrict__ kin,
                                                    const int* __restrict__ vin,
                                                    uint32_t* __restrict__ kout, int* __restrict__ vout,
                                                    int n, int shift, const int* __restrict__ hist,
                                                    int ntiles) {
    __shared__ int wh[RS_WARPS][256];
    __shared__ int wbase[RS_WARPS][256];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int d = threadIdx.x; d < RS_WARPS * 256; d += 256) (&wh[0][0])[d] = 0;
    __syncthreads();
    const int wbeg = blockIdx.x * RS_TILE + w * RS_ROUNDS * 32;
    const unsigned lt = (1u << lane) - 1u;
    uint32_t key[RS_ROUNDS];
    int digit[RS_ROUNDS], rank[RS_ROUNDS];
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; ++r) {
        const int i = wbeg + r * 32 + lane;
        const bool valid = i < n;
        key[r] = valid ? kin[i] : 0u;
        digit[r] = valid ? (int)((key[r] >> shift) & 255u) : 256 + lane;
        const unsigned peers = __match_any_sync(0xffffffffu, digit[r]);
        int pre = 0;
        if (valid) pre = wh[w][digit[r]];
        __syncwarp();
        if (valid && lane == __ffs(peers) - 1) wh[w][digit[r]] = pre + __popc(peers);
        __syncwarp();
        rank[r] = pre + __popc(peers & lt);
    }
    __syncthreads();
    {
        const int d = threadIdx.x;  // 256 threads == 256 digits
        int run = hist[d * ntiles + blockIdx.x];
        for (int ww = 0; ww < RS_WARPS; ++ww) {
            wbase[ww][d] = run;
            run += wh[ww][d];
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; ++r) {
        const int i = wbeg + r * 32 + lane;
        if (i < n) {
            const int pos = wbase[w][digit[r]] + rank[r];
            kout[pos] = key[r];
            vout[pos] = vin[i];
        }
    }
}

cudaError_t radix_sort_pairs(uint32_t* keys_a, int* vals_a, uint32_t* keys_b, int* vals_b, int n,
                             int bits, int* hist, cudaStream_t s) {
    if (n <= 1) return cudaSuccess;
    const int ntiles = ceil_div(n, RS_TILE);
    const int passes = (bits + 7) / 8;
    uint32_t *ki = keys_a, *ko = keys_b;
    int *vi = vals_a, *vo = vals_b;
    for (int p = 0; p < passes; ++p) {
        const int shift = 8 * p;
        k_rs_hist<<<ntiles, 256, 0, s>>>(ki, n, shift, hist, ntiles); ::mo::note_launch();
        cudaError_t e = exclusive_scan_i32(hist, 256 * ntiles, nullptr, s);
        if (e != cudaSuccess) return e;
        k_rs_scatter<<<ntiles, 256, 0, s>>>(ki, vi, ko, vo, n, shift, hist, ntiles); ::mo::note_launch();
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        uint32_t* tk = ki; ki = ko; ko = tk;
        int* tv = vi; vi = vo; vo = tv;
    }
    if (ki != keys_a) {  // odd number of passes: result is in *_b
        cudaError_t e = cudaMemcpyAsync(keys_a, ki, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return e;
        e = cudaMemcpyAsync(vals_a, vi, sizeof(int) * n, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace mo

extern "C" const char* mo_last_error(void) { return mo::g_err; }
extern "C" int mo_version(void) { return 100; }
extern "C" unsigned long long mo_launch_count(void) { return mo::g_launches.load(std::memory_order_relaxed); }
