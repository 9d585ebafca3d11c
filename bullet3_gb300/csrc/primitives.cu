// Stable LSD radix sort and exclusive scan with device-resident counts.
//
// Reference semantics: b3RadixSort32CL (stable 32-bit key/value LSD sort,
// src/Bullet3OpenCL/ParallelPrimitives/b3RadixSort32CL.h, host twin executeHost :89-155)
// and b3PrefixScanCL (exclusive scan + total, b3PrefixScanCL.h:31-32).
//
// Design (GB300): a fixed grid of G blocks; block b owns one contiguous chunk of the input,
// so stability holds by construction.  Per 8-bit digit pass: (1) per-block 256-bin
// histogram, (2) one-block exclusive scan of the digit-major histogram table, (3) stable
// scatter: the chunk is consumed in rounds of 256 keys; ranks inside a warp come from
// __match_any_sync, ranks across the 8 warps from a shared-memory prefix.
#include "primitives.h"

#include <cuda_runtime.h>
#include <stdint.h>

namespace b3g {

static constexpr int RS_THREADS = 256;
static constexpr int RS_WARPS = RS_THREADS / 32;
static constexpr int RADIX = 256;
static_assert(RS_THREADS == RADIX, "rs_scatter scans one digit total per thread");

size_t radix_scratch_bytes(const PrimConfig& pc) {
    return (size_t)RADIX * pc.sort_blocks * sizeof(int) + RADIX * sizeof(int) + 256;
}
size_t scan_scratch_bytes(const PrimConfig& pc) { return (size_t)(2 * pc.scan_blocks + 2) * sizeof(int) + 256; }

template <typename K>
__device__ __forceinline__ unsigned digit_of(K k, int shift, unsigned mask) {
    return (unsigned)((k >> shift) & (K)mask);
}

__device__ __forceinline__ void chunk_range(int n, int G, int b, int& lo, int& hi) {
    // chunk length rounded up to a multiple of RS_THREADS
    int per = (n + G - 1) / G;
    per = (per + RS_THREADS - 1) / RS_THREADS * RS_THREADS;
    lo = b * per;
    hi = lo + per;
    if (lo > n) lo = n;
    if (hi > n) hi = n;
}

template <typename K>
__global__ void __launch_bounds__(RS_THREADS) rs_histogram(const K* __restrict__ keys, const int* __restrict__ d_n,
                                                           int shift, unsigned mask, int* __restrict__ hist) {
    __shared__ int h[RADIX];
    const int G = gridDim.x;
    int n = *d_n;
    int lo, hi;
    chunk_range(n, G, blockIdx.x, lo, hi);
    for (int i = threadIdx.x; i < RADIX; i += RS_THREADS) h[i] = 0;
    __syncthreads();
    for (int i = lo + threadIdx.x; i < hi; i += RS_THREADS) atomicAdd(&h[digit_of(keys[i], shift, mask)], 1);
    __syncthreads();
    for (int d = threadIdx.x; d < RADIX; d += RS_THREADS) hist[d * G + blockIdx.x] = h[d];
}

// One block: in-place exclusive scan of `len` ints (len <= 1024 * per-thread segment).
__global__ void __launch_bounds__(1024) scan_small(int* __restrict__ a, int len, int* __restrict__ total) {
    __shared__ int sums[1024];
    const int T = blockDim.x;
    int seg = (len + T - 1) / T;
    int lo = threadIdx.x * seg, hi = lo + seg;
    if (hi > len) hi = len;
    int s = 0;
    for (int i = lo; i < hi; i++) s += a[i];
    sums[threadIdx.x] = s;
    __syncthreads();
    // Hillis-Steele inclusive scan over T partial sums
    for (int off = 1; off < T; off <<= 1) {
        int v = threadIdx.x >= off ? sums[threadIdx.x - off] : 0;
        __syncthreads();
        sums[threadIdx.x] += v;
        __syncthreads();
    }
    int run = threadIdx.x ? sums[threadIdx.x - 1] : 0;
    for (int i = lo; i < hi; i++) {
        int v = a[i];
        a[i] = run;
        run += v;
    }
    if (total && threadIdx.x == T - 1) *total = sums[T - 1];
}

// One block per digit: exclusive scan of that digit's per-block counts (in place) and the
// digit total.  Replaces a one-block scan of the whole digit-major table.
__global__ void __launch_bounds__(RS_THREADS) rs_digit_scan(int* __restrict__ hist, int G,
                                                            int* __restrict__ digit_total) {
    __shared__ int wsum[RS_WARPS];
    __shared__ int carry;
    const int d = blockIdx.x;
    int* row = hist + (size_t)d * G;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < G; base += RS_THREADS) {
        int i = base + threadIdx.x;
        int v = i < G ? row[i] : 0;
        int x = v;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[warp] = x;
        __syncthreads();
        int wpre = 0, tot = 0;
        for (int w = 0; w < RS_WARPS; w++) {
            int c = wsum[w];
            if (w < warp) wpre += c;
            tot += c;
        }
        if (i < G) row[i] = carry + wpre + x - v;
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) digit_total[d] = carry;
}

template <typename K, bool HAS_VALS>
__global__ void __launch_bounds__(RS_THREADS) rs_scatter(const K* __restrict__ keys_in, K* __restrict__ keys_out,
                                                         const uint32_t* __restrict__ vals_in,
                                                         uint32_t* __restrict__ vals_out, const int* __restrict__ d_n,
                                                         int shift, unsigned mask, const int* __restrict__ hist,
                                                         const int* __restrict__ digit_total) {
    __shared__ int warp_cnt[RS_WARPS][RADIX];
    __shared__ int running[RADIX];
    __shared__ int round_total[RADIX];
    const int G = gridDim.x;
    const int n = *d_n;
    int lo, hi;
    chunk_range(n, G, blockIdx.x, lo, hi);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // digit bases: exclusive scan of the 256 digit totals (RS_THREADS == RADIX: one digit per thread)
    {
        int v = digit_total[threadIdx.x];
        int x = v;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) round_total[warp] = x;
        __syncthreads();
        int wpre = 0;
        for (int w = 0; w < warp; w++) wpre += round_total[w];
        running[threadIdx.x] = wpre + x - v + hist[threadIdx.x * G + blockIdx.x];
        __syncthreads();
    }
    const unsigned lanemask_lt = (1u << lane) - 1u;
    for (int base = lo; base < hi; base += RS_THREADS) {
        for (int i = threadIdx.x; i < RS_WARPS * RADIX; i += RS_THREADS) (&warp_cnt[0][0])[i] = 0;
        __syncthreads();
        int idx = base + threadIdx.x;
        bool valid = idx < hi;
        K k = valid ? keys_in[idx] : (K)0;
        unsigned d = valid ? digit_of(k, shift, mask) : (RADIX + lane);
        unsigned peers = __match_any_sync(0xffffffffu, d);
        int rank = __popc(peers & lanemask_lt);
        if (valid && rank == 0) warp_cnt[warp][d] = __popc(peers);
        __syncthreads();
        for (int t = threadIdx.x; t < RADIX; t += RS_THREADS) {
            int s = 0;
            for (int w = 0; w < RS_WARPS; w++) {
                int c = warp_cnt[w][t];
                warp_cnt[w][t] = s;
                s += c;
            }
            round_total[t] = s;
        }
        __syncthreads();
        if (valid) {
            int pos = running[d] + warp_cnt[warp][d] + rank;
            keys_out[pos] = k;
            if (HAS_VALS) vals_out[pos] = vals_in[idx];
        }
        __syncthreads();
        for (int t = threadIdx.x; t < RADIX; t += RS_THREADS) running[t] += round_total[t];
        __syncthreads();
    }
}

template <typename K>
static int radix_sort_impl(const PrimConfig& pc, K* keys, K* keys_alt, uint32_t* vals, uint32_t* vals_alt,
                           const int* d_n, int bits, void* scratch, cudaStream_t s, long long* launches) {
    int* hist = reinterpret_cast<int*>(scratch);
    const int G = pc.sort_blocks;
    int* digit_total = hist + (size_t)RADIX * G;
    K* kin = keys;
    K* kout = keys_alt;
    uint32_t* vin = vals;
    uint32_t* vout = vals_alt;
    int which = 0;
    for (int shift = 0; shift < bits; shift += 8) {
        int nb = bits - shift < 8 ? bits - shift : 8;
        unsigned mask = (1u << nb) - 1u;
        rs_histogram<K><<<G, RS_THREADS, 0, s>>>(kin, d_n, shift, mask, hist);
        rs_digit_scan<<<RADIX, RS_THREADS, 0, s>>>(hist, G, digit_total);
        if (vals)
            rs_scatter<K, true><<<G, RS_THREADS, 0, s>>>(kin, kout, vin, vout, d_n, shift, mask, hist, digit_total);
        else
            rs_scatter<K, false><<<G, RS_THREADS, 0, s>>>(kin, kout, nullptr, nullptr, d_n, shift, mask, hist,
                                                          digit_total);
        if (launches) *launches += 3;
        K* tk = kin; kin = kout; kout = tk;
        uint32_t* tv = vin; vin = vout; vout = tv;
        which ^= 1;
    }
    return which;
}

int radix_sort_u32(const PrimConfig& pc, uint32_t* keys, uint32_t* keys_alt, uint32_t* vals, uint32_t* vals_alt,
                   const int* d_n, int bits, void* scratch, cudaStream_t s, long long* launches) {
    return radix_sort_impl<uint32_t>(pc, keys, keys_alt, vals, vals_alt, d_n, bits, scratch, s, launches);
}
int radix_sort_u64(const PrimConfig& pc, uint64_t* keys, uint64_t* keys_alt, uint32_t* vals, uint32_t* vals_alt,
                   const int* d_n, int bits, void* scratch, cudaStream_t s, long long* launches) {
    return radix_sort_impl<uint64_t>(pc, keys, keys_alt, vals, vals_alt, d_n, bits, scratch, s, launches);
}

// ---------------------------------------------------------------- exclusive scan
static constexpr int SC_THREADS = 512;

__device__ __forceinline__ void scan_chunk(int n, int G, int b, int& lo, int& hi) {
    int per = (n + G - 1) / G;
    lo = b * per;
    hi = lo + per;
    if (lo > n) lo = n;
    if (hi > n) hi = n;
}

__global__ void __launch_bounds__(SC_THREADS) scan_reduce(const int* __restrict__ in, const int* __restrict__ d_n,
                                                          int* __restrict__ block_sums) {
    __shared__ int red[SC_THREADS / 32];
    int n = *d_n, lo, hi;
    scan_chunk(n, gridDim.x, blockIdx.x, lo, hi);
    int s = 0;
    for (int i = lo + threadIdx.x; i < hi; i += SC_THREADS) s += in[i];
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < SC_THREADS / 32; w++) t += red[w];
        block_sums[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(SC_THREADS) scan_downsweep(const int* in, int* out, const int* __restrict__ d_n,
                                                             const int* __restrict__ block_offsets) {
    __shared__ int wsum[SC_THREADS / 32];
    __shared__ int carry;
    int n = *d_n, lo, hi;
    scan_chunk(n, gridDim.x, blockIdx.x, lo, hi);
    if (threadIdx.x == 0) carry = block_offsets[blockIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int base = lo; base < hi; base += SC_THREADS) {
        int i = base + threadIdx.x;
        int v = i < hi ? in[i] : 0;
        int x = v;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[warp] = x;
        __syncthreads();
        int wpre = 0, tot = 0;
        for (int w = 0; w < SC_THREADS / 32; w++) {
            int c = wsum[w];
            if (w < warp) wpre += c;
            tot += c;
        }
        int excl = carry + wpre + x - v;
        __syncthreads();
        if (i < hi) out[i] = excl;
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
}

__global__ void scan_total(const int* __restrict__ block_offsets, const int* __restrict__ block_sums, int G,
                           int* __restrict__ d_total) {
    *d_total = block_offsets[G - 1] + block_sums[G - 1];
}

void exclusive_scan_i32(const PrimConfig& pc, const int* in, int* out, const int* d_n, int* d_total, void* scratch,
                        cudaStream_t s, long long* launches) {
    const int G = pc.scan_blocks;
    int* block_sums = reinterpret_cast<int*>(scratch);
    int* block_offsets = block_sums + G;
    scan_reduce<<<G, SC_THREADS, 0, s>>>(in, d_n, block_sums);
    cudaMemcpyAsync(block_offsets, block_sums, sizeof(int) * G, cudaMemcpyDeviceToDevice, s);
    scan_small<<<1, 1024, 0, s>>>(block_offsets, G, nullptr);
    scan_downsweep<<<G, SC_THREADS, 0, s>>>(in, out, d_n, block_offsets);
    if (d_total) scan_total<<<1, 1, 0, s>>>(block_offsets, block_sums, G, d_total);
    if (launches) *launches += d_total ? 4 : 3;
}

}  // namespace b3g
