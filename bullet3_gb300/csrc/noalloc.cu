// Allocation-free grid broadphase: the pair search of launch_pairs (broadphase.cu) over caller
// AABBs, with every scratch buffer carved out of one file-scope device array.
//
// Reference behaviour followed: b3GpuGridBroadphase::calculateOverlappingPairs
// (src/Bullet3OpenCL/BroadphaseCollision/b3GpuGridBroadphase.cpp:134-229) -- cell of the AABB
// centre, sort by cell, search the 27 neighbouring cells, inclusive AABB overlap
// (gridBroadphase.cl:89-94), one pair per unordered body couple.  Pairs come out sorted by
// (a, b), the same canonical order as b3g_calculate_overlapping_pairs.
#include <cuda_runtime.h>
#include <stdint.h>

#include "b3g_capi.h"
#include "b3g_types.h"
#include "primitives.h"
#include "world_internal.h"

namespace b3g {

// kernels of broadphase.cu reused as they are
__global__ void k_cell_start(const uint32_t* keys, int n, uint32_t* cell_start);
__global__ void k_find_pairs(const b3gAabb* aabbs, const uint32_t* keys, const uint32_t* vals,
                             const uint32_t* cell_start, int n_dyn, const int* large_list, int n_large,
                             float inv_cell, int bits, int body_bits, uint64_t* out, int* counter, int cap,
                             unsigned int* status);
__global__ void k_clamp_count(int* counter, int cap, int* clamped);

namespace {

constexpr int NA_THREADS = 256;  // launch width of the reused broadphase kernels
constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// scratch layout (byte offsets into the static array)
constexpr size_t NA_KEYS = B3G_NOALLOC_MAX_AABBS * sizeof(uint32_t);
constexpr size_t NA_CELLS = (size_t)B3G_NOALLOC_MAX_GRID_DIM * B3G_NOALLOC_MAX_GRID_DIM * B3G_NOALLOC_MAX_GRID_DIM *
                            sizeof(uint32_t);
constexpr size_t NA_PAIRS = (size_t)B3G_NOALLOC_MAX_PAIRS * sizeof(uint64_t);
constexpr size_t NA_OFF_KEYS0 = 0;
constexpr size_t NA_OFF_KEYS1 = NA_OFF_KEYS0 + align256(NA_KEYS);
constexpr size_t NA_OFF_VALS0 = NA_OFF_KEYS1 + align256(NA_KEYS);
constexpr size_t NA_OFF_VALS1 = NA_OFF_VALS0 + align256(NA_KEYS);
constexpr size_t NA_OFF_CELLS = NA_OFF_VALS1 + align256(NA_KEYS);
constexpr size_t NA_OFF_PAIRS0 = NA_OFF_CELLS + align256(NA_CELLS);
constexpr size_t NA_OFF_PAIRS1 = NA_OFF_PAIRS0 + align256(NA_PAIRS);
constexpr size_t NA_OFF_SORT = NA_OFF_PAIRS1 + align256(NA_PAIRS);
constexpr size_t NA_SORT_BYTES = (size_t)256 * B3G_NOALLOC_MAX_SORT_BLOCKS * sizeof(int) + 256 * sizeof(int) + 256;
constexpr size_t NA_OFF_COUNTERS = NA_OFF_SORT + align256(NA_SORT_BYTES);
constexpr size_t NA_BYTES = NA_OFF_COUNTERS + 256;  // counters: n, raw pairs, clamped pairs, status

}  // namespace

// The scratch array.  Contents never need to start at zero (see launch_grid_pairs_noalloc).
static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

size_t noalloc_scratch_bytes() { return NA_BYTES; }

cudaError_t noalloc_scratch_address(void** out) { return cudaGetSymbolAddress(out, g_noalloc_scratch); }

// cell hash of the AABB centre, laid out exactly as k_aabb_hash does for dynamic bodies; thread 0
// also resets the per-call counters (this kernel runs first in every call)
__global__ void __launch_bounds__(NA_THREADS) k_na_hash(const b3gAabb* __restrict__ aabbs, int n, float inv_cell,
                                                         int bits, uint32_t* __restrict__ keys,
                                                         uint32_t* __restrict__ vals, int* __restrict__ counters) {
    const int mask = (1 << bits) - 1;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        counters[0] = n;
        counters[1] = 0;
        counters[2] = 0;
        counters[3] = 0;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const b3gAabb a = aabbs[i];
        const float cx = (a.minv[0] + a.maxv[0]) * 0.5f, cy = (a.minv[1] + a.maxv[1]) * 0.5f,
                    cz = (a.minv[2] + a.maxv[2]) * 0.5f;
        const int gx = ((int)floorf(cx * inv_cell)) & mask, gy = ((int)floorf(cy * inv_cell)) & mask,
                  gz = ((int)floorf(cz * inv_cell)) & mask;
        keys[i] = ((uint32_t)gz << (2 * bits)) | ((uint32_t)gy << bits) | (uint32_t)gx;
        vals[i] = (uint32_t)i;
    }
}

// sorted packed keys -> (a, b, -1, -1); the raw pair count goes to the caller's counter
__global__ void __launch_bounds__(NA_THREADS) k_na_unpack(const uint64_t* __restrict__ keys,
                                                           const int* __restrict__ counters, int body_bits,
                                                           b3gPair* __restrict__ pairs, int* __restrict__ num_out) {
    const int np = counters[2];
    const uint64_t bmask = (1ull << body_bits) - 1ull;
    if (blockIdx.x == 0 && threadIdx.x == 0) *num_out = counters[1];
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const uint64_t k = keys[p];
        b3gPair pr;
        pr.x = (int)(k >> body_bits);
        pr.y = (int)(k & bmask);
        pr.z = -1;
        pr.w = -1;
        pairs[p] = pr;
    }
}

int launch_grid_pairs_noalloc(void* scratch, int num_sms, const b3gAabb* aabbs, int n, float inv_cell, int bits,
                              int body_bits, b3gPair* pairs, int max_pairs, int* num_out, cudaStream_t s) {
    unsigned char* base = static_cast<unsigned char*>(scratch);
    uint32_t* keys0 = reinterpret_cast<uint32_t*>(base + NA_OFF_KEYS0);
    uint32_t* keys1 = reinterpret_cast<uint32_t*>(base + NA_OFF_KEYS1);
    uint32_t* vals0 = reinterpret_cast<uint32_t*>(base + NA_OFF_VALS0);
    uint32_t* vals1 = reinterpret_cast<uint32_t*>(base + NA_OFF_VALS1);
    uint32_t* cells = reinterpret_cast<uint32_t*>(base + NA_OFF_CELLS);
    uint64_t* pk0 = reinterpret_cast<uint64_t*>(base + NA_OFF_PAIRS0);
    uint64_t* pk1 = reinterpret_cast<uint64_t*>(base + NA_OFF_PAIRS1);
    void* sort_scratch = base + NA_OFF_SORT;
    int* counters = reinterpret_cast<int*>(base + NA_OFF_COUNTERS);
    PrimConfig pc;
    pc.sort_blocks = num_sms * 4;
    pc.scan_blocks = num_sms * 2;
    long long ll = 0;
    int launches = 0;
    const int grid = num_sms * 4;
    k_na_hash<<<grid, NA_THREADS, 0, s>>>(aabbs, n, inv_cell, bits, keys0, vals0, counters);
    launches++;
    const int w = radix_sort_u32(pc, keys0, keys1, vals0, vals1, &counters[0], 3 * bits, sort_scratch, s, &ll);
    const uint32_t* keys = w ? keys1 : keys0;
    const uint32_t* vals = w ? vals1 : vals0;
    k_cell_start<<<grid, NA_THREADS, 0, s>>>(keys, n, cells);
    launches++;
    k_find_pairs<<<num_sms * 8, NA_THREADS, 0, s>>>(aabbs, keys, vals, cells, n, nullptr, 0, inv_cell, bits,
                                                    body_bits, pk0, &counters[1], max_pairs,
                                                    reinterpret_cast<unsigned int*>(&counters[3]));
    launches++;
    k_clamp_count<<<1, 1, 0, s>>>(&counters[1], max_pairs, &counters[2]);
    launches++;
    const int w2 = radix_sort_u64(pc, pk0, pk1, nullptr, nullptr, &counters[2], 2 * body_bits, sort_scratch, s, &ll);
    k_na_unpack<<<grid, NA_THREADS, 0, s>>>(w2 ? pk1 : pk0, counters, body_bits, pairs, num_out);
    launches++;
    return launches + (int)ll;
}

}  // namespace b3g
