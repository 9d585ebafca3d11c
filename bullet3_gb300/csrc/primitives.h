// Device-wide parallel primitives with device-resident element counts, so that every
// launch has a fixed shape and the whole step can be captured in one CUDA graph.
//
// Semantics follow the reference's ParallelPrimitives tests
// (test/OpenCL/ParallelPrimitives/main.cpp:251-339): the radix sort is a STABLE LSD sort
// of (key, value) pairs, the scan is EXCLUSIVE and also reports the total.
#ifndef B3G_PRIMITIVES_H
#define B3G_PRIMITIVES_H

#include <cuda_runtime.h>
#include <stdint.h>

namespace b3g {

// Fixed launch width of the primitives (blocks); set once per device.
struct PrimConfig {
    int sort_blocks = 0;   // G: each block owns one contiguous chunk of the input
    int scan_blocks = 0;
};

// Scratch sizes (bytes) for the helpers below.
size_t radix_scratch_bytes(const PrimConfig& pc);
size_t scan_scratch_bytes(const PrimConfig& pc);

// Stable LSD radix sort of n = *d_n (<= capacity) u32 keys (+ u32 values if vals != nullptr)
// over key bits [0, bits).  Keys/values are ping-ponged between (keys, keys_alt);
// returns 0 when the sorted data ended in (keys, vals), 1 when in (keys_alt, vals_alt).
int radix_sort_u32(const PrimConfig& pc, uint32_t* keys, uint32_t* keys_alt, uint32_t* vals, uint32_t* vals_alt,
                   const int* d_n, int bits, void* scratch, cudaStream_t s, long long* launches);
// Same for u64 keys without values.
int radix_sort_u64(const PrimConfig& pc, uint64_t* keys, uint64_t* keys_alt, uint32_t* vals, uint32_t* vals_alt,
                   const int* d_n, int bits, void* scratch, cudaStream_t s, long long* launches);

// Exclusive scan of n = *d_n ints in `in` into `out`; *d_total = sum.  in may equal out.
void exclusive_scan_i32(const PrimConfig& pc, const int* in, int* out, const int* d_n, int* d_total, void* scratch,
                        cudaStream_t s, long long* launches);

}  // namespace b3g

#endif
