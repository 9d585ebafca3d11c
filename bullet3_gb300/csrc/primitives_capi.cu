// C ABI of the device-wide parallel primitives, for callers of the reference's
// ParallelPrimitives classes (src/Bullet3OpenCL/ParallelPrimitives/):
//   b3RadixSort32CL::execute  (b3RadixSort32CL.cpp:174)   -> b3g_radix_sort32 / b3g_radix_sort32_keys
//   b3PrefixScanCL::execute   (b3PrefixScanCL.cpp)        -> b3g_prefix_scan32
//   b3BoundSearchCL::execute  (b3BoundSearchCL.cpp:69,133) -> b3g_bound_search
//   b3FillCL::execute         (b3FillCL.cpp)              -> b3g_fill32
// Device buffers belong to the caller.  Each call allocates its own scratch, runs on the device's
// legacy default stream and synchronises before it returns (the reference's calls enqueue on the
// caller's queue; a caller here gets finished results, and the scan's sum, on return).
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>

#include "b3g_capi.h"
#include "primitives.h"
#include "world_internal.h"

namespace b3g {

namespace {

struct Scratch {
    void* p = nullptr;
    ~Scratch() {
        if (p) cudaFree(p);
    }
};

b3gStatus cuda_fail(cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return report_error(B3G_ERR_CUDA, m.c_str());
}

#define PRIM_TRY(expr, what)                          \
    do {                                              \
        cudaError_t _e = (expr);                      \
        if (_e != cudaSuccess) return cuda_fail(_e, what); \
    } while (0)

PrimConfig prim_config(int device) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    PrimConfig pc;
    pc.sort_blocks = (sms > 0 ? sms : 1) * 4;
    pc.scan_blocks = (sms > 0 ? sms : 1) * 2;
    return pc;
}

// (key, value) pairs <-> separate key and value arrays
__global__ void k_split_pairs(const uint2* __restrict__ kv, int n, uint32_t* __restrict__ k, uint32_t* __restrict__ v) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint2 x = kv[i];
        k[i] = x.x;
        v[i] = x.y;
    }
}
__global__ void k_join_pairs(const uint32_t* __restrict__ k, const uint32_t* __restrict__ v, int n, uint2* __restrict__ kv) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) kv[i] = make_uint2(k[i], v[i]);
}

// the reference's bound search, one thread per element of the sorted pairs: a key boundary
// between element i-1 and i writes lower[key(i)] = i and upper[key(i-1)] = i; buckets with no
// element are left as they are; keys outside [0, nDst) are skipped
__global__ void k_bound_search(const int2* __restrict__ src, int n, uint32_t* __restrict__ dst, int ndst, int upper) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += gridDim.x * blockDim.x) {
        if (!upper) {
            if (i >= n) continue;
            const int kj = src[i].x;
            if ((i == 0 || src[i - 1].x != kj) && kj >= 0 && kj < ndst) dst[kj] = (uint32_t)i;
        } else {
            if (i == 0) continue;
            const int ki = src[i - 1].x;
            const int kj = i == n ? ndst : src[i].x;
            if (ki != kj && ki >= 0 && ki < ndst) dst[ki] = (uint32_t)i;
        }
    }
}

__global__ void k_count(const uint32_t* __restrict__ lower, const uint32_t* __restrict__ upper, int ndst,
                        uint32_t* __restrict__ dst) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ndst; i += gridDim.x * blockDim.x)
        dst[i] = upper[i] - lower[i];
}

__global__ void k_fill(int* __restrict__ dst, int value, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = value;
}

b3gStatus sort_impl(int device, uint32_t* keys, uint32_t* vals, int n, int bits) {
    PRIM_TRY(cudaSetDevice(device), "cudaSetDevice");
    const PrimConfig pc = prim_config(device);
    const size_t words = 2 * (size_t)n + (vals ? 2 * (size_t)n : 0);
    Scratch buf, scratch;
    PRIM_TRY(cudaMalloc(&buf.p, words * sizeof(uint32_t) + 16), "cudaMalloc");
    PRIM_TRY(cudaMalloc(&scratch.p, radix_scratch_bytes(pc)), "cudaMalloc");
    uint32_t* kin = reinterpret_cast<uint32_t*>(buf.p);
    uint32_t* kalt = kin + n;
    uint32_t* vin = vals ? kalt + n : nullptr;
    uint32_t* valt = vals ? vin + n : nullptr;
    int* d_n = reinterpret_cast<int*>(kin + words);
    PRIM_TRY(cudaMemcpy(d_n, &n, sizeof(int), cudaMemcpyHostToDevice), "cudaMemcpy");
    PRIM_TRY(cudaMemcpy(kin, keys, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice), "cudaMemcpy");
    if (vals) PRIM_TRY(cudaMemcpy(vin, vals, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice), "cudaMemcpy");
    long long launches = 0;
    const int w = radix_sort_u32(pc, kin, kalt, vin, valt, d_n, bits, scratch.p, 0, &launches);
    PRIM_TRY(cudaGetLastError(), "radix sort launch");
    PRIM_TRY(cudaMemcpy(keys, w ? kalt : kin, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice), "cudaMemcpy");
    if (vals) PRIM_TRY(cudaMemcpy(vals, w ? valt : vin, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice), "cudaMemcpy");
    PRIM_TRY(cudaDeviceSynchronize(), "radix sort");
    return B3G_OK;
}

}  // namespace
}  // namespace b3g

using namespace b3g;

extern "C" b3gStatus b3g_radix_sort32(int cuda_device, void* d_key_values, int n, int sort_bits) {
    if (n < 0 || (n > 0 && !d_key_values)) return report_error(B3G_ERR_INVALID_ARG, "invalid sort arguments");
    if (sort_bits < 0 || sort_bits > 32) return report_error(B3G_ERR_INVALID_ARG, "sort_bits must be in [0, 32]");
    if (n < 2 || sort_bits == 0) return B3G_OK;
    PRIM_TRY(cudaSetDevice(cuda_device), "cudaSetDevice");
    Scratch sv;
    PRIM_TRY(cudaMalloc(&sv.p, 2 * sizeof(uint32_t) * (size_t)n), "cudaMalloc");
    uint32_t* k = reinterpret_cast<uint32_t*>(sv.p);
    uint32_t* v = k + n;
    k_split_pairs<<<256, 256>>>(reinterpret_cast<const uint2*>(d_key_values), n, k, v);
    PRIM_TRY(cudaGetLastError(), "split launch");
    b3gStatus st = sort_impl(cuda_device, k, v, n, sort_bits);
    if (st != B3G_OK) return st;
    k_join_pairs<<<256, 256>>>(k, v, n, reinterpret_cast<uint2*>(d_key_values));
    PRIM_TRY(cudaGetLastError(), "join launch");
    PRIM_TRY(cudaDeviceSynchronize(), "radix sort");
    return B3G_OK;
}

extern "C" b3gStatus b3g_radix_sort32_keys(int cuda_device, void* d_keys, int n, int sort_bits) {
    if (n < 0 || (n > 0 && !d_keys)) return report_error(B3G_ERR_INVALID_ARG, "invalid sort arguments");
    if (sort_bits < 0 || sort_bits > 32) return report_error(B3G_ERR_INVALID_ARG, "sort_bits must be in [0, 32]");
    if (n < 2 || sort_bits == 0) return B3G_OK;
    return sort_impl(cuda_device, reinterpret_cast<uint32_t*>(d_keys), nullptr, n, sort_bits);
}

extern "C" b3gStatus b3g_prefix_scan32(int cuda_device, const void* d_src, void* d_dst, int n, unsigned int* host_sum) {
    if (n < 0 || (n > 0 && (!d_src || !d_dst))) return report_error(B3G_ERR_INVALID_ARG, "invalid scan arguments");
    if (n == 0) {
        if (host_sum) *host_sum = 0;
        return B3G_OK;
    }
    PRIM_TRY(cudaSetDevice(cuda_device), "cudaSetDevice");
    const PrimConfig pc = prim_config(cuda_device);
    Scratch scratch, counts;
    PRIM_TRY(cudaMalloc(&scratch.p, scan_scratch_bytes(pc)), "cudaMalloc");
    PRIM_TRY(cudaMalloc(&counts.p, 2 * sizeof(int)), "cudaMalloc");
    int* d_n = reinterpret_cast<int*>(counts.p);
    PRIM_TRY(cudaMemcpy(d_n, &n, sizeof(int), cudaMemcpyHostToDevice), "cudaMemcpy");
    long long launches = 0;
    exclusive_scan_i32(pc, reinterpret_cast<const int*>(d_src), reinterpret_cast<int*>(d_dst), d_n, d_n + 1,
                       scratch.p, 0, &launches);
    PRIM_TRY(cudaGetLastError(), "scan launch");
    int total = 0;
    PRIM_TRY(cudaMemcpy(&total, d_n + 1, sizeof(int), cudaMemcpyDeviceToHost), "cudaMemcpy");
    if (host_sum) *host_sum = (unsigned int)total;
    return B3G_OK;
}

extern "C" b3gStatus b3g_bound_search(int cuda_device, const void* d_sorted_pairs, int n, void* d_dst, int n_dst,
                                      int option) {
    if (n < 0 || n_dst < 0 || (n > 0 && !d_sorted_pairs) || (n_dst > 0 && !d_dst))
        return report_error(B3G_ERR_INVALID_ARG, "invalid bound search arguments");
    if (option < B3G_BOUND_LOWER || option > B3G_BOUND_COUNT)
        return report_error(B3G_ERR_INVALID_ARG, "option must be B3G_BOUND_LOWER, _UPPER or _COUNT");
    PRIM_TRY(cudaSetDevice(cuda_device), "cudaSetDevice");
    const int2* src = reinterpret_cast<const int2*>(d_sorted_pairs);
    uint32_t* dst = reinterpret_cast<uint32_t*>(d_dst);
    if (option != B3G_BOUND_COUNT) {
        if (n > 0) k_bound_search<<<256, 256>>>(src, n, dst, n_dst, option == B3G_BOUND_UPPER);
        PRIM_TRY(cudaGetLastError(), "bound search launch");
        PRIM_TRY(cudaDeviceSynchronize(), "bound search");
        return B3G_OK;
    }
    // count = upper - lower, both starting from 0 for buckets without elements
    Scratch lu;
    PRIM_TRY(cudaMalloc(&lu.p, 2 * sizeof(uint32_t) * (size_t)(n_dst > 0 ? n_dst : 1)), "cudaMalloc");
    uint32_t* lower = reinterpret_cast<uint32_t*>(lu.p);
    uint32_t* upper = lower + n_dst;
    PRIM_TRY(cudaMemset(lu.p, 0, 2 * sizeof(uint32_t) * (size_t)n_dst), "cudaMemset");
    if (n > 0) {
        k_bound_search<<<256, 256>>>(src, n, lower, n_dst, 0);
        k_bound_search<<<256, 256>>>(src, n, upper, n_dst, 1);
    }
    if (n_dst > 0) k_count<<<64, 256>>>(lower, upper, n_dst, dst);
    PRIM_TRY(cudaGetLastError(), "bound search launch");
    PRIM_TRY(cudaDeviceSynchronize(), "bound search");
    return B3G_OK;
}

extern "C" b3gStatus b3g_fill32(int cuda_device, void* d_dst, int value, int n, int offset) {
    if (n < 0 || offset < 0 || (n > 0 && !d_dst)) return report_error(B3G_ERR_INVALID_ARG, "invalid fill arguments");
    if (n == 0) return B3G_OK;
    PRIM_TRY(cudaSetDevice(cuda_device), "cudaSetDevice");
    k_fill<<<256, 256>>>(reinterpret_cast<int*>(d_dst) + offset, value, n);
    PRIM_TRY(cudaGetLastError(), "fill launch");
    PRIM_TRY(cudaDeviceSynchronize(), "fill");
    return B3G_OK;
}
