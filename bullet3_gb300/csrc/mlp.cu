// Warm-start MLP (12 -> 128 -> 128 -> 128 -> 3, GELU) on the 5th-generation tensor cores.
//
// Every product of the forward and backward pass is one call of k_gemm: D[128 x N] tiles are
// accumulated in tensor memory (TMEM) by tcgen05.mma (BF16 operands from shared memory, FP32
// accumulation), then read back with tcgen05.ld by the four warps of the CTA (warp w owns TMEM
// lanes 32w..32w+31, i.e. rows 32w..32w+31 of the tile) and finished by a fused epilogue: bias +
// GELU (forward), bias only (output layer), upstream gradient x GELU'(pre-activation) with bias
// gradient (backward), or split-K accumulation into FP32 weight gradients.
//
// Operand layout: both operands K-major (row r of A and row n of B hold their K elements
// contiguously in global memory).  A K-chunk of 64 is copied into shared memory in the
// canonical no-swizzle core-matrix layout: core matrix = 8 rows x 16 bytes; element (r, k) of a
// chunk lives at (r % 8) * 16 + (k % 8) * 2 + (k / 8) * 128 + (r / 8) * 1024 bytes, so the
// leading-dimension byte offset (next core matrix along K) is 128 and the stride-dimension byte
// offset (next 8-row group) is 1024.  One MMA consumes K = 16 (two core matrices along K).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "b3g_capi.h"
#include "mlp.h"
#include "warmstart.h"

namespace b3g {
namespace mlp {

static constexpr int GT = 128;         // threads per GEMM CTA (4 warps = 128 TMEM lanes)
static constexpr int KC = 64;          // K elements per shared-memory chunk
static constexpr int SBO = 1024;       // bytes between 8-row groups in a chunk (KC / 8 * 128)
static constexpr int LBO = 128;        // bytes between core matrices along K
static constexpr unsigned WAIT_LIMIT = 1u << 22;

// ---------------------------------------------------------------------------- PTX wrappers
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t sbo = SBO) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFFu);              // start address
    d |= (uint64_t)((LBO >> 4) & 0x3FFFu) << 16;         // leading-dimension byte offset (along K)
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;         // stride-dimension byte offset (8-row groups)
    d |= (uint64_t)1 << 46;                              // descriptor version for tcgen05
    // base offset 0, absolute LBO mode 0, layout type 0 = no swizzle
    return d;
}

// kind::f16 instruction descriptor: D = F32, A = B = BF16, both K-major, M = 128, N = n
__host__ __device__ constexpr uint32_t instr_desc(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_commit(unsigned long long* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long* bar, unsigned parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
    for (unsigned i = 0; i < WAIT_LIMIT; i++) {
        if (mbar_test(bar, parity)) return true;
        __nanosleep(20);
    }
    return false;
}
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// ---------------------------------------------------------------------------- activation
// GELU(x) = x * Phi(x) (exact, erf form) and its derivative Phi(x) + x * phi(x)
__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
    const float cdf = 0.5f * (1.f + erff(x * 0.70710678118654752f));
    const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
    return cdf + x * pdf;
}

// ---------------------------------------------------------------------------- the GEMM
// Copies rows [r0, r0 + nrows_tile) x K [k0, k0 + kc) of a K-major bf16 matrix into the chunk
// layout; rows >= rows_valid and K >= kend are zero.
__device__ __forceinline__ void load_chunk(char* dst, const __nv_bfloat16* src, int ld, int r0, int nrows_tile,
                                           int rows_valid, int k0, int kend) {
    const int pieces = nrows_tile * (KC / 8);
    for (int p = threadIdx.x; p < pieces; p += blockDim.x) {
        const int r = p / (KC / 8), kq = p % (KC / 8);
        const int row = r0 + r, k = k0 + kq * 8;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (row < rows_valid && k < kend) v = *reinterpret_cast<const uint4*>(src + (size_t)row * ld + k);
        *reinterpret_cast<uint4*>(dst + (r & 7) * 16 + kq * LBO + (r >> 3) * SBO) = v;
    }
}

__global__ void __launch_bounds__(GT) k_gemm(GemmArgs g) {
    extern __shared__ __align__(1024) char smem[];
    char* sA = smem;                       // 128 x KC bf16 = 16 KB
    char* sB = smem + 128 * KC * 2;        // N x KC bf16
    __shared__ unsigned long long bar;
    __shared__ uint32_t tslot;
    bool failed = false;  // block-uniform: set from a __syncthreads_or
    const int N = g.N;
    const uint32_t ncols = N <= 32 ? 32u : (N <= 64 ? 64u : (N <= 128 ? 128u : 256u));
    const int rows = g.d_rows ? min(*g.d_rows, g.rows_cap) : g.rows;
    const int m_tiles = (rows + 127) / 128;
    const int units = m_tiles * g.k_split;
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    if (threadIdx.x < 32) tmem_alloc(&tslot, ncols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tslot;
    const uint32_t idesc = instr_desc(N);
    unsigned phase = 0;
    const int ksteps_total = (g.K + 15) / 16;
    const int kchunks_total = (g.K + KC - 1) / KC;
    const int chunks_per_part = (kchunks_total + g.k_split - 1) / g.k_split;
    for (int u = blockIdx.x; u < units && !failed; u += gridDim.x) {
        const int mt = u % m_tiles, part = u / m_tiles;
        const int r0 = mt * 128;
        const int c_beg = part * chunks_per_part, c_end = min(kchunks_total, c_beg + chunks_per_part);
        if (c_beg >= c_end) continue;
        for (int c = c_beg; c < c_end; c++) {
            const int k0 = c * KC;
            load_chunk(sA, g.A, g.lda, r0, 128, rows, k0, g.K);
            load_chunk(sB, g.B, g.ldb, 0, N, N, k0, g.K);
            fence_async_smem();
            tc_fence_before();
            __syncthreads();
            tc_fence_after();
            if (threadIdx.x == 0) {
                const int steps = min(KC / 16, ksteps_total - k0 / 16);
                for (int s = 0; s < steps; s++) {
                    const uint64_t ad = smem_desc(smem_u32(sA) + s * 2 * LBO);
                    const uint64_t bd = smem_desc(smem_u32(sB) + s * 2 * LBO);
                    mma_bf16(tmem, ad, bd, idesc, (c > c_beg || s > 0) ? 1u : 0u);
                }
                mma_commit(&bar);
            }
            // the chunk buffers are rewritten next round: wait until the MMAs have read them
            const bool ok = mbar_wait(&bar, phase);
            phase ^= 1u;
            if (__syncthreads_or(!ok)) {
                failed = true;
                if (threadIdx.x == 0) {
                    if (g.status) atomicOr(g.status, B3G_FLAG_MLP_TIMEOUT);
                    mbar_wait(&bar, phase ^ 1u);  // drain: one more bounded wait for the MMAs in flight
                }
                break;
            }
            tc_fence_after();
        }
        if (failed) break;
        // ---- epilogue: thread t owns row r0 + t of the tile
        const int r = r0 + threadIdx.x;
        const uint32_t trow = tmem + ((uint32_t)(threadIdx.x & ~31) << 16);
        for (int n0 = 0; n0 < N; n0 += 16) {
            float v[16];
            tmem_ld16(trow + n0, v);
            if (g.epi == EPI_DGELU) {
                // every lane takes part in the warp sums of the bias gradient (rows past the end
                // add zero), so the rows are masked instead of skipped
#pragma unroll
                for (int i = 0; i < 16; i++) {
                    const int n = n0 + i;
                    float hv = 0.f;
                    if (r < rows) {
                        const float d = v[i] * gelu_grad(g.pre_in[(size_t)r * g.ld_out + n]);
                        const __nv_bfloat16 hb = __float2bfloat16_rn(d);
                        if (g.out_row) g.out_row[(size_t)r * g.ld_row + n] = hb;
                        if (g.out_col) g.out_col[(size_t)n * g.ld_col + r] = hb;
                        hv = __bfloat162float(hb);
                    }
                    // bias gradient: sum of the rounded values, as the next layer consumes them,
                    // over the warp's 32 rows first, one atomic per warp
                    if (g.atomic_out) {
                        for (int o = 16; o; o >>= 1) hv += __shfl_xor_sync(0xffffffffu, hv, o);
                        if ((threadIdx.x & 31) == 0) atomicAdd(&g.atomic_out[n], hv);
                    }
                }
                continue;
            }
            if (r >= rows) continue;
#pragma unroll
            for (int i = 0; i < 16; i++) {
                const int n = n0 + i;
                float x = v[i];
                switch (g.epi) {
                    case EPI_BIAS_F32:
                        g.out_f32[(size_t)r * g.ld_out + n] = x + g.bias[n];
                        break;
                    case EPI_BIAS_GELU: {
                        const float pre = x + g.bias[n];
                        if (g.pre_out) g.pre_out[(size_t)r * g.ld_out + n] = pre;
                        const __nv_bfloat16 h = __float2bfloat16_rn(gelu(pre));
                        g.out_row[(size_t)r * g.ld_row + n] = h;
                        if (g.out_col) g.out_col[(size_t)n * g.ld_col + r] = h;
                        break;
                    }
                    case EPI_ATOMIC:
                        atomicAdd(&g.atomic_out[(size_t)r * g.ld_out + n], x);
                        break;
                }
            }
        }
        tc_fence_before();
        __syncthreads();  // TMEM reads done before the next tile's MMAs overwrite it
        tc_fence_after();
    }
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x < 32) tmem_dealloc(tmem, ncols);
}

size_t gemm_smem_bytes(int N) { return (size_t)128 * KC * 2 + (size_t)N * KC * 2; }

// ---------------------------------------------------------------------------- fused inference
// Shared memory, every block 1 KB aligned: W1 (128 x 16) and the tile's inputs (128 x 16) in a
// 16-wide layout (core matrices of 8 rows x 8 K as in load_chunk, 256 bytes between 8-row groups),
// W2 and W3 (128 x 128, two 64-K chunks each), W4 (16 x 128, two 16-row chunks) and the
// activations (128 x 128, two chunks) in the chunk layout of load_chunk; 108 KB, so two CTAs share
// an SM.  Eight warps: the TMEM lane quarter of warp w is w % 4 (rows 32 (w % 4) ..), warps 0-3 take
// columns 0-63 of each hidden layer's epilogue and warps 4-7 columns 64-127.
static constexpr int FIN = 16, FOUT = 16, HID = 128, IT = 256;
static constexpr size_t CH128 = 128 * KC * 2;  // a 128-row chunk: 16 KB
static constexpr size_t CH16 = 16 * KC * 2;    // a 16-row chunk: 2 KB
static constexpr uint32_t SBO16 = 256;         // 8-row group stride of the 16-wide layout
static constexpr size_t N16 = 128 * FIN * 2;   // a 128 x 16 operand: 4 KB
static constexpr size_t S_W1 = 0, S_X = S_W1 + N16, S_W2 = S_X + N16, S_W3 = S_W2 + 2 * CH128,
                        S_W4 = S_W3 + 2 * CH128, S_H = S_W4 + 2 * CH16, S_END = S_H + 2 * CH128;

// 16 values (bf16) of row r at columns n0..n0+15 of a K-chunked 128-row operand (base: chunk 0)
__device__ __forceinline__ void put_row16(char* base, int r, int n0, const float* v, uint32_t sbo, size_t chunk_bytes) {
    uint32_t w[8];
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
        w[i] = *reinterpret_cast<const uint32_t*>(&h);
    }
    char* chunk = base + (size_t)(n0 / KC) * chunk_bytes;
    const int k = n0 % KC;
    char* row = chunk + (r & 7) * 16 + (r >> 3) * sbo;
    *reinterpret_cast<uint4*>(row + (k / 8) * LBO) = make_uint4(w[0], w[1], w[2], w[3]);
    *reinterpret_cast<uint4*>(row + (k / 8 + 1) * LBO) = make_uint4(w[4], w[5], w[6], w[7]);
}

// the rows of a K-major bf16 matrix with 16 K elements into the 16-wide layout
__device__ __forceinline__ void load16(char* dst, const __nv_bfloat16* src, int nrows) {
    for (int p = threadIdx.x; p < nrows * 2; p += blockDim.x) {
        const int r = p >> 1, kq = p & 1;
        *reinterpret_cast<uint4*>(dst + (r & 7) * 16 + kq * LBO + (r >> 3) * SBO16) =
            *reinterpret_cast<const uint4*>(src + (size_t)r * FIN + kq * 8);
    }
}

__global__ void __launch_bounds__(IT, 2) k_mlp_infer(InferArgs a) {
    extern __shared__ __align__(1024) char smem[];
    __shared__ unsigned long long bar;
    __shared__ uint32_t tslot;
    const int rows = min(*a.d_rows, a.rows_cap);
    const int m_tiles = (rows + 127) / 128;
    if ((int)blockIdx.x >= m_tiles) return;  // block-uniform, before any barrier or TMEM use
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    if (threadIdx.x < 32) tmem_alloc(&tslot, HID);
    load16(smem + S_W1, a.wt1, HID);
    for (int c = 0; c < 2; c++) {
        load_chunk(smem + S_W2 + c * CH128, a.wt2, HID, 0, HID, HID, c * KC, HID);
        load_chunk(smem + S_W3 + c * CH128, a.wt3, HID, 0, HID, HID, c * KC, HID);
        load_chunk(smem + S_W4 + c * CH16, a.wt4, HID, 0, FOUT, FOUT, c * KC, HID);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tslot;
    const int t = threadIdx.x;
    const int lane_row = t & 127;        // this thread's row of the tile (its TMEM lane)
    const int half = t >> 7;             // 0: columns 0-63, 1: columns 64-127
    const uint32_t trow = tmem + ((uint32_t)(lane_row & ~31) << 16);
    unsigned phase = 0;
    bool failed = false;
    // one layer: MMAs of K = 16 over `chunks` K-chunks of A at sA and B at sB; false when the wait
    // gave up (the status flag is set and the MMAs drained)
    auto layer = [&](uint32_t sA, size_t a_chunk, uint32_t sB, size_t b_chunk, uint32_t sbo, int chunks, int steps,
                     uint32_t idesc) -> bool {
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (t == 0) {
            for (int c = 0; c < chunks; c++)
                for (int s = 0; s < steps; s++) {
                    const uint64_t ad = smem_desc(sA + (uint32_t)(c * a_chunk) + s * 2 * LBO, sbo);
                    const uint64_t bd = smem_desc(sB + (uint32_t)(c * b_chunk) + s * 2 * LBO, sbo);
                    mma_bf16(tmem, ad, bd, idesc, (c > 0 || s > 0) ? 1u : 0u);
                }
            mma_commit(&bar);
        }
        const bool ok = mbar_wait(&bar, phase);
        phase ^= 1u;
        if (__syncthreads_or(!ok)) {
            if (t == 0) {
                if (a.status) atomicOr(a.status, B3G_FLAG_MLP_TIMEOUT);
                mbar_wait(&bar, phase ^ 1u);
            }
            return false;
        }
        tc_fence_after();
        return true;
    };
    const uint32_t sX = smem_u32(smem + S_X), sH = smem_u32(smem + S_H);
    const float* bias[3] = {a.b1, a.b2, a.b3};
    for (int tile = blockIdx.x; tile < m_tiles && !failed; tile += gridDim.x) {
        const int r = tile * 128 + lane_row;
        if (half == 0) {
            // the normalised features of row r (k_pack's arithmetic), zero past the rows
            float v[16];
#pragma unroll
            for (int f = 0; f < 16; f++)
                v[f] = (r < rows && f < WS_FEATURES) ? (a.x[(size_t)r * a.ld_x + f] - a.norm[f]) * a.norm[WS_FEATURES + f]
                                                    : 0.f;
            put_row16(smem + S_X, lane_row, 0, v, SBO16, N16);
        }
        for (int l = 0; l < 3; l++) {
            const bool ok = l == 0 ? layer(sX, N16, smem_u32(smem + S_W1), N16, SBO16, 1, 1, instr_desc(HID))
                                   : layer(sH, CH128, smem_u32(smem + (l == 1 ? S_W2 : S_W3)), CH128, SBO, 2,
                                           KC / 16, instr_desc(HID));
            if (!ok) { failed = true; break; }
            for (int n0 = half * 64; n0 < half * 64 + 64; n0 += 16) {
                float v[16];
                tmem_ld16(trow + n0, v);
#pragma unroll
                for (int i = 0; i < 16; i++) v[i] = gelu(v[i] + bias[l][n0 + i]);
                put_row16(smem + S_H, lane_row, n0, v, SBO, CH128);
            }
            tc_fence_before();  // TMEM reads done before the next layer's MMAs overwrite it
        }
        if (failed) break;
        if (!layer(sH, CH128, smem_u32(smem + S_W4), CH16, SBO, 2, KC / 16, instr_desc(FOUT))) { failed = true; break; }
        if (half == 0) {
            float v[16];
            tmem_ld16(trow, v);
            if (r < rows) {
                float4* out = reinterpret_cast<float4*>(a.y + (size_t)r * FOUT);
#pragma unroll
                for (int q = 0; q < 4; q++)
                    out[q] = make_float4(v[4 * q] + a.b4[4 * q], v[4 * q + 1] + a.b4[4 * q + 1],
                                         v[4 * q + 2] + a.b4[4 * q + 2], v[4 * q + 3] + a.b4[4 * q + 3]);
            }
        }
        tc_fence_before();
        __syncthreads();  // TMEM reads done before the next tile's MMAs
        tc_fence_after();
    }
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x < 32) tmem_dealloc(tmem, HID);
}

void launch_infer(const InferArgs& a, int grid, cudaStream_t s) { k_mlp_infer<<<grid, IT, S_END, s>>>(a); }

cudaError_t gemm_prepare() {
    cudaError_t e = cudaFuncSetAttribute(k_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gemm_smem_bytes(256));
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S_END);
    return e;
}

void launch_gemm(const GemmArgs& g, int grid, cudaStream_t s) {
    k_gemm<<<grid, GT, gemm_smem_bytes(g.N), s>>>(g);
}

}  // namespace mlp
}  // namespace b3g
