// Tensor-core GEMM with fused epilogues, the building block of the warm-start MLP (mlp.cu).
#ifndef B3G_MLP_H
#define B3G_MLP_H

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stddef.h>

namespace b3g {
namespace mlp {

enum Epilogue {
    EPI_BIAS_F32 = 0,   // out_f32[r][n] = acc + bias[n]
    EPI_BIAS_GELU = 1,  // pre_out[r][n] = acc + bias[n]; h = GELU(pre) -> out_row (and out_col) in bf16
    EPI_DGELU = 2,      // d = acc * GELU'(pre_in[r][n]) -> out_row / out_col in bf16; atomic_out[n] += d
    EPI_ATOMIC = 3,     // atomic_out[r][n] += acc (split-K partial sums)
};

// D[rows x N] = A[rows x K] * B[N x K]^T: both operands bf16 and K-major (row i of A / row n of
// B holds K contiguous elements); rows from *d_rows (clamped to rows_cap) when d_rows != nullptr.
// K a multiple of 16 (rows of A / B padded with zeros), N a multiple of 16 in 16..256, lda and
// ldb multiples of 8 and every row start 16-byte aligned.
struct GemmArgs {
    const __nv_bfloat16* A = nullptr;
    int lda = 0;
    const __nv_bfloat16* B = nullptr;
    int ldb = 0;
    int K = 0;
    int N = 0;
    int rows = 0;
    const int* d_rows = nullptr;
    int rows_cap = 0;
    int k_split = 1;          // CTAs sharing one 128-row tile along K (EPI_ATOMIC only)
    int epi = EPI_BIAS_F32;
    const float* bias = nullptr;
    float* out_f32 = nullptr;  // EPI_BIAS_F32
    float* pre_out = nullptr;  // EPI_BIAS_GELU (optional)
    const float* pre_in = nullptr;  // EPI_DGELU
    int ld_out = 0;            // row stride of out_f32 / pre_out / pre_in / atomic_out (EPI_ATOMIC)
    __nv_bfloat16* out_row = nullptr;
    int ld_row = 0;
    __nv_bfloat16* out_col = nullptr;  // column-major copy: out_col[n * ld_col + r]
    int ld_col = 0;
    float* atomic_out = nullptr;
    unsigned int* status = nullptr;    // B3G_FLAG_MLP_TIMEOUT on a wait that gave up
};

size_t gemm_smem_bytes(int N);
cudaError_t gemm_prepare();  // once per device: the dynamic shared-memory attributes (GEMM and inference)
void launch_gemm(const GemmArgs& g, int grid, cudaStream_t s);

// The whole forward pass of the 16 (12 used) -> 128 -> 128 -> 128 -> 16 (3 used) network on one
// SM per 128-row tile: the four weight matrices stay in shared memory, each layer's activations go
// from TMEM through the epilogue back into shared memory as the next layer's A operand; only the
// features are read and the FP32 outputs written.  The same MMA sequence, biases, GELU and bf16
// roundings as the layer-by-layer GEMMs, so the same outputs.
struct InferArgs {
    const float* x = nullptr;  // features, WS_FEATURES used of ld_x per row
    int ld_x = 0;
    const int* d_rows = nullptr;  // rows on the device, clamped to rows_cap
    int rows_cap = 0;
    const float* norm = nullptr;  // feature mean[12], 1/std[12]
    const __nv_bfloat16 *wt1 = nullptr, *wt2 = nullptr, *wt3 = nullptr, *wt4 = nullptr;  // [N][K] K-major
    const float *b1 = nullptr, *b2 = nullptr, *b3 = nullptr, *b4 = nullptr;
    float* y = nullptr;  // [rows][16]
    unsigned int* status = nullptr;
};
void launch_infer(const InferArgs& a, int grid, cudaStream_t s);

}  // namespace mlp
}  // namespace b3g

#endif
