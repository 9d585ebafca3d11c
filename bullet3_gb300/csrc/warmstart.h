// Learned warm start: model state shared by the C ABI (warmstart.cu) and the step (world.cu).
#ifndef B3G_WARMSTART_H
#define B3G_WARMSTART_H

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <vector>

#define WS_FEATURES 12
#define WS_OUTPUTS 3
#define WS_HIDDEN 128
#define WS_FEAT_PAD 16
#define WS_OUT_PAD 16
// public flat parameter count: W1[12x128] b1 W2[128x128] b2 W3[128x128] b3 W4[128x3] b4
#define WS_PARAMS (WS_FEATURES * WS_HIDDEN + WS_HIDDEN + 2 * (WS_HIDDEN * WS_HIDDEN + WS_HIDDEN) + WS_HIDDEN * WS_OUTPUTS + WS_OUTPUTS)
// normalisation: feature mean[12], feature 1/std[12], target mean[3], target 1/std[3]
#define WS_NORM (2 * WS_FEATURES + 2 * WS_OUTPUTS)

namespace b3g {
namespace mlp {

// Activation buffers for up to `cap` rows (cap a multiple of 64).
struct Acts {
    int cap = 0;
    __nv_bfloat16 *x_row = nullptr, *x_col = nullptr;
    float *pre[3] = {nullptr, nullptr, nullptr};
    __nv_bfloat16 *h_row[3] = {nullptr, nullptr, nullptr}, *h_col[3] = {nullptr, nullptr, nullptr};
    float* y = nullptr;
    __nv_bfloat16 *dy_row = nullptr, *dy_col = nullptr;
    __nv_bfloat16 *dp_row[3] = {nullptr, nullptr, nullptr}, *dp_col[3] = {nullptr, nullptr, nullptr};
};

struct Model {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    float* params = nullptr;      // padded FP32 masters
    float *adam_m = nullptr, *adam_v = nullptr, *grads = nullptr, *grad_w1t = nullptr;
    __nv_bfloat16 *wt1 = nullptr, *wt2 = nullptr, *w2 = nullptr, *wt3 = nullptr, *w3 = nullptr, *wt4 = nullptr,
                  *w4 = nullptr;
    float* norm = nullptr;        // device copy of the normalisation (WS_NORM floats)
    float norm_host[WS_NORM];
    Acts train;                   // training batch buffers
    Acts infer;                   // inference buffers (grown on demand)
    float* data_x = nullptr;      // uploaded training set
    float* data_t = nullptr;
    float* batch_t = nullptr;
    int data_n = 0;
    double* loss = nullptr;
    unsigned int* status = nullptr;
    long long adam_step = 0;
    std::vector<void*> allocations;
};

// Forward pass over rows of 12 float features (row stride ld_x floats), the row count read on
// the device (*d_rows, clamped to rows_cap); the predictions, in normalised units, are left in
// last_predictions().  Buffers for rows_cap rows must exist (ensure_infer).  Returns launches.
cudaError_t ensure_infer(Model& m, int rows_cap);
int forward_device(Model& m, const float* x, int ld_x, const int* d_rows, int rows_cap, cudaStream_t s);
// the device predictions of the last forward_device: [rows][WS_OUT_PAD] normalised units
const float* last_predictions(const Model& m);
// device target normalisation: mean[3], 1/std[3]
const float* target_norm(const Model& m);

}  // namespace mlp
}  // namespace b3g

#include "b3g_capi.h"
// the model behind a C handle (nullptr for nullptr)
b3g::mlp::Model* b3g_mlp_model(b3g_mlp m);

#endif
