// The learned warm start: a 12 -> 128 -> 128 -> 128 -> 3 GELU network that predicts the converged
// normal and friction impulses of a contact point from local contact features.  Weights live on
// the device as FP32 masters (Adam) with BF16 copies in both orientations for the tensor-core
// GEMMs of mlp.cu; training and inference run entirely on the GPU.  No counterpart in the
// reference (its solvers start cold or from the previous step's impulses).
//
// Features (12 per contact point, computed where the solver rows are set up):
//   0-2  relative velocity of A w.r.t. B at the contact point (world frame)
//   3-5  contact normal (world frame, B -> A)
//   6    separation (negative = penetration)
//   7,8  inverse masses of A and B
//   9    points in the manifold
//   10   |tangential relative velocity|
//   11   dt * (gravity . normal)
// Targets (3): converged applied impulses of the point's contact row and of its two friction
// rows (second direction, then first, the order the rows are solved in).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "b3g_capi.h"
#include "mlp.h"
#include "warmstart.h"
#include "world_internal.h"

namespace b3g {
namespace mlp {

static constexpr int H = WS_HIDDEN;
static constexpr int FI = WS_FEAT_PAD;   // padded input width
static constexpr int FO = WS_OUT_PAD;    // padded output width

// padded FP32 parameter layout on the device
static constexpr size_t OFF_W1 = 0;                      // [FI][H]
static constexpr size_t OFF_B1 = OFF_W1 + FI * H;        // [H]
static constexpr size_t OFF_W2 = OFF_B1 + H;             // [H][H]
static constexpr size_t OFF_B2 = OFF_W2 + H * H;
static constexpr size_t OFF_W3 = OFF_B2 + H;
static constexpr size_t OFF_B3 = OFF_W3 + H * H;
static constexpr size_t OFF_W4 = OFF_B3 + H;             // [H][FO]
static constexpr size_t OFF_B4 = OFF_W4 + H * FO;        // [FO]
static constexpr size_t NPAD = OFF_B4 + FO;

// ---------------------------------------------------------------------------- kernels
// features (float, 12 per row) -> normalised bf16 rows of FI (and the column-major copy)
__global__ void k_pack(const float* __restrict__ x, int ld_x, const int* __restrict__ d_rows, int rows_host,
                       int rows_cap, const float* __restrict__ norm, __nv_bfloat16* __restrict__ xr,
                       __nv_bfloat16* __restrict__ xc, int ld_c, int pad_rows) {
    const int rows = d_rows ? min(*d_rows, rows_cap) : rows_host;
    const int total = max(rows, pad_rows);
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < total; r += gridDim.x * blockDim.x) {
        for (int f = 0; f < FI; f++) {
            float v = 0.f;
            if (r < rows && f < WS_FEATURES) v = (x[(size_t)r * ld_x + f] - norm[f]) * norm[WS_FEATURES + f];
            const __nv_bfloat16 b = __float2bfloat16_rn(v);
            xr[(size_t)r * FI + f] = b;
            if (xc) xc[(size_t)f * ld_c + r] = b;
        }
    }
}

// mean-squared-error gradient in normalised target units; rows >= n are padding (zero gradient)
__global__ void k_loss(const float* __restrict__ y, const float* __restrict__ t, int n, int pad_rows,
                       const float* __restrict__ tnorm, __nv_bfloat16* __restrict__ dyr, __nv_bfloat16* __restrict__ dyc,
                       int ld_c, float* __restrict__ db4, double* __restrict__ loss) {
    const float scale = 2.f / (3.f * (float)n);
    double acc = 0.0;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < pad_rows; r += gridDim.x * blockDim.x) {
        for (int o = 0; o < FO; o++) {
            float d = 0.f;
            if (r < n && o < WS_OUTPUTS) {
                const float e = y[(size_t)r * FO + o] - (t[(size_t)r * WS_OUTPUTS + o] - tnorm[o]) * tnorm[WS_OUTPUTS + o];
                acc += (double)e * e;
                d = scale * e;
            }
            const __nv_bfloat16 b = __float2bfloat16_rn(d);
            dyr[(size_t)r * FO + o] = b;
            dyc[(size_t)o * ld_c + r] = b;
            if (o < WS_OUTPUTS && d != 0.f) atomicAdd(&db4[o], __bfloat162float(b));
        }
    }
    for (int s = 16; s; s >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, s);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc / (3.0 * n));
}

// Adam on the padded FP32 parameters (padding stays zero: its gradients are zero), then the
// bf16 copies: Wt (out x in, forward B operand) and W (in x out, backward B operand).
__global__ void k_adam(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ g, const float* __restrict__ g_w1t, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < NPAD; i += (size_t)gridDim.x * blockDim.x) {
        float gi;
        if (i < OFF_B1) {  // W1[in][out] gradient arrives transposed: g_w1t[out][in]
            const size_t in = i / H, out = i % H;
            gi = in < WS_FEATURES ? g_w1t[out * FI + in] : 0.f;
        } else if (i >= OFF_W4 && i < OFF_B4) {
            gi = ((i - OFF_W4) % FO) < WS_OUTPUTS ? g[i] : 0.f;
        } else if (i >= OFF_B4) {
            gi = (i - OFF_B4) < WS_OUTPUTS ? g[i] : 0.f;
        } else {
            gi = g[i];
        }
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] = p[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    }
}

__global__ void k_to_bf16(const float* __restrict__ p, __nv_bfloat16* __restrict__ wt1, __nv_bfloat16* __restrict__ wt2,
                          __nv_bfloat16* __restrict__ w2, __nv_bfloat16* __restrict__ wt3, __nv_bfloat16* __restrict__ w3,
                          __nv_bfloat16* __restrict__ wt4, __nv_bfloat16* __restrict__ w4) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    for (int i = t; i < FI * H; i += stride) {  // W1[in][out] -> Wt1[out][in]
        const int in = i / H, out = i % H;
        wt1[out * FI + in] = __float2bfloat16_rn(p[OFF_W1 + i]);
    }
    for (int i = t; i < H * H; i += stride) {
        const int in = i / H, out = i % H;
        const __nv_bfloat16 a = __float2bfloat16_rn(p[OFF_W2 + i]), b = __float2bfloat16_rn(p[OFF_W3 + i]);
        w2[i] = a;
        wt2[out * H + in] = a;
        w3[i] = b;
        wt3[out * H + in] = b;
    }
    for (int i = t; i < H * FO; i += stride) {  // W4[in][out]
        const int in = i / FO, out = i % FO;
        const __nv_bfloat16 a = __float2bfloat16_rn(p[OFF_W4 + i]);
        w4[i] = a;
        wt4[out * H + in] = a;
    }
}

}  // namespace mlp
}  // namespace b3g

// ============================================================================ host side
namespace b3g {
namespace mlp {

static int round_up(int x, int m) { return (x + m - 1) / m * m; }

template <typename T>
static cudaError_t dalloc(Model& m, T** p, size_t count) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, (count ? count : 1) * sizeof(T));
    if (e != cudaSuccess) return e;
    m.allocations.push_back(q);
    *p = static_cast<T*>(q);
    return cudaSuccess;
}

#define WS_CUDA(expr)                          \
    do {                                       \
        cudaError_t _e = (expr);               \
        if (_e != cudaSuccess) return _e;      \
    } while (0)

static cudaError_t alloc_acts(Model& m, Acts& a, int cap, bool training) {
    a.cap = cap;
    WS_CUDA(dalloc(m, &a.x_row, (size_t)cap * FI));
    // inference ping-pongs two activation buffers; training keeps all three for the backward pass
    for (int l = 0; l < (training ? 3 : 2); l++) WS_CUDA(dalloc(m, &a.h_row[l], (size_t)cap * H));
    WS_CUDA(dalloc(m, &a.y, (size_t)cap * FO));
    if (!training) return cudaSuccess;
    WS_CUDA(dalloc(m, &a.x_col, (size_t)cap * FI));
    for (int l = 0; l < 3; l++) {
        WS_CUDA(dalloc(m, &a.pre[l], (size_t)cap * H));
        WS_CUDA(dalloc(m, &a.h_col[l], (size_t)cap * H));
        WS_CUDA(dalloc(m, &a.dp_row[l], (size_t)cap * H));
        WS_CUDA(dalloc(m, &a.dp_col[l], (size_t)cap * H));
    }
    WS_CUDA(dalloc(m, &a.dy_row, (size_t)cap * FO));
    WS_CUDA(dalloc(m, &a.dy_col, (size_t)cap * FO));
    return cudaSuccess;
}

static int gemm_grid(const Model& m, int rows_cap) {
    const int tiles = (rows_cap + 127) / 128;
    return tiles < m.num_sms * 2 ? (tiles > 0 ? tiles : 1) : m.num_sms * 2;
}

// the four layers; with `training` the pre-activations and column-major copies are kept
static int run_forward(Model& m, Acts& a, const int* d_rows, int rows, int rows_cap, bool training, cudaStream_t s) {
    const int grid = gemm_grid(m, rows_cap);
    const __nv_bfloat16* wt[3] = {m.wt1, m.wt2, m.wt3};
    const size_t boff[3] = {OFF_B1, OFF_B2, OFF_B3};
    auto hbuf = [&](int l) { return a.h_row[training ? l : (l & 1)]; };
    for (int l = 0; l < 3; l++) {
        GemmArgs g;
        g.A = l == 0 ? a.x_row : hbuf(l - 1);
        g.lda = l == 0 ? FI : H;
        g.B = wt[l];
        g.ldb = l == 0 ? FI : H;
        g.K = l == 0 ? FI : H;
        g.N = H;
        g.rows = rows;
        g.d_rows = d_rows;
        g.rows_cap = rows_cap;
        g.epi = EPI_BIAS_GELU;
        g.bias = m.params + boff[l];
        g.pre_out = training ? a.pre[l] : nullptr;
        g.ld_out = H;
        g.out_row = hbuf(l);
        g.ld_row = H;
        g.out_col = training ? a.h_col[l] : nullptr;
        g.ld_col = a.cap;
        g.status = m.status;
        launch_gemm(g, grid, s);
    }
    GemmArgs g;
    g.A = hbuf(2);
    g.lda = H;
    g.B = m.wt4;
    g.ldb = H;
    g.K = H;
    g.N = FO;
    g.rows = rows;
    g.d_rows = d_rows;
    g.rows_cap = rows_cap;
    g.epi = EPI_BIAS_F32;
    g.bias = m.params + OFF_B4;
    g.out_f32 = a.y;
    g.ld_out = FO;
    g.status = m.status;
    launch_gemm(g, grid, s);
    return 4;
}

// gradients of the mean-squared error for one batch of `rows` rows (padded to a.cap) into
// m.grads / m.grad_w1t (zeroed here); the batch's inputs are already packed in a.x_row/x_col
static void run_backward(Model& m, Acts& a, int rows, const float* t, cudaStream_t s) {
    cudaMemsetAsync(m.grads, 0, sizeof(float) * NPAD, s);
    cudaMemsetAsync(m.grad_w1t, 0, sizeof(float) * H * FI, s);
    const int pad = a.cap;
    k_loss<<<m.num_sms * 2, 256, 0, s>>>(a.y, t, rows, pad, m.norm + 2 * WS_FEATURES, a.dy_row, a.dy_col, a.cap,
                                         m.grads + OFF_B4, m.loss);
    const int grid = gemm_grid(m, pad);
    const int ksplit = m.num_sms;  // split the batch reduction of the weight gradients
    const __nv_bfloat16* wrow[3] = {nullptr, m.w2, m.w3};
    const size_t boff[3] = {OFF_B1, OFF_B2, OFF_B3};
    const size_t woff[3] = {OFF_W1, OFF_W2, OFF_W3};
    // layer 4: dH3 = dY W4^T, dPre3 = dH3 * GELU'(pre3); dW4 = H3^T dY
    for (int l = 2; l >= 0; l--) {
        GemmArgs g;
        g.A = l == 2 ? a.dy_row : a.dp_row[l + 1];
        g.lda = l == 2 ? FO : H;
        g.B = l == 2 ? m.w4 : wrow[l + 1];
        g.ldb = l == 2 ? FO : H;
        g.K = l == 2 ? FO : H;
        g.N = H;
        g.rows = pad;
        g.epi = EPI_DGELU;
        g.pre_in = a.pre[l];
        g.ld_out = H;
        g.out_row = l > 0 ? a.dp_row[l] : nullptr;
        g.ld_row = H;
        g.out_col = a.dp_col[l];
        g.ld_col = a.cap;
        g.atomic_out = m.grads + boff[l];
        g.status = m.status;
        launch_gemm(g, grid, s);
        // weight gradient of the layer above: dW(l+1) = H_l^T dPre(l+1)  (128 x N, reduction over rows)
        GemmArgs w;
        w.A = a.h_col[l];
        w.lda = a.cap;
        w.B = l == 2 ? a.dy_col : a.dp_col[l + 1];
        w.ldb = a.cap;
        w.K = pad;
        w.N = l == 2 ? FO : H;
        w.rows = H;
        w.k_split = ksplit;
        w.epi = EPI_ATOMIC;
        w.atomic_out = m.grads + (l == 2 ? OFF_W4 : woff[l + 1]);
        w.ld_out = l == 2 ? FO : H;
        w.status = m.status;
        launch_gemm(w, ksplit, s);
    }
    // first layer: dW1^T = dPre1^T X  (128 x 16)
    GemmArgs w;
    w.A = a.dp_col[0];
    w.lda = a.cap;
    w.B = a.x_col;
    w.ldb = a.cap;
    w.K = pad;
    w.N = FI;
    w.rows = H;
    w.k_split = ksplit;
    w.epi = EPI_ATOMIC;
    w.atomic_out = m.grad_w1t;
    w.ld_out = FI;
    w.status = m.status;
    launch_gemm(w, ksplit, s);
}

static void refresh_bf16(Model& m, cudaStream_t s) {
    k_to_bf16<<<m.num_sms, 256, 0, s>>>(m.params, m.wt1, m.wt2, m.w2, m.wt3, m.w3, m.wt4, m.w4);
}

cudaError_t ensure_infer(Model& m, int rows_cap) {
    rows_cap = round_up(rows_cap < 64 ? 64 : rows_cap, 64);
    if (m.infer.cap >= rows_cap) return cudaSuccess;
    // grow: the old buffers stay owned by the model until it is destroyed
    return alloc_acts(m, m.infer, rows_cap, false);
}

int forward_device(Model& m, const float* x, int ld_x, const int* d_rows, int rows_cap, cudaStream_t s) {
    // the fused on-chip forward pass (mlp.cu k_mlp_infer): the same outputs as packing the features
    // and running the four layer GEMMs, with the activations kept in shared memory and TMEM
    InferArgs a;
    a.x = x;
    a.ld_x = ld_x;
    a.d_rows = d_rows;
    a.rows_cap = rows_cap;
    a.norm = m.norm;
    a.wt1 = m.wt1;
    a.wt2 = m.wt2;
    a.wt3 = m.wt3;
    a.wt4 = m.wt4;
    a.b1 = m.params + OFF_B1;
    a.b2 = m.params + OFF_B2;
    a.b3 = m.params + OFF_B3;
    a.b4 = m.params + OFF_B4;
    a.y = m.infer.y;
    a.status = m.status;
    const int tiles = (rows_cap + 127) / 128;
    launch_infer(a, tiles < 2 * m.num_sms ? (tiles > 0 ? tiles : 1) : 2 * m.num_sms, s);  // two CTAs an SM
    return 1;
}

const float* last_predictions(const Model& m) { return m.infer.y; }

const float* target_norm(const Model& m) { return m.norm + 2 * WS_FEATURES; }

}  // namespace mlp
}  // namespace b3g

// ============================================================================ C ABI
using b3g::mlp::Model;

struct b3gMlpImpl {
    Model m;
};

namespace {

b3gStatus ws_fail(b3gStatus st, const char* msg) { return b3g::report_error(st, msg); }

#define WS_TRY(expr)                                                                  \
    do {                                                                              \
        cudaError_t _e = (expr);                                                      \
        if (_e != cudaSuccess) return ws_fail(B3G_ERR_CUDA, cudaGetErrorString(_e));  \
    } while (0)

using namespace b3g::mlp;

// public flat layout <-> padded device layout
void to_padded(const float* p, std::vector<float>& d) {
    d.assign(NPAD, 0.f);
    size_t k = 0;
    for (int i = 0; i < WS_FEATURES; i++)
        for (int o = 0; o < H; o++) d[OFF_W1 + i * H + o] = p[k++];
    for (int o = 0; o < H; o++) d[OFF_B1 + o] = p[k++];
    for (int i = 0; i < H * H; i++) d[OFF_W2 + i] = p[k++];
    for (int o = 0; o < H; o++) d[OFF_B2 + o] = p[k++];
    for (int i = 0; i < H * H; i++) d[OFF_W3 + i] = p[k++];
    for (int o = 0; o < H; o++) d[OFF_B3 + o] = p[k++];
    for (int i = 0; i < H; i++)
        for (int o = 0; o < WS_OUTPUTS; o++) d[OFF_W4 + i * FO + o] = p[k++];
    for (int o = 0; o < WS_OUTPUTS; o++) d[OFF_B4 + o] = p[k++];
}
void from_padded(const std::vector<float>& d, float* p) {
    size_t k = 0;
    for (int i = 0; i < WS_FEATURES; i++)
        for (int o = 0; o < H; o++) p[k++] = d[OFF_W1 + i * H + o];
    for (int o = 0; o < H; o++) p[k++] = d[OFF_B1 + o];
    for (int i = 0; i < H * H; i++) p[k++] = d[OFF_W2 + i];
    for (int o = 0; o < H; o++) p[k++] = d[OFF_B2 + o];
    for (int i = 0; i < H * H; i++) p[k++] = d[OFF_W3 + i];
    for (int o = 0; o < H; o++) p[k++] = d[OFF_B3 + o];
    for (int i = 0; i < H; i++)
        for (int o = 0; o < WS_OUTPUTS; o++) p[k++] = d[OFF_W4 + i * FO + o];
    for (int o = 0; o < WS_OUTPUTS; o++) p[k++] = d[OFF_B4 + o];
}

b3gStatus upload_params(b3g_mlp m, const std::vector<float>& d) {
    WS_TRY(cudaSetDevice(m->m.device));
    WS_TRY(cudaMemcpyAsync(m->m.params, d.data(), sizeof(float) * NPAD, cudaMemcpyHostToDevice, m->m.stream));
    refresh_bf16(m->m, m->m.stream);
    WS_TRY(cudaStreamSynchronize(m->m.stream));
    return B3G_OK;
}

}  // namespace

extern "C" b3gStatus b3g_mlp_create(int cuda_device, unsigned long long seed, b3g_mlp* out) {
    if (!out) return ws_fail(B3G_ERR_INVALID_ARG, "null output");
    b3g_mlp m = new b3gMlpImpl();
    Model& M = m->m;
    M.device = cuda_device;
    cudaError_t e = cudaSetDevice(cuda_device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&M.num_sms, cudaDevAttrMultiProcessorCount, cuda_device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&M.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = gemm_prepare();
    if (e == cudaSuccess) e = dalloc(M, &M.params, NPAD);
    if (e == cudaSuccess) e = dalloc(M, &M.adam_m, NPAD);
    if (e == cudaSuccess) e = dalloc(M, &M.adam_v, NPAD);
    if (e == cudaSuccess) e = dalloc(M, &M.grads, NPAD);
    if (e == cudaSuccess) e = dalloc(M, &M.grad_w1t, (size_t)H * FI);
    if (e == cudaSuccess) e = dalloc(M, &M.wt1, (size_t)H * FI);
    if (e == cudaSuccess) e = dalloc(M, &M.wt2, (size_t)H * H);
    if (e == cudaSuccess) e = dalloc(M, &M.w2, (size_t)H * H);
    if (e == cudaSuccess) e = dalloc(M, &M.wt3, (size_t)H * H);
    if (e == cudaSuccess) e = dalloc(M, &M.w3, (size_t)H * H);
    if (e == cudaSuccess) e = dalloc(M, &M.wt4, (size_t)FO * H);
    if (e == cudaSuccess) e = dalloc(M, &M.w4, (size_t)H * FO);
    if (e == cudaSuccess) e = dalloc(M, &M.norm, WS_NORM);
    if (e == cudaSuccess) e = dalloc(M, &M.loss, 1);
    if (e == cudaSuccess) e = dalloc(M, &M.status, 1);
    if (e == cudaSuccess) e = cudaMemsetAsync(M.adam_m, 0, sizeof(float) * NPAD, M.stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(M.adam_v, 0, sizeof(float) * NPAD, M.stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(M.status, 0, sizeof(unsigned int), M.stream);
    if (e != cudaSuccess) {
        b3g_mlp_destroy(m);
        return ws_fail(B3G_ERR_CUDA, cudaGetErrorString(e));
    }
    // He-style initialisation from the seed; identity normalisation
    std::mt19937_64 rng(seed);
    std::normal_distribution<float> nd(0.f, 1.f);
    std::vector<float> p(WS_PARAMS, 0.f);
    size_t k = 0;
    auto fill = [&](int fan_in, int count) {
        const float s = std::sqrt(2.f / (float)fan_in);
        for (int i = 0; i < count; i++) p[k++] = nd(rng) * s;
    };
    fill(WS_FEATURES, WS_FEATURES * H);
    k += H;
    fill(H, H * H);
    k += H;
    fill(H, H * H);
    k += H;
    fill(H, H * WS_OUTPUTS);
    k += WS_OUTPUTS;
    for (int i = 0; i < WS_NORM; i++) M.norm_host[i] = (i / WS_FEATURES == 1 && i < 2 * WS_FEATURES) ? 1.f : 0.f;
    for (int i = 0; i < WS_OUTPUTS; i++) M.norm_host[2 * WS_FEATURES + WS_OUTPUTS + i] = 1.f;
    std::vector<float> d;
    to_padded(p.data(), d);
    e = cudaMemcpyAsync(M.norm, M.norm_host, sizeof(float) * WS_NORM, cudaMemcpyHostToDevice, M.stream);
    if (e != cudaSuccess) {
        b3g_mlp_destroy(m);
        return ws_fail(B3G_ERR_CUDA, cudaGetErrorString(e));
    }
    b3gStatus st = upload_params(m, d);
    if (st != B3G_OK) {
        b3g_mlp_destroy(m);
        return st;
    }
    *out = m;
    return B3G_OK;
}

extern "C" b3gStatus b3g_mlp_destroy(b3g_mlp m) {
    if (!m) return ws_fail(B3G_ERR_INVALID_ARG, "null model");
    cudaSetDevice(m->m.device);
    if (m->m.stream) cudaStreamSynchronize(m->m.stream);
    for (void* p : m->m.allocations) cudaFree(p);
    if (m->m.stream) cudaStreamDestroy(m->m.stream);
    delete m;
    return B3G_OK;
}

extern "C" b3gStatus b3g_mlp_set_params(b3g_mlp m, const float* params, int n) {
    if (!m || !params || n != WS_PARAMS) return ws_fail(B3G_ERR_INVALID_ARG, "need WS_PARAMS floats");
    std::vector<float> d;
    to_padded(params, d);
    return upload_params(m, d);
}

extern "C" b3gStatus b3g_mlp_get_params(b3g_mlp m, float* params, int n) {
    if (!m || !params || n != WS_PARAMS) return ws_fail(B3G_ERR_INVALID_ARG, "need WS_PARAMS floats");
    std::vector<float> d(NPAD);
    WS_TRY(cudaSetDevice(m->m.device));
    WS_TRY(cudaMemcpyAsync(d.data(), m->m.params, sizeof(float) * NPAD, cudaMemcpyDeviceToHost, m->m.stream));
    WS_TRY(cudaStreamSynchronize(m->m.stream));
    from_padded(d, params);
    return B3G_OK;
}

extern "C" b3gStatus b3g_mlp_set_normalization(b3g_mlp m, const float* norm, int n) {
    if (!m || !norm || n != WS_NORM) return ws_fail(B3G_ERR_INVALID_ARG, "need WS_NORM floats");
    std::memcpy(m->m.norm_host, norm, sizeof(float) * WS_NORM);
    WS_TRY(cudaSetDevice(m->m.device));
    WS_TRY(cudaMemcpyAsync(m->m.norm, m->m.norm_host, sizeof(float) * WS_NORM, cudaMemcpyHostToDevice, m->m.stream));
    WS_TRY(cudaStreamSynchronize(m->m.stream));
    return B3G_OK;
}

extern "C" b3gStatus b3g_mlp_get_normalization(b3g_mlp m, float* norm, int n) {
    if (!m || !norm || n != WS_NORM) return ws_fail(B3G_ERR_INVALID_ARG, "need WS_NORM floats");
    std::memcpy(norm, m->m.norm_host, sizeof(float) * WS_NORM);
    return B3G_OK;
}

namespace {

b3gStatus ensure_train(b3g_mlp m, int batch) {
    Model& M = m->m;
    const int cap = round_up(batch < 64 ? 64 : batch, 64);
    if (M.train.cap >= cap) return B3G_OK;
    M.train = Acts();
    cudaError_t e = alloc_acts(M, M.train, cap, true);
    if (e == cudaSuccess) e = dalloc(M, &M.batch_t, (size_t)cap * WS_OUTPUTS);
    if (e != cudaSuccess) return ws_fail(B3G_ERR_CUDA, cudaGetErrorString(e));
    return B3G_OK;
}

// one forward + backward over rows [0, n) of (x, t) already on the device
void grads_on_device(Model& M, const float* x, const float* t, int n) {
    Acts& a = M.train;
    k_pack<<<M.num_sms * 2, 256, 0, M.stream>>>(x, WS_FEATURES, nullptr, n, n, M.norm, a.x_row, a.x_col, a.cap,
                                                 a.cap);
    run_forward(M, a, nullptr, a.cap, a.cap, true, M.stream);
    run_backward(M, a, n, t, M.stream);
}

}  // namespace

extern "C" b3gStatus b3g_mlp_predict(b3g_mlp m, const float* host_x, int n, float* host_y) {
    if (!m || n < 0 || (n > 0 && (!host_x || !host_y))) return ws_fail(B3G_ERR_INVALID_ARG, "bad arguments");
    if (n == 0) return B3G_OK;
    Model& M = m->m;
    WS_TRY(cudaSetDevice(M.device));
    WS_TRY(ensure_infer(M, n));
    float* dx = nullptr;
    int* drows = nullptr;
    WS_TRY(cudaMalloc(&dx, sizeof(float) * (size_t)n * WS_FEATURES));
    cudaError_t e = cudaMalloc(&drows, sizeof(int));
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dx, host_x, sizeof(float) * (size_t)n * WS_FEATURES, cudaMemcpyHostToDevice, M.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(drows, &n, sizeof(int), cudaMemcpyHostToDevice, M.stream);
    std::vector<float> y((size_t)n * FO);
    if (e == cudaSuccess) {
        forward_device(M, dx, WS_FEATURES, drows, M.infer.cap, M.stream);
        e = cudaMemcpyAsync(y.data(), M.infer.y, sizeof(float) * y.size(), cudaMemcpyDeviceToHost, M.stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(M.stream);
    cudaFree(dx);
    cudaFree(drows);
    if (e != cudaSuccess) return ws_fail(B3G_ERR_CUDA, cudaGetErrorString(e));
    const float* tn = M.norm_host + 2 * WS_FEATURES;
    for (int r = 0; r < n; r++)
        for (int o = 0; o < WS_OUTPUTS; o++) host_y[(size_t)r * WS_OUTPUTS + o] = y[(size_t)r * FO + o] / tn[WS_OUTPUTS + o] + tn[o];
    return B3G_OK;
}

extern "C" b3gStatus b3g_mlp_set_training_data(b3g_mlp m, const float* host_x, const float* host_t, int n) {
    if (!m || n <= 0 || !host_x || !host_t) return ws_fail(B3G_ERR_INVALID_ARG, "bad arguments");
    Model& M = m->m;
    WS_TRY(cudaSetDevice(M.device));
    if (n > M.data_n) {
        cudaError_t e = dalloc(M, &M.data_x, (size_t)n * WS_FEATURES);
        if (e == cudaSuccess) e = dalloc(M, &M.data_t, (size_t)n * WS_OUTPUTS);
        if (e != cudaSuccess) return ws_fail(B3G_ERR_CUDA, cudaGetErrorString(e));
    }
    M.data_n = n;
    WS_TRY(cudaMemcpyAsync(M.data_x, host_x, sizeof(float) * (size_t)n * WS_FEATURES, cudaMemcpyHostToDevice, M.stream));
    WS_TRY(cudaMemcpyAsync(M.data_t, host_t, sizeof(float) * (size_t)n * WS_OUTPUTS, cudaMemcpyHostToDevice, M.stream));
    WS_TRY(cudaStreamSynchronize(M.stream));
    return B3G_OK;
}

extern "C" b3gStatus b3g_mlp_train(b3g_mlp m, int steps, int batch, float lr, int first_batch, double* mean_loss) {
    if (!m || steps <= 0 || batch <= 0) return ws_fail(B3G_ERR_INVALID_ARG, "bad arguments");
    Model& M = m->m;
    if (M.data_n < batch) return ws_fail(B3G_ERR_INVALID_ARG, "training set smaller than one batch");
    WS_TRY(cudaSetDevice(M.device));
    b3gStatus st = ensure_train(m, batch);
    if (st != B3G_OK) return st;
    WS_TRY(cudaMemsetAsync(M.loss, 0, sizeof(double), M.stream));
    const int nb = M.data_n / batch;
    for (int s = 0; s < steps; s++) {
        const long long start = (long long)((first_batch + s) % nb) * batch;
        grads_on_device(M, M.data_x + start * WS_FEATURES, M.data_t + start * WS_OUTPUTS, batch);
        M.adam_step++;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.f / (1.f - std::pow(b1, (float)M.adam_step));
        const float c2 = 1.f / (1.f - std::pow(b2, (float)M.adam_step));
        k_adam<<<M.num_sms, 256, 0, M.stream>>>(M.params, M.adam_m, M.adam_v, M.grads, M.grad_w1t, lr, b1, b2, 1e-8f,
                                                 c1, c2);
        refresh_bf16(M, M.stream);
    }
    double loss = 0.0;
    unsigned int status = 0;
    WS_TRY(cudaMemcpyAsync(&loss, M.loss, sizeof(double), cudaMemcpyDeviceToHost, M.stream));
    WS_TRY(cudaMemcpyAsync(&status, M.status, sizeof(unsigned int), cudaMemcpyDeviceToHost, M.stream));
    WS_TRY(cudaStreamSynchronize(M.stream));
    WS_TRY(cudaGetLastError());
    if (status & B3G_FLAG_MLP_TIMEOUT) return ws_fail(B3G_ERR_BARRIER_TIMEOUT, "tensor-core wait gave up");
    if (mean_loss) *mean_loss = loss / steps;
    return B3G_OK;
}

extern "C" b3gStatus b3g_mlp_gradients(b3g_mlp m, const float* host_x, const float* host_t, int n, float* host_grads,
                                       double* loss_out) {
    if (!m || n <= 0 || !host_x || !host_t || !host_grads) return ws_fail(B3G_ERR_INVALID_ARG, "bad arguments");
    Model& M = m->m;
    WS_TRY(cudaSetDevice(M.device));
    b3gStatus st = ensure_train(m, n);
    if (st != B3G_OK) return st;
    float *dx = nullptr, *dt = nullptr;
    WS_TRY(cudaMalloc(&dx, sizeof(float) * (size_t)n * WS_FEATURES));
    cudaError_t e = cudaMalloc(&dt, sizeof(float) * (size_t)n * WS_OUTPUTS);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dx, host_x, sizeof(float) * (size_t)n * WS_FEATURES, cudaMemcpyHostToDevice, M.stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dt, host_t, sizeof(float) * (size_t)n * WS_OUTPUTS, cudaMemcpyHostToDevice, M.stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(M.loss, 0, sizeof(double), M.stream);
    std::vector<float> g(NPAD), gw1t((size_t)H * FI);
    double loss = 0.0;
    unsigned int status = 0;
    if (e == cudaSuccess) {
        grads_on_device(M, dx, dt, n);
        e = cudaMemcpyAsync(g.data(), M.grads, sizeof(float) * NPAD, cudaMemcpyDeviceToHost, M.stream);
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(gw1t.data(), M.grad_w1t, sizeof(float) * gw1t.size(), cudaMemcpyDeviceToHost, M.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&loss, M.loss, sizeof(double), cudaMemcpyDeviceToHost, M.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&status, M.status, sizeof(unsigned int), cudaMemcpyDeviceToHost, M.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(M.stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    cudaFree(dx);
    cudaFree(dt);
    if (e != cudaSuccess) return ws_fail(B3G_ERR_CUDA, cudaGetErrorString(e));
    if (status & B3G_FLAG_MLP_TIMEOUT) return ws_fail(B3G_ERR_BARRIER_TIMEOUT, "tensor-core wait gave up");
    for (int i = 0; i < WS_FEATURES; i++)
        for (int o = 0; o < H; o++) g[OFF_W1 + i * H + o] = gw1t[(size_t)o * FI + i];
    from_padded(g, host_grads);
    if (loss_out) *loss_out = loss;
    return B3G_OK;
}

b3g::mlp::Model* b3g_mlp_model(b3g_mlp m) { return m ? &m->m : nullptr; }
