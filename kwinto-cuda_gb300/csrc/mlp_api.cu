// mlp_api.cu -- the learned surrogate: an MLP 5 -> 128 -> 128 -> 128 -> 128 -> 1
// (SiLU, BF16 weights, FP32 accumulation on the tcgen05 tensor cores) that maps
// normalised option parameters (log K/S, vol sqrt T, r T, q T, put/call) to the
// early-exercise premium  (American price - European price) / K,  trained on prices
// the GPU FD solver generates.  Price = Black-Scholes European + K * premium.
//
// No counterpart in the reference (it has no learned component); the FD solver that
// generates its labels, and that it falls back to, is the reference's FD1D path.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "kwg.h"
#include "kwg_ctx.h"
#include "mlp.h"

using kwg::kMlpIn;
using kwg::kMlpLayers;
using kwg::kMlpParams;
using kwg::kMlpWeights;
using kwg::kMlpWidth;

struct kwg_mlp {
    int device = 0;
    int sms = 1;
    cudaStream_t stream = nullptr;
    std::string err;
    kwg::MlpBox box;
    float y_scale = 1.f;
    // parameters (FP32 master), gradients, Adam moments; BF16 forward weights
    // (K-doubled, mlp.h) and W^T for the backward
    float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
    __nv_bfloat16 *wb = nullptr, *wt = nullptr;
    long long adam_t = 0;
    // batch workspace (capacity `cap` rows)
    int cap = 0;
    __nv_bfloat16 *x = nullptr, *xt = nullptr;             // split input rows [64] / transposed hi
    __nv_bfloat16 *act[3] = {}, *actt[4] = {};              // split activations [256] / transposed hi
    float* dact[4] = {};                                      // SiLU'(z)
    float *y = nullptr, *tb = nullptr, *fb = nullptr, *da = nullptr;
    float* feat = nullptr;                                    // features [cap][5]
    double* base = nullptr;                                   // analytic base prices [cap]
    __nv_bfloat16 *dy = nullptr, *dyt = nullptr, *dz = nullptr, *dzt = nullptr;
    double* loss = nullptr;
    int* error = nullptr;
    // the last training run: mean loss of every epoch, the epoch whose parameters
    // were kept, and how many loss spikes sent it back to them
    std::vector<double> loss_hist;
    int best_epoch = -1, restarts = 0;
    // surrogate pricing arena (grow-only), carved by route_layout()
    char* d_arena = nullptr;
    size_t arena_bytes = 0;
    char* h_arena = nullptr;  // pinned: counters and audit statistics
};

namespace {

int mlp_err(kwg_mlp* h, int code, const std::string& msg)
{
    if (h) h->err = msg;
    return code;
}

#define MLP_CUDA(h, call)                                                               \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) return mlp_err(h, KWG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

void free_ws(kwg_mlp* h)
{
    void* bufs[] = {h->x, h->xt, h->y, h->tb, h->fb, h->da, h->dy, h->dyt, h->dz, h->dzt, h->feat, h->base};
    for (void* b : bufs)
        if (b) cudaFree(b);
    for (int l = 0; l < 4; ++l) {
        if (l < 3 && h->act[l]) cudaFree(h->act[l]);
        if (h->actt[l]) cudaFree(h->actt[l]);
        if (h->dact[l]) cudaFree(h->dact[l]);
        if (l < 3) h->act[l] = nullptr;
        h->actt[l] = nullptr;
        h->dact[l] = nullptr;
    }
    h->x = h->xt = h->dy = h->dyt = h->dz = h->dzt = nullptr;
    h->y = h->tb = h->fb = h->da = h->feat = nullptr;
    h->base = nullptr;
    h->cap = 0;
}

// Workspace for batches of up to `rows` rows (a multiple of 64).
int ensure_ws(kwg_mlp* h, int rows)
{
    if (rows <= h->cap) return KWG_OK;
    free_ws(h);
    const size_t r = (size_t)rows, w = kMlpWidth;
    MLP_CUDA(h, cudaMalloc(&h->x, r * kwg::kMlpInK * 2));
    MLP_CUDA(h, cudaMalloc(&h->xt, r * kwg::kMlpInK * 2));
    for (int l = 0; l < 4; ++l) {
        if (l < 3) MLP_CUDA(h, cudaMalloc(&h->act[l], r * kwg::kMlpHidK * 2));
        MLP_CUDA(h, cudaMalloc(&h->actt[l], r * w * 2));
        MLP_CUDA(h, cudaMalloc(&h->dact[l], r * w * 4));
    }
    MLP_CUDA(h, cudaMalloc(&h->y, r * 4));
    MLP_CUDA(h, cudaMalloc(&h->feat, r * kMlpIn * 4));
    MLP_CUDA(h, cudaMalloc(&h->base, r * 8));
    MLP_CUDA(h, cudaMalloc(&h->tb, r * 4));
    MLP_CUDA(h, cudaMalloc(&h->fb, r * 4));
    MLP_CUDA(h, cudaMalloc(&h->da, r * w * 4));
    MLP_CUDA(h, cudaMalloc(&h->dy, r * w * 2));
    MLP_CUDA(h, cudaMalloc(&h->dyt, r * w * 2));
    MLP_CUDA(h, cudaMalloc(&h->dz, r * w * 2));
    MLP_CUDA(h, cudaMalloc(&h->dzt, r * w * 2));
    // dY has one nonzero column (dY^T one nonzero row): the rest stays zero
    MLP_CUDA(h, cudaMemset(h->dy, 0, r * w * 2));
    MLP_CUDA(h, cudaMemset(h->dyt, 0, r * w * 2));
    h->cap = rows;
    return KWG_OK;
}

kwg::GemmArgs gemm_args(const __nv_bfloat16* a, const __nv_bfloat16* b, int m, int n, int k, int* error)
{
    kwg::GemmArgs g = {};
    g.A = a;
    g.B = b;
    g.M = m;
    g.N = n;
    g.K = k;
    g.lda = k;
    g.ldb = k;
    g.k_per_split = k;
    g.ldo = n;
    g.ldt = m;
    g.ldb16 = n;
    g.error = error;
    return g;
}

float* bias_of(float* p, int layer) { return p + kMlpWeights + layer * kMlpWidth; }
const __nv_bfloat16* wt_of(const __nv_bfloat16* w, int layer) { return w + (size_t)layer * kMlpWidth * kMlpWidth; }
const __nv_bfloat16* wb_of(const __nv_bfloat16* w, int layer) { return w + (size_t)layer * kwg::kMlpFwdSlot; }

// Forward over rows [0, rows) of h->x.  train: keep transposed hi activations and
// SiLU' for the backward pass.  Output (the scaled premium) in h->y.
int forward(kwg_mlp* h, int rows, bool train)
{
    const __nv_bfloat16* in = h->x;
    for (int l = 0; l < 4; ++l) {
        const int k = l == 0 ? kwg::kMlpInK : kwg::kMlpHidK;
        kwg::GemmArgs g = gemm_args(in, wb_of(h->wb, l), rows, kMlpWidth, k, h->error);
        g.bias = bias_of(h->p, l);
        g.silu = true;
        if (l < 3) {
            g.out_bf16 = h->act[l];
            g.ldb16 = kwg::kMlpHidK;
            g.split_bf16 = true;
        } else {
            g.head_w = wb_of(h->wb, 4);
            g.head_bias = bias_of(h->p, 4);
            g.out_head = h->y;
        }
        if (train) {
            g.out_bf16_t = h->actt[l];
            g.out_dact = h->dact[l];
        }
        MLP_CUDA(h, kwg::gemm_launch(g, 1, h->stream));
        if (l < 3) in = h->act[l];
    }
    return KWG_OK;
}

// Backward of the MSE loss over rows [0, b) (b_pad rows in the buffers); gradients
// accumulate into h->g (zeroed here), the loss into *h->loss.
int backward(kwg_mlp* h, int b, int b_pad)
{
    MLP_CUDA(h, cudaMemsetAsync(h->g, 0, sizeof(float) * kMlpParams, h->stream));
    // dY^T is [128][b_pad]: only row 0 is written, so clear the rest for this b_pad
    MLP_CUDA(h, cudaMemsetAsync(h->dyt, 0, (size_t)kMlpWidth * b_pad * 2, h->stream));
    kwg::mlp_launch_out_grad(h->y, h->tb, h->fb, b, b_pad, h->dy, h->dyt, bias_of(h->g, 4), h->loss, h->stream);
    const int split = 256;
    // dW[out][in] += dZ^T A over the batch (A: transposed hi activations, `ins` rows)
    auto dw = [&](const __nv_bfloat16* dzt, const __nv_bfloat16* xt, int layer, int ins) -> int {
        kwg::GemmArgs g = gemm_args(dzt, xt, kMlpWidth, ins, b_pad, h->error);
        g.ldo = kMlpWidth;
        g.atomic_f32 = true;
        g.out_f32 = h->g + (size_t)layer * kMlpWidth * kMlpWidth;
        g.k_per_split = split;
        MLP_CUDA(h, kwg::gemm_launch(g, (b_pad + split - 1) / split, h->stream));
        return KWG_OK;
    };
    auto dx = [&](const __nv_bfloat16* dzr, int layer) -> int {
        kwg::GemmArgs g = gemm_args(dzr, wt_of(h->wt, layer), b_pad, kMlpWidth, kMlpWidth, h->error);
        g.out_f32 = h->da;
        MLP_CUDA(h, kwg::gemm_launch(g, 1, h->stream));
        return KWG_OK;
    };
    // output layer: dW5 = dY^T act4, dA4 = dY W5
    if (int rc = dw(h->dyt, h->actt[3], 4, kMlpWidth)) return rc;
    if (int rc = dx(h->dy, 4)) return rc;
    for (int l = 3; l >= 0; --l) {
        kwg::mlp_launch_dz(h->da, h->dact[l], b, b_pad, h->dz, h->dzt, bias_of(h->g, l), h->stream);
        if (int rc = l == 0 ? dw(h->dzt, h->xt, 0, kwg::kMlpInK) : dw(h->dzt, h->actt[l - 1], l, kMlpWidth))
            return rc;
        if (l > 0)
            if (int rc = dx(h->dz, l)) return rc;
    }
    return KWG_OK;
}

int check_error(kwg_mlp* h)
{
    int e = 0;
    MLP_CUDA(h, cudaMemcpyAsync(&e, h->error, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    MLP_CUDA(h, cudaStreamSynchronize(h->stream));
    if (e) return mlp_err(h, KWG_ERR_CUDA, "kwg_mlp: a tensor-core wait timed out");
    return KWG_OK;
}

// Training targets of row i: premium t = (price - base) / K over the analytic base
// price and, in the early-exercise region (price within 1e-6 K of a positive
// intrinsic value, or below it), the floor f = (intrinsic - base) / K; elsewhere
// f = -kNoFloor.
__global__ void premium_targets(const kwg_option* __restrict__ o, const double* __restrict__ price,
                                const double* __restrict__ base, int n, float* __restrict__ prem,
                                float* __restrict__ floor_)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double k = o[i].k, intr = fmax(0., o[i].w < 0 ? k - o[i].s : o[i].s - k);
    prem[i] = (float)((price[i] - base[i]) / k);
    const bool exercise = intr > 0. && price[i] - intr <= 1e-6 * k;
    floor_[i] = exercise ? (float)((intr - base[i]) / k) : -kwg::kNoFloor;
}

__global__ void scale_targets(float* t, float* f, int n, float s)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    t[i] *= s;
    if (f[i] > -kwg::kNoFloor) f[i] *= s;
}

// ---- surrogate routing on the device
// Route of option i: 2 outside the training box, else 1 for a seeded audit sample
// (splitmix64 of seed + (i + 1) * golden ratio below audit_frac * 2^64), else 0.
__device__ __forceinline__ int32_t route_of(uint8_t inside, uint64_t seed, uint64_t i, double thresh)
{
    if (!inside) return 2;
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (i + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)z < thresh ? 1 : 0;
}

// Routes every option and gathers the FD ones (route > 0) into sub/sub_idx at
// slots taken with warp-aggregated atomics; cnt[0] = FD options, cnt[1] audited,
// cnt[2] out of the box.
__global__ void route_gather(const kwg_option* __restrict__ opts, const uint8_t* __restrict__ inside, int n,
                             uint64_t seed, double thresh, int32_t* __restrict__ route, kwg_option* __restrict__ sub,
                             int32_t* __restrict__ sub_idx, int* __restrict__ cnt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int32_t r = i < n ? route_of(inside[i], seed, (uint64_t)i, thresh) : 0;
    if (i < n) route[i] = r;
    // every lane of the warp reaches the ballots (lanes past n carry route 0)
    const unsigned fd = __ballot_sync(0xffffffffu, r > 0);
    const unsigned aud = __ballot_sync(0xffffffffu, r == 1);
    const unsigned oob = __ballot_sync(0xffffffffu, r == 2);
    const int lane = threadIdx.x & 31, leader = fd ? __ffs(fd) - 1 : 0;
    int base = 0;
    if (fd && lane == leader) base = atomicAdd(&cnt[0], __popc(fd));
    if (lane == 0) {
        if (aud) atomicAdd(&cnt[1], __popc(aud));
        if (oob) atomicAdd(&cnt[2], __popc(oob));
    }
    base = __shfl_sync(0xffffffffu, base, leader);
    if (r > 0) {
        const int slot = base + __popc(fd & ((1u << lane) - 1u));
        sub[slot] = opts[i];
        sub_idx[slot] = i;
    }
}

// FD prices back into the output; audit statistics (sum and max of |network - FD|
// over audited options; the max as the ordered bits of a non-negative double);
// options whose FD solve failed get route 3.
__global__ void route_scatter(int m, const int32_t* __restrict__ sub_idx, const double* __restrict__ fdp,
                              const int32_t* __restrict__ fst, int32_t* __restrict__ route,
                              double* __restrict__ prices, double* __restrict__ stats)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    const int i = sub_idx[j];
    if (route[i] == 1) {
        const double e = fabs(prices[i] - fdp[j]);
        atomicAdd(&stats[0], e);
        atomicMax(reinterpret_cast<unsigned long long*>(&stats[1]), (unsigned long long)__double_as_longlong(e));
    }
    prices[i] = fdp[j];
    if (fst[j] != KWG_STATUS_OK) route[i] = 3;
}

}  // namespace

extern "C" {

int kwg_gemm_bf16(const void* d_a, const void* d_b, float* d_c, int m, int n, int k, void* stream)
{
    if (!d_a || !d_b || !d_c || m <= 0 || n <= 0 || k <= 0 || k % 64 != 0) return KWG_ERR_INVALID;
    kwg::GemmArgs g = gemm_args(static_cast<const __nv_bfloat16*>(d_a), static_cast<const __nv_bfloat16*>(d_b), m, n,
                                k, nullptr);
    g.out_f32 = d_c;
    return kwg::gemm_launch(g, 1, (cudaStream_t)stream) == cudaSuccess ? KWG_OK : KWG_ERR_CUDA;
}

kwg_mlp* kwg_mlp_create(int device, uint64_t seed)
{
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) return nullptr;
    if (cudaSetDevice(device) != cudaSuccess) return nullptr;
    kwg_mlp* h = new kwg_mlp();
    h->device = device;
    bool ok = cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, device) == cudaSuccess;
    ok = ok && cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) == cudaSuccess;
    ok = ok && cudaMalloc(&h->p, sizeof(float) * kMlpParams) == cudaSuccess;
    ok = ok && cudaMalloc(&h->g, sizeof(float) * kMlpParams) == cudaSuccess;
    ok = ok && cudaMalloc(&h->m, sizeof(float) * kMlpParams) == cudaSuccess;
    ok = ok && cudaMalloc(&h->v, sizeof(float) * kMlpParams) == cudaSuccess;
    ok = ok && cudaMalloc(&h->wb, sizeof(__nv_bfloat16) * kwg::kMlpFwdWeights) == cudaSuccess;
    ok = ok && cudaMalloc(&h->wt, sizeof(__nv_bfloat16) * kMlpWeights) == cudaSuccess;
    ok = ok && cudaMalloc(&h->loss, sizeof(double)) == cudaSuccess;
    ok = ok && cudaMalloc(&h->error, sizeof(int)) == cudaSuccess;
    if (!ok) {
        kwg_mlp_destroy(h);
        return nullptr;
    }
    // training box of the 32768-option workload's distributions, with a margin:
    // K/S in [0.8, 1.2], vol sqrt T in [0.05, 0.85], r T and q T in [0, 0.2]
    const double lo[kMlpIn] = {-0.25, 0.04, 0.0, 0.0, -1.0}, hi[kMlpIn] = {0.20, 0.86, 0.2, 0.2, 1.0};
    std::memcpy(h->box.lo, lo, sizeof lo);
    std::memcpy(h->box.hi, hi, sizeof hi);
    // He-uniform weights on the active entries; padded rows/columns stay zero
    std::vector<float> p(kMlpParams, 0.f);
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<float> u(-1.f, 1.f);
    for (int l = 0; l < kMlpLayers; ++l) {
        const int fan_in = l == 0 ? kMlpIn : kMlpWidth;
        const int outs = l == kMlpLayers - 1 ? 1 : kMlpWidth;
        const float a = std::sqrt(6.f / fan_in);
        for (int o = 0; o < outs; ++o)
            for (int i = 0; i < fan_in; ++i) p[(size_t)l * kMlpWidth * kMlpWidth + o * kMlpWidth + i] = a * u(rng);
    }
    if (kwg_mlp_set_params(h, p.data(), nullptr, nullptr, 1.f) != KWG_OK) {
        kwg_mlp_destroy(h);
        return nullptr;
    }
    return h;
}

void kwg_mlp_destroy(kwg_mlp* h)
{
    if (!h) return;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_ws(h);
    void* bufs[] = {h->p, h->g, h->m, h->v, h->wb, h->wt, h->loss, h->error, h->d_arena};
    for (void* b : bufs)
        if (b) cudaFree(b);
    if (h->h_arena) cudaFreeHost(h->h_arena);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

const char* kwg_mlp_last_error(const kwg_mlp* h) { return h ? h->err.c_str() : "kwg_mlp: null handle"; }

int kwg_mlp_set_params(kwg_mlp* h, const float* params, const double* box_lo, const double* box_hi, float y_scale)
{
    if (!h || !params || !(y_scale > 0.f)) return KWG_ERR_INVALID;
    h->err.clear();
    MLP_CUDA(h, cudaSetDevice(h->device));
    if (box_lo && box_hi) {
        std::memcpy(h->box.lo, box_lo, sizeof h->box.lo);
        std::memcpy(h->box.hi, box_hi, sizeof h->box.hi);
    }
    h->y_scale = y_scale;
    MLP_CUDA(h, cudaMemcpyAsync(h->p, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, h->stream));
    MLP_CUDA(h, cudaMemsetAsync(h->m, 0, sizeof(float) * kMlpParams, h->stream));
    MLP_CUDA(h, cudaMemsetAsync(h->v, 0, sizeof(float) * kMlpParams, h->stream));
    MLP_CUDA(h, cudaMemsetAsync(h->error, 0, sizeof(int), h->stream));
    h->adam_t = 0;
    kwg::mlp_launch_refresh(h->p, h->wb, h->wt, h->stream);
    MLP_CUDA(h, cudaStreamSynchronize(h->stream));
    return KWG_OK;
}

int kwg_mlp_get_params(kwg_mlp* h, float* params, double* box_lo, double* box_hi, float* y_scale)
{
    if (!h) return KWG_ERR_INVALID;
    h->err.clear();
    if (params) {
        MLP_CUDA(h, cudaMemcpyAsync(params, h->p, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, h->stream));
        MLP_CUDA(h, cudaStreamSynchronize(h->stream));
    }
    if (box_lo) std::memcpy(box_lo, h->box.lo, sizeof h->box.lo);
    if (box_hi) std::memcpy(box_hi, h->box.hi, sizeof h->box.hi);
    if (y_scale) *y_scale = h->y_scale;
    return KWG_OK;
}

int kwg_mlp_forward(kwg_mlp* h, const float* d_x, int n, float* d_y)
{
    if (!h || !d_x || !d_y || n <= 0) return KWG_ERR_INVALID;
    h->err.clear();
    MLP_CUDA(h, cudaSetDevice(h->device));
    const int rows = (n + 63) / 64 * 64;
    if (int rc = ensure_ws(h, rows)) return rc;
    kwg::mlp_launch_pack(d_x, nullptr, nullptr, nullptr, n, rows, h->x, nullptr, nullptr, nullptr, h->stream);
    if (int rc = forward(h, rows, false)) return rc;
    MLP_CUDA(h, cudaMemcpyAsync(d_y, h->y, (size_t)n * 4, cudaMemcpyDeviceToDevice, h->stream));
    return check_error(h);
}

int kwg_mlp_gradients(kwg_mlp* h, const float* d_x, const float* d_t, const float* d_floor, int n, float* d_grad,
                      double* loss)
{
    if (!h || !d_x || !d_t || !d_grad || n <= 0) return KWG_ERR_INVALID;
    h->err.clear();
    MLP_CUDA(h, cudaSetDevice(h->device));
    const int rows = (n + 63) / 64 * 64;
    if (int rc = ensure_ws(h, rows)) return rc;
    kwg::mlp_launch_pack(d_x, d_t, d_floor, nullptr, n, rows, h->x, h->xt, h->tb, h->fb, h->stream);
    MLP_CUDA(h, cudaMemsetAsync(h->loss, 0, sizeof(double), h->stream));
    if (int rc = forward(h, rows, true)) return rc;
    if (int rc = backward(h, n, rows)) return rc;
    MLP_CUDA(h, cudaMemcpyAsync(d_grad, h->g, sizeof(float) * kMlpParams, cudaMemcpyDeviceToDevice, h->stream));
    if (loss) MLP_CUDA(h, cudaMemcpyAsync(loss, h->loss, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    return check_error(h);
}

int kwg_mlp_featurize(kwg_mlp* h, const kwg_option* d_opts, int n, float* d_x, uint8_t* d_inside, double* d_base)
{
    if (!h || !d_opts || n <= 0) return KWG_ERR_INVALID;
    h->err.clear();
    MLP_CUDA(h, cudaSetDevice(h->device));
    kwg::mlp_launch_featurize(d_opts, n, h->box, d_x, d_inside, d_base, h->stream);
    MLP_CUDA(h, cudaStreamSynchronize(h->stream));
    return KWG_OK;
}

int kwg_mlp_train(kwg_mlp* h, const kwg_option* d_opts, const double* d_prices, int n, int epochs, int batch,
                  float lr, uint64_t seed, double* final_loss)
{
    if (!h || !d_opts || !d_prices || n <= 0 || epochs <= 0 || batch <= 0 || !(lr > 0.f)) return KWG_ERR_INVALID;
    h->err.clear();
    MLP_CUDA(h, cudaSetDevice(h->device));
    const int b_pad = (std::min(batch, n) + 63) / 64 * 64;
    if (int rc = ensure_ws(h, b_pad)) return rc;
    // features, premium targets and exercise-region floors of the whole training set
    float *X = nullptr, *T = nullptr, *F = nullptr, *pbest = nullptr;
    double* base = nullptr;
    int32_t* idx = nullptr;
    auto cleanup = [&]() {
        cudaFree(X);
        cudaFree(T);
        cudaFree(F);
        cudaFree(pbest);
        cudaFree(base);
        cudaFree(idx);
    };
    if (cudaMalloc(&X, (size_t)n * kMlpIn * 4) != cudaSuccess || cudaMalloc(&T, (size_t)n * 4) != cudaSuccess ||
        cudaMalloc(&F, (size_t)n * 4) != cudaSuccess || cudaMalloc(&base, (size_t)n * 8) != cudaSuccess ||
        cudaMalloc(&idx, (size_t)n * 4) != cudaSuccess || cudaMalloc(&pbest, sizeof(float) * kMlpParams) != cudaSuccess) {
        cleanup();
        return mlp_err(h, KWG_ERR_CUDA, "kwg_mlp_train: out of device memory");
    }
    kwg::mlp_launch_featurize(d_opts, n, h->box, X, nullptr, base, h->stream);
    premium_targets<<<(n + 255) / 256, 256, 0, h->stream>>>(d_opts, d_prices, base, n, T, F);
    std::vector<float> prem(n);
    if (cudaMemcpyAsync(prem.data(), T, (size_t)n * 4, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
        cudaStreamSynchronize(h->stream) != cudaSuccess) {
        cleanup();
        return mlp_err(h, KWG_ERR_CUDA, "kwg_mlp_train: target copy failed");
    }
    double s1 = 0., s2 = 0.;
    for (float x : prem) {
        s1 += x;
        s2 += (double)x * x;
    }
    const double sd = std::sqrt(std::max(1e-30, s2 / n - (s1 / n) * (s1 / n)));
    h->y_scale = (float)(1. / sd);
    scale_targets<<<(n + 255) / 256, 256, 0, h->stream>>>(T, F, n, h->y_scale);

    std::vector<int32_t> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::mt19937_64 rng(seed);
    const int steps_per_epoch = (n + batch - 1) / batch;
    const long long total = (long long)steps_per_epoch * epochs;
    long long step = 0;
    // the parameters of the epoch with the lowest mean loss are kept (before the first
    // finite epoch: the initial ones); an epoch whose loss is not finite or above
    // kSpike x that best goes back to them with fresh Adam moments and half the
    // learning rate for the rest of the run
    constexpr double kSpike = 3.;
    double best = HUGE_VAL;
    float lr_scale = 1.f;
    h->loss_hist.clear();
    h->best_epoch = -1;
    h->restarts = 0;
    if (cudaMemcpyAsync(pbest, h->p, sizeof(float) * kMlpParams, cudaMemcpyDeviceToDevice, h->stream) !=
        cudaSuccess) {
        cleanup();
        return mlp_err(h, KWG_ERR_CUDA, "kwg_mlp_train: parameter snapshot failed");
    }
    for (int ep = 0; ep < epochs; ++ep) {
        std::shuffle(order.begin(), order.end(), rng);
        if (cudaMemcpyAsync(idx, order.data(), (size_t)n * 4, cudaMemcpyHostToDevice, h->stream) != cudaSuccess ||
            cudaMemsetAsync(h->loss, 0, sizeof(double), h->stream) != cudaSuccess) {
            cleanup();
            return mlp_err(h, KWG_ERR_CUDA, "kwg_mlp_train: index upload failed");
        }
        for (int s = 0; s < steps_per_epoch; ++s, ++step) {
            const int b = std::min(batch, n - s * batch);
            const int bp = (b + 63) / 64 * 64;
            kwg::mlp_launch_pack(X, T, F, idx + (size_t)s * batch, b, bp, h->x, h->xt, h->tb, h->fb, h->stream);
            int rc = forward(h, bp, true);
            if (!rc) rc = backward(h, b, bp);
            if (rc) {
                cleanup();
                return rc;
            }
            // Adam with a cosine-decayed learning rate (to 1% of lr)
            ++h->adam_t;
            const double frac = (double)step / std::max(1LL, total - 1);
            const float lr_t = lr_scale * (float)(lr * (0.01 + 0.99 * 0.5 * (1. + std::cos(M_PI * frac))));
            const float b1 = 0.9f, b2 = 0.999f;
            kwg::mlp_launch_adam(h->p, h->g, h->m, h->v, kMlpParams, lr_t, b1, b2, 1e-8f,
                                 1.f - std::pow(b1, (float)h->adam_t), 1.f - std::pow(b2, (float)h->adam_t),
                                 h->stream);
            kwg::mlp_launch_refresh(h->p, h->wb, h->wt, h->stream);
        }
        // mean of the epoch's minibatch losses
        double l = 0.;
        if (cudaMemcpyAsync(&l, h->loss, sizeof(double), cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
            cudaStreamSynchronize(h->stream) != cudaSuccess) {
            cleanup();
            return mlp_err(h, KWG_ERR_CUDA, "kwg_mlp_train: loss copy failed");
        }
        const double mean = l / steps_per_epoch;
        h->loss_hist.push_back(mean);
        cudaError_t e = cudaSuccess;
        if (std::isfinite(mean) && mean < best) {
            best = mean;
            h->best_epoch = ep;
            e = cudaMemcpyAsync(pbest, h->p, sizeof(float) * kMlpParams, cudaMemcpyDeviceToDevice, h->stream);
        } else if (!std::isfinite(mean) || !(mean <= kSpike * best)) {
            ++h->restarts;
            lr_scale *= 0.5f;
            h->adam_t = 0;
            e = cudaMemcpyAsync(h->p, pbest, sizeof(float) * kMlpParams, cudaMemcpyDeviceToDevice, h->stream);
            if (e == cudaSuccess) e = cudaMemsetAsync(h->m, 0, sizeof(float) * kMlpParams, h->stream);
            if (e == cudaSuccess) e = cudaMemsetAsync(h->v, 0, sizeof(float) * kMlpParams, h->stream);
            if (e == cudaSuccess) kwg::mlp_launch_refresh(h->p, h->wb, h->wt, h->stream);
        }
        if (e != cudaSuccess) {
            cleanup();
            return mlp_err(h, KWG_ERR_CUDA, std::string("kwg_mlp_train: parameter snapshot: ") + cudaGetErrorString(e));
        }
    }
    if (h->best_epoch != epochs - 1) {
        // the last epoch was not the best: its parameters give way to the best epoch's
        // (or to the initial ones when no epoch had a finite loss)
        if (cudaMemcpyAsync(h->p, pbest, sizeof(float) * kMlpParams, cudaMemcpyDeviceToDevice, h->stream) !=
            cudaSuccess) {
            cleanup();
            return mlp_err(h, KWG_ERR_CUDA, "kwg_mlp_train: parameter restore failed");
        }
        kwg::mlp_launch_refresh(h->p, h->wb, h->wt, h->stream);
    }
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) {
        cleanup();
        return mlp_err(h, KWG_ERR_CUDA, "kwg_mlp_train: final synchronisation failed");
    }
    const int rc = check_error(h);
    cleanup();
    if (final_loss) *final_loss = h->best_epoch >= 0 ? best : h->loss_hist.back();
    return rc;
}

int kwg_mlp_train_history(kwg_mlp* h, double* losses, int cap, int* best_epoch, int* restarts)
{
    if (!h || cap < 0 || (cap > 0 && !losses)) return -1;
    const int n = (int)h->loss_hist.size();
    for (int i = 0; i < std::min(n, cap); ++i) losses[i] = h->loss_hist[i];
    if (best_epoch) *best_epoch = h->best_epoch;
    if (restarts) *restarts = h->restarts;
    return n;
}

int kwg_mlp_price_device(kwg_mlp* h, const kwg_option* d_opts, int n, double* d_prices, uint8_t* d_inside)
{
    if (!h || !d_opts || !d_prices || n <= 0) return KWG_ERR_INVALID;
    h->err.clear();
    MLP_CUDA(h, cudaSetDevice(h->device));
    MLP_CUDA(h, kwg::mlp_launch_price_fused(d_opts, n, h->box, h->wb, h->p, h->y_scale, d_prices, d_inside, h->error,
                                            h->sms, h->stream));
    return check_error(h);
}

// Surrogate pricing with FD fallback and audit (host arrays in and out).  On the
// device: network prices (fused kernel), routing and gathering of the FD options,
// the FD solve (kwg_fd1d_price_device on the same stream), scatter and audit
// statistics; the host copies options in, reads the FD count once, and copies
// prices, routes and statistics out.
int kwg_surrogate_price(kwg_ctx* ctx, kwg_mlp* h, const kwg_option* opts, size_t n, const kwg_fd1d_params* fd,
                        double audit_frac, uint64_t seed, double* prices, int32_t* route, kwg_audit* audit)
{
    if (!ctx || !h || !opts || !prices || !fd || n == 0 || n > (size_t)INT32_MAX / 2 || !(audit_frac >= 0.) ||
        !(audit_frac <= 1.))
        return KWG_ERR_INVALID;
    h->err.clear();
    MLP_CUDA(h, cudaSetDevice(h->device));
    // arena: opts | prices | inside | route | sub | sub_idx | sub prices | sub status | counters | stats
    auto al = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t o_opts = 0, o_prices = o_opts + al(n * sizeof(kwg_option)), o_inside = o_prices + al(n * 8),
                 o_route = o_inside + al(n), o_sub = o_route + al(n * 4), o_subidx = o_sub + al(n * sizeof(kwg_option)),
                 o_subp = o_subidx + al(n * 4), o_subs = o_subp + al(n * 8), o_cnt = o_subs + al(n * 4),
                 o_stats = o_cnt + 256, total = o_stats + 256;
    if (total > h->arena_bytes) {
        if (h->d_arena) cudaFree(h->d_arena);
        h->d_arena = nullptr;
        h->arena_bytes = 0;
        MLP_CUDA(h, cudaMalloc(&h->d_arena, total));
        h->arena_bytes = total;
    }
    if (!h->h_arena) MLP_CUDA(h, cudaMallocHost(&h->h_arena, 512));
    char* A = h->d_arena;
    kwg_option* d_opts = (kwg_option*)(A + o_opts);
    double* d_prices = (double*)(A + o_prices);
    uint8_t* d_inside = (uint8_t*)(A + o_inside);
    int32_t* d_route = (int32_t*)(A + o_route);
    kwg_option* d_sub = (kwg_option*)(A + o_sub);
    int32_t* d_subidx = (int32_t*)(A + o_subidx);
    double* d_subp = (double*)(A + o_subp);
    int32_t* d_subs = (int32_t*)(A + o_subs);
    int* d_cnt = (int*)(A + o_cnt);
    double* d_stats = (double*)(A + o_stats);
    MLP_CUDA(h, cudaMemcpyAsync(d_opts, opts, n * sizeof(kwg_option), cudaMemcpyHostToDevice, h->stream));
    MLP_CUDA(h, cudaMemsetAsync(d_cnt, 0, 512, h->stream));  // counters and statistics
    MLP_CUDA(h, kwg::mlp_launch_price_fused(d_opts, (int)n, h->box, h->wb, h->p, h->y_scale, d_prices, d_inside,
                                            h->error, h->sms, h->stream));
    const double thresh = audit_frac * 18446744073709551616.0;
    route_gather<<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(d_opts, d_inside, (int)n, seed, thresh, d_route,
                                                                     d_sub, d_subidx, d_cnt);
    int* hc = (int*)h->h_arena;
    MLP_CUDA(h, cudaMemcpyAsync(hc, d_cnt, 3 * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    MLP_CUDA(h, cudaStreamSynchronize(h->stream));
    const int m = hc[0];
    kwg_audit a = {};
    a.audited = hc[1];
    a.out_of_box = hc[2];
    if (m > 0) {
        kwg_fd1d_params q = *fd;
        q.strict = 0;
        if (int rc = kwg_fd1d_price_device(ctx, d_sub, (size_t)m, &q, d_subp, d_subs, h->stream)) {
            h->err = std::string("kwg_surrogate_price: FD fallback: ") + kwg_last_error(ctx);
            return rc;
        }
        route_scatter<<<(unsigned)((m + 255) / 256), 256, 0, h->stream>>>(m, d_subidx, d_subp, d_subs, d_route,
                                                                          d_prices, d_stats);
    }
    MLP_CUDA(h, cudaMemcpyAsync(prices, d_prices, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (route) MLP_CUDA(h, cudaMemcpyAsync(route, d_route, n * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    double* hs = (double*)(h->h_arena + 256);
    MLP_CUDA(h, cudaMemcpyAsync(hs, d_stats, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (int rc = check_error(h)) return rc;  // synchronises the stream
    a.audit_abs_sum = hs[0];
    a.audit_abs_max = hs[1];
    if (audit) *audit = a;
    return KWG_OK;
}

}  // extern "C"
