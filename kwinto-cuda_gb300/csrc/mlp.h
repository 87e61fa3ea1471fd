// mlp.h -- internal interface of the MLP surrogate kernels (tensor-core GEMM,
// elementwise passes, optimiser).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "kwg.h"

namespace kwg {

// Arguments of gemm_bf16_tn: acc = A[M][K] * B[N][K]^T, then the epilogue selected
// by the non-null outputs.  K must be a multiple of 64 (and k_per_split too);
// lda, ldb multiples of 8 elements; M and N any size (tiles are 128 x 128).
struct GemmArgs {
    const __nv_bfloat16* A;
    const __nv_bfloat16* B;
    int M, N, K, lda, ldb;
    int k_per_split;                  // K range of one blockIdx.z
    const float* bias;                // [N] or null
    bool silu;                        // activation applied to out_bf16 / out_bf16_t
    bool atomic_f32;                  // out_f32 += acc (split-K reduction), no other outputs
    float* out_f32;                   // [M][ldo]
    __nv_bfloat16* out_bf16;          // [M][ldo]
    __nv_bfloat16* out_bf16_t;        // [N][ldt] (transposed)
    float* out_dact;                  // [M][ldo]: act'(z)
    int ldo, ldt;
    // out_bf16 row stride; with split_bf16 the value is stored as hi at column n and
    // lo = bf16(a - hi) at column n + N, so the next layer reads a 16-bit mantissa
    int ldb16;
    bool split_bf16;
    // fused 128 -> 1 head: out_head[m] = *head_bias + sum_n head_w[n] * act(z[m][n]),
    // in FP32 (requires N <= 128: the whole row sits in one tile)
    const __nv_bfloat16* head_w;
    const float* head_bias;
    float* out_head;
    int* error;                       // set to 1 if a tensor-core wait timed out
};

size_t gemm_smem_bytes();
cudaError_t gemm_set_smem_limit();  // on the current device
cudaError_t gemm_launch(const GemmArgs& g, int splits, cudaStream_t stream);

// Shared-memory limits of the surrogate kernels on the current device, once per
// device (bit d of a process-wide mask); every launcher calls it first.
cudaError_t mlp_prepare_device();

// ---- MLP surrogate: 5 -> 128 -> 128 -> 128 -> 128 -> 1, SiLU.
// Parameters (FP32 master copy): five [128 out][128 in] weight matrices (layer 1 uses
// inputs 0..4, the head output 0) then five biases of 128.  Every layer input is
// carried as a BF16 pair (hi, lo = bf16(a - hi)) and every BF16 weight matrix is
// stored twice along K, [W | W], so one K-doubled GEMM sums both halves:
//   layer 1: rows of kMlpInK = 64: features hi in columns 0..4, lo in 5..9;
//   layers 2-4: rows of 256: hi in 0..127, lo in 128..255;
//   head: FP32 dot product of the layer-4 activations with BF16 W5 row 0.
constexpr int kMlpIn = 5;
constexpr int kMlpWidth = 128;
constexpr int kMlpInK = 64;
constexpr int kMlpHidK = 2 * kMlpWidth;
constexpr int kMlpLayers = 5;  // four hidden layers + the output layer
constexpr int kMlpWeights = kMlpLayers * kMlpWidth * kMlpWidth;
constexpr int kMlpParams = kMlpWeights + kMlpLayers * kMlpWidth;  // weights then biases
// BF16 forward weights: 4 slots of [128][256] (layer 1 uses [128][64]) + head row
constexpr int kMlpFwdSlot = kMlpWidth * kMlpHidK;
constexpr int kMlpFwdWeights = 4 * kMlpFwdSlot + kMlpWidth;

// Floors at or below -kNoFloor mark training rows outside the early-exercise region.
constexpr float kNoFloor = 1e30f;

// Box of the raw features the network was trained on; inputs outside go to FD.
struct MlpBox {
    double lo[kMlpIn];
    double hi[kMlpIn];
};

// Features [n][5] (may be null), in-box flags and analytic base prices (may be null):
// Barone-Adesi-Whaley for American options, Black-Scholes for European ones.
void mlp_launch_featurize(const kwg_option* opts, int n, const MlpBox& box, float* x, uint8_t* inside, double* base,
                          cudaStream_t st);
// Feature rows f[idx[r]] (idx null: f[r]) for r < b -> split BF16 rows x [b_pad][64]
// (rows >= b zero), transposed hi rows xt [64][b_pad] (may be null), targets tb and
// floors fb (either may be null; a null fl gives no floor).
void mlp_launch_pack(const float* f, const float* t, const float* fl, const int32_t* idx, int b, int b_pad,
                     __nv_bfloat16* x, __nv_bfloat16* xt, float* tb, float* fb, cudaStream_t st);
void mlp_launch_out_grad(const float* y, const float* t, const float* fl, int b, int b_pad, __nv_bfloat16* dy,
                         __nv_bfloat16* dyt, float* db5, double* loss, cudaStream_t st);
void mlp_launch_dz(const float* da, const float* dact, int b, int b_pad, __nv_bfloat16* dz, __nv_bfloat16* dzt,
                   float* db, cudaStream_t st);
void mlp_launch_adam(float* p, const float* g, float* m, float* v, int n, float lr, float b1, float b2, float eps,
                     float c1, float c2, cudaStream_t st);
// BF16 forward weights (layout above) and W^T [5][128 in][128 out] for the backward.
void mlp_launch_refresh(const float* w, __nv_bfloat16* wb, __nv_bfloat16* wt, cudaStream_t st);
void mlp_launch_price(const kwg_option* opts, const float* y, const double* base, int n, float y_scale,
                      double* prices, cudaStream_t st);

// Network prices of n options in one persistent launch (mlp_fused.cu): `sms` CTAs at
// most, weights resident in shared memory, activations on chip.
cudaError_t mlp_launch_price_fused(const kwg_option* opts, int n, const MlpBox& box, const __nv_bfloat16* wb,
                                   const float* params, float y_scale, double* prices, uint8_t* inside, int* error,
                                   int sms, cudaStream_t st);

}  // namespace kwg
