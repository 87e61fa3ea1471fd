// mlp_kernels.cu -- elementwise and reduction kernels of the MLP surrogate (the
// GEMMs are in mlp_gemm.cu).  Layer inputs are BF16 (hi, lo) pairs and the forward
// weights are stored twice along K (layout in mlp.h).
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "kwg.h"
#include "mlp.h"
#include "mlp_math.cuh"

namespace kwg {

// Features, in-box flag and the analytic base price: Barone-Adesi-Whaley for
// American options, Black-Scholes for European ones.
__global__ void mlp_featurize(const kwg_option* __restrict__ opts, int n, MlpBox box, float* __restrict__ x,
                              uint8_t* __restrict__ inside, double* __restrict__ base)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const kwg_option o = opts[i];
    float f[kMlpIn];
    bool in = false;
    features(o, box, f, in);
    if (x)
#pragma unroll
        for (int c = 0; c < kMlpIn; ++c) x[(size_t)i * kMlpIn + c] = f[c];
    if (base) base[i] = base_price(o);
    if (inside) inside[i] = in ? 1 : 0;
}

// One thread per row r < b_pad: split BF16 row of 64 (hi 0..4, lo 5..9, zeros),
// transposed hi (rows 0..4 of xt; rows 5..63 zero), target and floor.
__global__ void mlp_pack(const float* __restrict__ f, const float* __restrict__ t, const float* __restrict__ fl,
                         const int32_t* __restrict__ idx, int b, int b_pad, __nv_bfloat16* __restrict__ x,
                         __nv_bfloat16* __restrict__ xt, float* __restrict__ tb, float* __restrict__ fb)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= b_pad) return;
    const bool real = r < b;
    const int src = real ? (idx ? idx[r] : r) : 0;
    float fr[kMlpIn];
#pragma unroll
    for (int c = 0; c < kMlpIn; ++c) fr[c] = real ? f[(size_t)src * kMlpIn + c] : 0.f;
    __align__(16) __nv_bfloat16 row[kMlpInK];
    split_features<kMlpInK>(fr, row);
    uint4* dst = reinterpret_cast<uint4*>(x + (size_t)r * kMlpInK);
    const uint4* srcv = reinterpret_cast<const uint4*>(row);
#pragma unroll
    for (int q = 0; q < kMlpInK / 8; ++q) dst[q] = srcv[q];
    if (xt)
        for (int c = 0; c < kMlpInK; ++c) xt[(size_t)c * b_pad + r] = c < kMlpIn ? row[c] : __float2bfloat16(0.f);
    if (tb) tb[r] = real && t ? t[src] : 0.f;
    if (fb) fb[r] = real && fl ? fl[src] : -kNoFloor;
}

// Output gradient of the loss mean(e^2): e = y - t for rows without a floor; for
// rows in the early-exercise region (floor f > -kNoFloor) the price is the intrinsic
// value and e = max(0, y - f) only keeps y at or below the floor.  dy = 2 e / b;
// dY (row-major) and dY^T (column 0 / row 0 only nonzero) feed the output layer's GEMMs.
__global__ void mlp_out_grad(const float* __restrict__ y, const float* __restrict__ t, const float* __restrict__ fl,
                             int b, int b_pad, __nv_bfloat16* __restrict__ dy, __nv_bfloat16* __restrict__ dyt,
                             float* __restrict__ db5, double* __restrict__ loss)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= b_pad) return;
    float g = 0.f;
    if (r < b) {
        const float f = fl ? fl[r] : -kNoFloor;
        const float e = f > -kNoFloor ? fmaxf(0.f, y[r] - f) : y[r] - t[r];
        g = 2.f * e / (float)b;
        atomicAdd(loss, (double)e * (double)e / (double)b);
        atomicAdd(db5, g);
    }
    dy[(size_t)r * kMlpWidth] = __float2bfloat16(g);
    dyt[r] = __float2bfloat16(g);  // row 0 of dY^T [128][b_pad]
}

// dZ = dA * act'(z) on real rows; row-major and transposed BF16 copies; bias
// gradient db[c] += sum over rows of dZ[:, c] (FP32, before rounding).
__global__ void mlp_dz(const float* __restrict__ da, const float* __restrict__ dact, int b, int b_pad,
                       __nv_bfloat16* __restrict__ dz, __nv_bfloat16* __restrict__ dzt, float* __restrict__ db)
{
    const int c = threadIdx.x;  // one thread per column
    const int r0 = blockIdx.x * 32;
    float acc = 0.f;
    for (int rr = 0; rr < 32; ++rr) {
        const int r = r0 + rr;
        if (r >= b_pad) break;
        const float v = r < b ? da[(size_t)r * kMlpWidth + c] * dact[(size_t)r * kMlpWidth + c] : 0.f;
        acc += v;
        const __nv_bfloat16 h = __float2bfloat16(v);
        dz[(size_t)r * kMlpWidth + c] = h;
        dzt[(size_t)c * b_pad + r] = h;
    }
    atomicAdd(db + c, acc);
}

// Adam on FP32 master parameters.
__global__ void mlp_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                         float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// BF16 copies of the weights: the K-doubled forward operands [W | W] (layer 1:
// inputs 0..4 at columns 0..4 and 5..9 of a 64-wide row), the head row, and
// W^T [in][out] for every layer.  Grid (128 rows, 5 layers), 128 threads.
__global__ void mlp_refresh(const float* __restrict__ w, __nv_bfloat16* __restrict__ wb,
                            __nv_bfloat16* __restrict__ wt)
{
    const int l = blockIdx.y;
    const int o = blockIdx.x, i = threadIdx.x;
    const size_t base = (size_t)l * kMlpWidth * kMlpWidth;
    const __nv_bfloat16 h = __float2bfloat16(w[base + (size_t)o * kMlpWidth + i]);
    wt[base + (size_t)i * kMlpWidth + o] = h;
    __nv_bfloat16* slot = wb + (size_t)l * kMlpFwdSlot;
    if (l == 0) {
        if (i < kMlpInK) {
            const int src = i < kMlpIn ? i : i < 2 * kMlpIn ? i - kMlpIn : -1;
            slot[(size_t)o * kMlpInK + i] =
                src >= 0 ? __float2bfloat16(w[base + (size_t)o * kMlpWidth + src]) : __float2bfloat16(0.f);
        }
    } else if (l < 4) {
        slot[(size_t)o * kMlpHidK + i] = h;
        slot[(size_t)o * kMlpHidK + kMlpWidth + i] = h;
    } else if (o == 0) {
        slot[i] = h;  // head row: W5[0][i]
    }
}

// Surrogate price = max(intrinsic, base + K * premium), premium = y / y_scale, base
// the analytic price of mlp_featurize.
__global__ void mlp_price(const kwg_option* __restrict__ opts, const float* __restrict__ y,
                          const double* __restrict__ base, int n, float y_scale, double* __restrict__ prices)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const kwg_option o = opts[i];
    const double v = base[i] + o.k * (double)(y[i] / y_scale);
    prices[i] = o.e ? fmax(v, intrinsic(o)) : v;
}

void mlp_launch_featurize(const kwg_option* opts, int n, const MlpBox& box, float* x, uint8_t* inside, double* base,
                          cudaStream_t st)
{
    mlp_featurize<<<(n + 127) / 128, 128, 0, st>>>(opts, n, box, x, inside, base);
}

void mlp_launch_pack(const float* f, const float* t, const float* fl, const int32_t* idx, int b, int b_pad,
                     __nv_bfloat16* x, __nv_bfloat16* xt, float* tb, float* fb, cudaStream_t st)
{
    mlp_pack<<<(b_pad + 127) / 128, 128, 0, st>>>(f, t, fl, idx, b, b_pad, x, xt, tb, fb);
}

void mlp_launch_out_grad(const float* y, const float* t, const float* fl, int b, int b_pad, __nv_bfloat16* dy,
                         __nv_bfloat16* dyt, float* db5, double* loss, cudaStream_t st)
{
    mlp_out_grad<<<(b_pad + 127) / 128, 128, 0, st>>>(y, t, fl, b, b_pad, dy, dyt, db5, loss);
}

void mlp_launch_dz(const float* da, const float* dact, int b, int b_pad, __nv_bfloat16* dz, __nv_bfloat16* dzt,
                   float* db, cudaStream_t st)
{
    mlp_dz<<<(b_pad + 31) / 32, kMlpWidth, 0, st>>>(da, dact, b, b_pad, dz, dzt, db);
}

void mlp_launch_adam(float* p, const float* g, float* m, float* v, int n, float lr, float b1, float b2, float eps,
                     float c1, float c2, cudaStream_t st)
{
    mlp_adam<<<(n + 255) / 256, 256, 0, st>>>(p, g, m, v, n, lr, b1, b2, eps, c1, c2);
}

void mlp_launch_refresh(const float* w, __nv_bfloat16* wb, __nv_bfloat16* wt, cudaStream_t st)
{
    mlp_refresh<<<dim3(kMlpWidth, kMlpLayers), kMlpWidth, 0, st>>>(w, wb, wt);
}

void mlp_launch_price(const kwg_option* opts, const float* y, const double* base, int n, float y_scale,
                      double* prices, cudaStream_t st)
{
    mlp_price<<<(n + 127) / 128, 128, 0, st>>>(opts, y, base, n, y_scale, prices);
}

}  // namespace kwg
