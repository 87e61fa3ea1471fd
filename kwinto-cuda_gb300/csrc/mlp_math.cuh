// mlp_math.cuh -- per-option device math of the MLP surrogate, shared by the
// layer-by-layer kernels (mlp_kernels.cu) and the fused pricing kernel
// (mlp_fused.cu): features, intrinsic value, Black-Scholes and Barone-Adesi-Whaley
// prices.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "kwg.h"
#include "mlp.h"

namespace kwg {

// Features of one option (normalised by the box to [-1, 1]) and its Black-Scholes
// European price.  Features: log(K/S), vol*sqrt(T), r*T, q*T, put/call (-1/+1).
__device__ __forceinline__ void features(const kwg_option& o, const MlpBox& box, float f[kMlpIn], bool& inside)
{
    const double raw[kMlpIn] = {log(o.k / o.s), o.z * sqrt(o.t), o.r * o.t, o.q * o.t, o.w < 0 ? -1. : 1.};
    inside = o.e != 0 && o.t > 0. && o.z > 0. && o.s > 0. && o.k > 0.;
    for (int i = 0; i < kMlpIn; ++i) {
        const double lo = box.lo[i], hi = box.hi[i];
        if (!(raw[i] >= lo && raw[i] <= hi)) inside = false;
        f[i] = (float)(2. * (raw[i] - lo) / (hi - lo) - 1.);
    }
}

// Black-Scholes European price (the reference's formula, src/Pricer/kwBlackScholes.cpp:36-47).
__device__ __forceinline__ double bs_euro(const kwg_option& o)
{
    const double zt = o.z * sqrt(o.t);
    const double d1 = 1. / zt * (log(o.s / o.k) + (o.r - o.q + 0.5 * o.z * o.z) * o.t);
    const double d2 = d1 - zt;
    const double w = o.w < 0 ? -1. : 1.;
    return w * (o.s * normcdf(w * d1) * exp(-o.q * o.t) - o.k * normcdf(w * d2) * exp(-o.r * o.t));
}

// Barone-Adesi & Whaley (1987) quadratic approximation of the American price, with
// continuous dividend yield q (cost of carry b = r - q).  With
//     M/K(T) = 2r / (sigma^2 (1 - e^{-rT})),  N = 2b / sigma^2,
//     qe = (-(N - 1) -+ sqrt((N - 1)^2 + 4 M/K(T))) / 2      (put -, call +),
// the critical price S_c solves  g(S) = w (S - K) - E(S) - w (1 - e^{-qT} N(w d1(S))) S / qe = 0
// (E the European price); the American price is E(S) + A (S / S_c)^qe with
// A = w (S_c / qe)(1 - e^{-qT} N(w d1(S_c))) on the continuation side of S_c and the
// intrinsic value beyond it.  Puts with r <= 0 and calls with q <= 0 are never
// exercised early (the European price), nor are contracts whose S_c lies beyond e^60 K.
//
// Precision: E(S) comes in FP64; S_c and the premium term A (S/S_c)^qe are FP32.
// The price is stationary in S_c at the root (value matching and smooth pasting),
// so the FP32 root moves it to second order only, and the premium term is a small
// part of the price: the FP32 parts change the price by ~1e-7 K.
struct BawSetup {
    float w, K, lk, zt, mu, qe, dq, dr;
};

__device__ __forceinline__ float ncdf(float x) { return normcdff(x); }

// g(u) at S = e^u and dg/du; g > 0 on the exercise side (put: below S_c, call: above).
__device__ __forceinline__ float baw_g(const BawSetup& b, float u, float& slope)
{
    const float s = expf(u);
    const float d1 = (u - b.lk + b.mu) / b.zt, d2 = d1 - b.zt;
    const float nd1 = ncdf(b.w * d1);
    const float e = b.w * (s * b.dq * nd1 - b.K * b.dr * ncdf(b.w * d2));
    const float c = 1.f - b.dq * nd1;
    const float pdf = 0.3989422804f * expf(-0.5f * d1 * d1);
    slope = s * (b.w * c * (1.f - 1.f / b.qe) + b.dq * pdf / (b.zt * b.qe));
    return b.w * (s - b.K) - e - b.w * c * s / b.qe;
}

__device__ inline double baw_price(const kwg_option& o, double euro)
{
    const float w = o.w < 0 ? -1.f : 1.f;
    if (w < 0 ? !(o.r > 0.) : !(o.q > 0.)) return euro;
    const float T = (float)o.t, z = (float)o.z, r = (float)o.r, q = (float)o.q, S = (float)o.s;
    BawSetup b;
    b.w = w;
    b.K = (float)o.k;
    b.lk = logf(b.K);
    const float s2 = z * z;
    b.zt = z * sqrtf(T);
    b.mu = (r - q + 0.5f * s2) * T;
    const float nn = 2.f * (r - q) / s2;
    const float mk = r * T < 1e-6f ? 2.f / (s2 * T) : 2.f * r / (s2 * (-expm1f(-r * T)));
    b.qe = 0.5f * (-(nn - 1.f) + w * sqrtf((nn - 1.f) * (nn - 1.f) + 4.f * mk));
    b.dq = expf(-q * T);
    b.dr = expf(-r * T);
    float lo = w < 0 ? b.lk - 60.f : b.lk, hi = w < 0 ? b.lk : b.lk + 60.f;
    float sl;
    if (!(baw_g(b, w < 0 ? lo : hi, sl) > 0.f)) return euro;
    // Newton in u = log S from one standard deviation off the strike, safeguarded by
    // the sign bracket (bisection whenever a step leaves it)
    float u = b.lk + w * fminf(b.zt, 30.f);
    for (int it = 0; it < 60; ++it) {
        const float gu = baw_g(b, u, sl);
        if ((gu > 0.f) == (w < 0.f)) lo = u; else hi = u;
        float un = u - gu / sl;
        if (!(un > lo && un < hi)) un = 0.5f * (lo + hi);
        const float du = fabsf(un - u);
        u = un;
        if (du < 2e-7f * fmaxf(1.f, fabsf(u)) || hi - lo < 2e-7f * fmaxf(1.f, fabsf(u))) break;
    }
    const float sc = expf(u);
    const float d1c = (u - b.lk + b.mu) / b.zt;
    const float a = w * (sc / b.qe) * (1.f - b.dq * ncdf(w * d1c));
    const bool cont = w < 0 ? S > sc : S < sc;
    const double v = cont ? euro + (double)(a * expf(b.qe * logf(S / sc))) : (double)w * (o.s - o.k);
    return fmax(v, euro);
}

__device__ __forceinline__ double intrinsic(const kwg_option& o)
{
    return fmax(0., o.w < 0 ? o.k - o.s : o.s - o.k);
}

// Feature row of the first layer: hi parts of the 5 features in columns 0..4, lo
// parts (bf16(f - hi)) in columns 5..9, zeros up to `width`.
template <int kWidth>
__device__ __forceinline__ void split_features(const float f[kMlpIn], __nv_bfloat16 (&row)[kWidth])
{
#pragma unroll
    for (int c = 0; c < kWidth; ++c) row[c] = __float2bfloat16(0.f);
#pragma unroll
    for (int c = 0; c < kMlpIn; ++c) {
        const __nv_bfloat16 hi = __float2bfloat16(f[c]);
        row[c] = hi;
        row[kMlpIn + c] = __float2bfloat16(f[c] - __bfloat162float(hi));
    }
}

__device__ __forceinline__ float silu_f(float z) { return z / (1.f + __expf(-z)); }

// Analytic base price of a valid contract: Barone-Adesi-Whaley for American
// exercise, Black-Scholes for European; 0 for invalid inputs.
__device__ __forceinline__ double base_price(const kwg_option& o)
{
    const bool valid = o.t > 0. && o.z > 0. && o.s > 0. && o.k > 0.;
    if (!valid) return 0.;
    const double e = bs_euro(o);
    return o.e ? baw_price(o, e) : e;
}

}  // namespace kwg
