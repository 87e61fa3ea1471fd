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
struct BawSetup {
    double w, K, lk, zt, mu, qe, dq, dr;
};

__device__ __forceinline__ float ncdf(float x) { return normcdff(x); }
__device__ __forceinline__ double ncdf(double x) { return normcdf(x); }
__device__ __forceinline__ float ex(float x) { return expf(x); }
__device__ __forceinline__ double ex(double x) { return exp(x); }

// g(u) at S = e^u and dg/du; g > 0 on the exercise side (put: below S_c, call: above).
template <typename F>
__device__ __forceinline__ F baw_g(const BawSetup& b, F u, F& slope)
{
    const F w = (F)b.w, K = (F)b.K, zt = (F)b.zt, qe = (F)b.qe, dq = (F)b.dq;
    const F s = ex(u);
    const F d1 = (u - (F)b.lk + (F)b.mu) / zt, d2 = d1 - zt;
    const F nd1 = ncdf(w * d1);
    const F e = w * (s * dq * nd1 - K * (F)b.dr * ncdf(w * d2));
    const F c = F(1) - dq * nd1;
    const F pdf = F(0.3989422804014327) * ex(F(-0.5) * d1 * d1);
    slope = s * (w * c * (F(1) - F(1) / qe) + dq * pdf / (zt * qe));
    return w * (s - K) - e - w * c * s / qe;
}

// Newton steps in u safeguarded by the sign bracket [lo, hi] (bisection whenever a
// step leaves it), at most `iters` evaluations, until a step is below tol.
template <typename F>
__device__ F baw_root(const BawSetup& b, F u, F lo, F hi, int iters, F tol)
{
    for (int it = 0; it < iters; ++it) {
        F sl;
        const F gu = baw_g<F>(b, u, sl);
        if ((gu > F(0)) == (b.w < 0.)) lo = u; else hi = u;
        F un = u - gu / sl;
        if (!(un > lo && un < hi)) un = F(0.5) * (lo + hi);
        const F du = fabs(un - u);
        u = un;
        if (du < tol || hi - lo < tol) break;
    }
    return u;
}

__device__ inline double baw_price(const kwg_option& o, double euro)
{
    const double S = o.s, K = o.k, T = o.t, z = o.z, r = o.r, q = o.q;
    BawSetup b;
    b.w = o.w < 0 ? -1. : 1.;
    if (b.w < 0 ? !(r > 0.) : !(q > 0.)) return euro;
    const double s2 = z * z;
    b.K = K;
    b.lk = log(K);
    b.zt = z * sqrt(T);
    b.mu = (r - q + 0.5 * s2) * T;
    const double nn = 2. * (r - q) / s2;
    const double mk = r * T < 1e-12 ? 2. / (s2 * T) : 2. * r / (s2 * (-expm1(-r * T)));
    b.qe = 0.5 * (-(nn - 1.) + b.w * sqrt((nn - 1.) * (nn - 1.) + 4. * mk));
    b.dq = exp(-q * T);
    b.dr = exp(-r * T);
    const double lo = b.w < 0 ? b.lk - 60. : b.lk, hi = b.w < 0 ? b.lk : b.lk + 60.;
    double sl;
    if (!(baw_g<double>(b, b.w < 0 ? lo : hi, sl) > 0.)) return euro;
    // FP32 search from one standard deviation off the strike, then FP64 Newton polish;
    // a polish step that jumps by more than 1e-3 falls back to the FP64 search
    const float u32 = baw_root<float>(b, (float)(b.lk + b.w * fmin(b.zt, 30.)), (float)lo, (float)hi, 80, 1e-6f);
    double u = u32;
    bool ok = true;
    for (int it = 0; it < 4; ++it) {
        const double gu = baw_g<double>(b, u, sl);
        const double du = gu / sl;
        if (!(fabs(du) < 1e-3)) {
            ok = false;
            break;
        }
        u -= du;
        if (fabs(du) < 1e-14) break;
    }
    if (!ok) u = baw_root<double>(b, b.lk + b.w * fmin(b.zt, 30.), lo, hi, 200, 1e-14);
    const double sc = exp(u);
    const double d1c = (u - b.lk + b.mu) / b.zt;
    const double a = b.w * (sc / b.qe) * (1. - b.dq * normcdf(b.w * d1c));
    const bool cont = b.w < 0 ? S > sc : S < sc;
    const double v = cont ? euro + a * exp(b.qe * log(S / sc)) : b.w * (S - K);
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
