// fd1d_common.cuh -- device helpers shared by the FD1D kernels: the per-PDE grid
// (x-grid, t-step, payoff) and the reference's tridiagonal operator rows.
//
// All grid and operator arithmetic uses explicitly rounded FP64 intrinsics
// (__dmul_rn, __dadd_rn, ...) so the compiler cannot contract it into FMAs: the
// evaluation order is the reference's, and the same inline code is used by every
// kernel that needs a node coordinate, so the setup and the interpolation see
// bit-identical grids.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "fd1d_kernels.h"
#include "kwg.h"

namespace kwg {

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }

// Geometry of one PDE's log(S/K) grid (src/Pricer/kwFd1d.cpp:110-125): centred at
// 0, half-width scale*z*sqrt(t), nodes x_j = d*sinh(yMin(1-y_j) + yMax y_j) with
// y_j = j/(N-1).  uniform: the d -> infinity limit, x_j = xMin(1-y_j) + xMax y_j.
struct Grid {
    double xMin, xMax, yMin, yMax, density, dy;
    int n;
    bool uniform;

    __device__ __forceinline__ void init(double z, double t, double scale, double dens, int n_,
                                         bool unif)
    {
        const double xMid = 0.;
        const double w = mul(mul(scale, z), sqrt(t));
        xMin = sub(xMid, w);
        xMax = add(xMid, w);
        density = dens;
        uniform = unif;
        n = n_;
        dy = dvd(1., (double)(n_ - 1));
        if (!unif) {
            yMin = asinh(dvd(sub(xMin, xMid), dens));
            yMax = asinh(dvd(sub(xMax, xMid), dens));
        } else {
            yMin = yMax = 0.;
        }
    }

    __device__ __forceinline__ double x(int j) const
    {
        const double yj = mul((double)j, dy);
        if (uniform) return add(mul(xMin, sub(1.0, yj)), mul(xMax, yj));
        return add(0., mul(density, sinh(add(mul(yMin, sub(1.0, yj)), mul(yMax, yj)))));
    }
};

// Normalised payoff on the grid (src/Pricer/kwFd1d.cpp:129-139):
// put max(0, 1 - e^x), call max(0, e^x - 1); max<f64>(0, v) == (0 < v) ? v : 0.
__device__ __forceinline__ double payoff(int8_t w, double x)
{
    const double ex = exp(x);
    const double v = (w < 0) ? sub(1., ex) : sub(ex, 1.);
    return (0. < v) ? v : 0.;
}

// One row (bl, b, bu) of a tridiagonal matrix.
struct Row {
    double bl, b, bu;
};

// Row j of the reference's implicit matrix B = 1 - theta dt A
// (src/Math/kwFd1d.cpp:73-114), with the reference's operation order, from the
// reciprocal spacings inv_u = 1/(xp - x0), inv_m = 1/(xp - xm),
// inv_d = 1/(x0 - xm) (row 0 reads inv_u, row n-1 inv_d): a caller walking the grid
// passes a node's inv_u on as the next node's inv_d.  Bit-identical to implicit_row.
__device__ __forceinline__ Row implicit_row_r(int j, int n, double inv_u, double inv_m, double inv_d,
                                              double theta, double dt, double a0, double ax, double axx)
{
    Row r;
    const double tdt = mul(theta, dt);    // theta * dt
    const double ntdt = mul(-theta, dt);  // -theta * dt
    if (j == 0) {
        r.bl = 0.;
        r.b = sub(1., mul(tdt, sub(a0, mul(inv_u, ax))));
        r.bu = mul(ntdt, mul(inv_u, ax));
    } else if (j == n - 1) {
        r.bl = mul(ntdt, mul(-inv_d, ax));
        r.b = sub(1., mul(tdt, add(a0, mul(inv_d, ax))));
        r.bu = 0.;
    } else {
        const double inv_dx2u = mul(mul(2., inv_u), inv_m);
        const double inv_dx2m = mul(mul(2., inv_d), inv_u);
        const double inv_dx2l = mul(mul(2., inv_d), inv_m);
        r.bl = mul(ntdt, add(mul(-inv_m, ax), mul(inv_dx2l, axx)));
        r.b = sub(1., mul(tdt, sub(a0, mul(inv_dx2m, axx))));
        r.bu = mul(ntdt, add(mul(inv_m, ax), mul(inv_dx2u, axx)));
    }
    return r;
}

// The same row from the nodes: xm, x0, xp are x_{j-1}, x_j, x_{j+1} (unused ones ignored).
__device__ __forceinline__ Row implicit_row(int j, int n, double xm, double x0, double xp,
                                            double theta, double dt, double a0, double ax,
                                            double axx)
{
    if (j == 0) return implicit_row_r(j, n, dvd(1., sub(xp, x0)), 0., 0., theta, dt, a0, ax, axx);
    if (j == n - 1) return implicit_row_r(j, n, 0., 0., dvd(1., sub(x0, xm)), theta, dt, a0, ax, axx);
    return implicit_row_r(j, n, dvd(1., sub(xp, x0)), dvd(1., sub(xp, xm)), dvd(1., sub(x0, xm)), theta, dt, a0,
                          ax, axx);
}

// PDE coefficients of one option (src/Pricer/kwFd1d.cpp:79-85):
// a0 = -r, ax = r - q - z^2/2, axx = z^2/2.
struct Coef {
    double a0, ax, axx;
};

__device__ __forceinline__ Coef pde_coef(double r, double q, double z)
{
    Coef c;
    const double zz2 = dvd(mul(z, z), 2.);
    c.a0 = -r;
    c.ax = sub(sub(r, q), zz2);
    c.axx = zz2;
    return c;
}

// The reference's time step: the t-grid is t_j = j * T/(tDim-1)
// (src/Pricer/kwFd1d.cpp:97-103); the GPU uses that constant step on every row.
__device__ __forceinline__ double time_step(double t, int t_dim)
{
    return dvd(sub(t, 0.0), (double)(t_dim - 1));
}

// max(v, p) for p >= +0 without the FP64 pipe: as signed 64-bit integers the bit
// patterns of doubles >= +0 are ordered like the values, and every negative double
// (sign bit set) is a negative integer, so it loses to p.
__device__ __forceinline__ double max_floor(double v, double p)
{
    const long long vb = __double_as_longlong(v), pb = __double_as_longlong(p);
    return (vb < pb) ? p : v;
}

}  // namespace kwg
