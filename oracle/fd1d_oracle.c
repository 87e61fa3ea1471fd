/*
 * fd1d_oracle.c -- CPU restatement of the reference FD1D American-option pricer.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: the parity tests, the smoke
 * check and the CPU-baseline leg of the benchmark compare against it.  The product
 * path (libkwg.so) never links, loads or calls it.
 *
 * It restates, in plain C and in the same floating-point evaluation order, the
 * algorithm of gituliar/kwinto-cuda:
 *   - Fd1d_Pricer::price          src/Pricer/kwFd1d.cpp:21-160
 *       dedup by (t,r,q,z,e,w)    src/Pricer/kwFd1d.cpp:28-65
 *       PDE coefficients          src/Pricer/kwFd1d.cpp:74-86
 *       t-grid                    src/Pricer/kwFd1d.cpp:97-103
 *       sinh-stretched x-grid     src/Pricer/kwFd1d.cpp:110-125
 *       payoff                    src/Pricer/kwFd1d.cpp:129-139
 *       price = k * value         src/Pricer/kwFd1d.cpp:148-157
 *   - Fd1d::solveOne              src/Math/kwFd1d.cpp:61-136 (theta scheme + projection)
 *   - kw::solveTridiagonal        src/Math/kwMath.cpp:16-49  (Thomas)
 *   - Fd1d::value                 src/Math/kwFd1d.cpp:139-158 (linear search + interpolation)
 *   - BlackScholes_Pricer         src/Pricer/kwBlackScholes.cpp:27-49, cdfNormal src/Math/kwMath.cpp:9-13
 *   - Fd1d_BlackScholes_Pricer    src/Pricer/kwFd1d_BlackScholes.cpp:15-42
 *
 * Compiled with -ffp-contract=off so that no multiply-add is fused: with the same
 * libm it reproduces the reference bit for bit (checked against the reference
 * built from its own sources, see oracle/Makefile and tests/test_oracle.py).
 *
 * Extensions over the reference, each off by default so that the default call is
 * the reference algorithm:
 *   theta      any value in [0,1] (the reference hard-codes 0.5, src/Math/kwFd1d.h:31)
 *   uniform    exactly uniform x-grid, the density -> infinity limit of the sinh grid
 *   const_dt   dt = T/(tDim-1) on every step instead of t[j+1]-t[j]
 * Work is spread over POSIX threads, one PDE at a time, like the reference's
 * thread pool (src/kwThreadPool.cpp:43-53, one job per PDE).
 */
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* Same layout as kw::Option (src/Core/kwAsset.h:12-22): 6 f64, u8, i8, padded to 56 B. */
typedef struct {
    double t, k, z, r, q, s;
    uint8_t e;
    int8_t w;
} kwor_option;

typedef struct {
    double density;   /* FD1D.DENSITY, reference default 0.25 */
    double scale;     /* FD1D.SCALE,   reference default 50   */
    double theta;     /* 0.5 in the reference                 */
    int64_t t_dim;    /* FD1D.T_GRID_SIZE, default 512        */
    int64_t x_dim;    /* FD1D.X_GRID_SIZE, default 512        */
    int32_t uniform;  /* 0 = reference sinh grid              */
    int32_t const_dt; /* 0 = reference per-step dt            */
} kwor_params;

enum { KWOR_OK = 0, KWOR_OUT_OF_GRID = 1, KWOR_SOLVER_ERROR = 2, KWOR_BAD_INPUT = 3 };

/* ---------------------------------------------------------------- dedup (kwFd1d.cpp:28-65) */

static const kwor_option* g_sort_assets; /* qsort has no context argument; guarded by g_sort_mu */
static pthread_mutex_t g_sort_mu = PTHREAD_MUTEX_INITIALIZER;

/* std::tie(l.t, l.r, l.q, l.z, l.e, l.w) < std::tie(...) (kwFd1d.cpp:33-35) */
static int key_less(const kwor_option* l, const kwor_option* r)
{
    if (l->t < r->t) return 1;
    if (r->t < l->t) return 0;
    if (l->r < r->r) return 1;
    if (r->r < l->r) return 0;
    if (l->q < r->q) return 1;
    if (r->q < l->q) return 0;
    if (l->z < r->z) return 1;
    if (r->z < l->z) return 0;
    if (l->e < r->e) return 1;
    if (r->e < l->e) return 0;
    return l->w < r->w;
}

static int key_cmp_idx(const void* a, const void* b)
{
    uint32_t ia = *(const uint32_t*)a, ib = *(const uint32_t*)b;
    const kwor_option* l = &g_sort_assets[ia];
    const kwor_option* r = &g_sort_assets[ib];
    if (key_less(l, r)) return -1;
    if (key_less(r, l)) return 1;
    return (ia > ib) - (ia < ib);
}

/* Builds asset2pde[n] and pde2asset[m]; returns m.  Equal keys share one PDE. */
size_t kwor_dedup(const kwor_option* assets, size_t n, uint32_t* asset2pde, uint32_t* pde2asset)
{
    if (n == 0) return 0;
    uint32_t* idx = (uint32_t*)malloc(n * sizeof(uint32_t));
    for (size_t i = 0; i < n; ++i) idx[i] = (uint32_t)i;
    pthread_mutex_lock(&g_sort_mu);
    g_sort_assets = assets;
    qsort(idx, n, sizeof(uint32_t), key_cmp_idx);
    pthread_mutex_unlock(&g_sort_mu);
    size_t k = 0;
    asset2pde[idx[0]] = 0;
    pde2asset[0] = idx[0];
    for (size_t i = 1; i < n; ++i) {
        const kwor_option* l = &assets[idx[i - 1]];
        const kwor_option* r = &assets[idx[i]];
        int equal = key_less(l, r) == key_less(r, l);
        if (!equal) {
            k += 1;
            pde2asset[k] = idx[i];
        }
        asset2pde[idx[i]] = (uint32_t)k;
    }
    free(idx);
    return k + 1;
}

/* ---------------------------------------------------------------- grids (kwFd1d.cpp:97-139) */

/* t-grid: t_j = tMin + j*dt, dt = (tMax - tMin)/(tDim-1) (kwFd1d.cpp:97-103). */
void kwor_t_grid(double t_mat, int64_t t_dim, double* t)
{
    double tMin = 0.0, tMax = t_mat;
    double dt = (tMax - tMin) / (double)(t_dim - 1);
    for (int64_t j = 0; j < t_dim; ++j) t[j] = tMin + (double)j * dt;
}

/* x-grid (kwFd1d.cpp:110-125): x_j = xMid + d*sinh(yMin(1-y_j) + yMax y_j), centred at 0. */
void kwor_x_grid(double z, double t_mat, double scale, double density, int uniform, int64_t x_dim,
                 double* x)
{
    const double xMid = 0.;
    const double xMin = xMid - scale * z * sqrt(t_mat);
    const double xMax = xMid + scale * z * sqrt(t_mat);
    const double dy = 1. / (double)(x_dim - 1);
    if (uniform) {
        for (int64_t j = 0; j < x_dim; ++j) {
            const double yj = (double)j * dy;
            x[j] = xMin * (1.0 - yj) + xMax * yj;
        }
        return;
    }
    const double yMin = asinh((xMin - xMid) / density);
    const double yMax = asinh((xMax - xMid) / density);
    for (int64_t j = 0; j < x_dim; ++j) {
        const double yj = (double)j * dy;
        x[j] = xMid + density * sinh(yMin * (1.0 - yj) + yMax * yj);
    }
}

/* std::max<f64>(0, v) == (0 < v) ? v : 0 (kwFd1d.cpp:132-137). */
static double max0(double v) { return (0. < v) ? v : 0.; }

void kwor_payoff(int8_t w, const double* x, int64_t x_dim, double* v)
{
    for (int64_t j = 0; j < x_dim; ++j) {
        if (w < 0)
            v[j] = max0(1. - exp(x[j]));
        else
            v[j] = max0(exp(x[j]) - 1.);
    }
}

/* ---------------------------------------------------------------- Thomas (kwMath.cpp:16-49) */

static int solve_tridiagonal(int n, const double* al, const double* a, const double* au,
                             const double* y, double* x, double* gam)
{
    if (a[0] == 0) return 1;
    if (n <= 2) return 3;
    double bet;
    x[0] = y[0] / (bet = a[0]);
    for (int j = 1; j < n; j++) {
        gam[j] = au[j - 1] / bet;
        bet = a[j] - al[j] * gam[j];
        if (bet == 0) return 2;
        x[j] = (y[j] - al[j] * x[j - 1]) / bet;
    }
    for (int j = n - 2; j >= 0; --j) x[j] -= gam[j + 1] * x[j + 1];
    return 0;
}

/* ---------------------------------------------------------------- theta scheme (kwFd1d.cpp:61-136) */

typedef struct {
    double *bl, *b, *bu, *w, *gam;
} scratch_t;

/* Steps v (in: payoff, out: value at t=0) backward over the t-grid.  `payoff` is the
 * projection floor.  Returns the first solver error code (the reference prints it
 * and carries on, kwFd1d.cpp:46-48; so does this). */
int kwor_solve_one(double a0, double ax, double axx, int early, double theta, const double* t,
                   int64_t t_dim, const double* x, int64_t x_dim, const double* payoff, double* v,
                   int const_dt, scratch_t* s)
{
    const int64_t N = x_dim;
    double *bl = s->bl, *b = s->b, *bu = s->bu, *w = s->w;
    int first_err = 0;
    const double dt_const = (t[t_dim - 1] - t[0]) / (double)(t_dim - 1);
    for (int64_t ti = t_dim - 2; ti >= 0; --ti) {
        const double dt = const_dt ? dt_const : t[ti + 1] - t[ti];
        {
            const int64_t xi = 0;
            const double inv_dx = 1. / (x[xi + 1] - x[xi]);
            bl[xi] = 0;
            b[xi] = 1 - theta * dt * (a0 - inv_dx * ax);
            bu[xi] = -theta * dt * (inv_dx * ax);
            w[xi] = (1 + (1 - theta) * dt * a0) * v[xi] +
                    (1 - theta) * dt * (ax * inv_dx) * (v[xi + 1] - v[xi]);
        }
        for (int64_t xi = 1; xi < N - 1; ++xi) {
            const double inv_dxu = 1. / (x[xi + 1] - x[xi]);
            const double inv_dxm = 1. / (x[xi + 1] - x[xi - 1]);
            const double inv_dxd = 1. / (x[xi] - x[xi - 1]);
            const double inv_dx2u = 2. * inv_dxu * inv_dxm;
            const double inv_dx2m = 2. * inv_dxd * inv_dxu;
            const double inv_dx2l = 2. * inv_dxd * inv_dxm;
            bl[xi] = -theta * dt * (-inv_dxm * ax + inv_dx2l * axx);
            b[xi] = 1 - theta * dt * (a0 - inv_dx2m * axx);
            bu[xi] = -theta * dt * (inv_dxm * ax + inv_dx2u * axx);
            w[xi] = (1 + (1 - theta) * dt * a0) * v[xi] +
                    (1 - theta) * dt * (ax * inv_dxm) * (v[xi + 1] - v[xi - 1]) +
                    (1 - theta) * dt * (axx) *
                        (inv_dx2u * v[xi + 1] - inv_dx2m * v[xi] + inv_dx2l * v[xi - 1]);
        }
        {
            const int64_t xi = N - 1;
            const double inv_dx = 1. / (x[xi] - x[xi - 1]);
            bl[N - 1] = -theta * dt * (-inv_dx * ax);
            b[N - 1] = 1 - theta * dt * (a0 + inv_dx * ax);
            bu[N - 1] = 0;
            w[N - 1] = (1 + (1 - theta) * dt * a0) * v[xi] +
                       (1 - theta) * dt * (ax * inv_dx) * (v[xi] - v[xi - 1]);
        }
        int err = solve_tridiagonal((int)N, bl, b, bu, w, v, s->gam);
        if (err && !first_err) first_err = err;
        if (early) {
            for (int64_t xi = 0; xi < N - 1; ++xi) v[xi] = (v[xi] < payoff[xi]) ? payoff[xi] : v[xi];
        }
    }
    return first_err;
}

/* Fd1d::value (kwFd1d.cpp:139-158): first x_i >= x*, linear interpolation. 0 = ok. */
int kwor_value(const double* x, const double* v, int64_t x_dim, double xs, double* out)
{
    int64_t xi = 0;
    while ((xi < x_dim) && (x[xi] < xs)) ++xi;
    if ((xi == 0) || (xi == x_dim)) return 1;
    *out = ((x[xi] - xs) * v[xi - 1] + (xs - x[xi - 1]) * v[xi]) / (x[xi] - x[xi - 1]);
    return 0;
}

/* ---------------------------------------------------------------- batch pricer */

typedef struct {
    const kwor_option* assets;
    const uint32_t* pde2asset;
    size_t m;
    const kwor_params* p;
    double* xg;    /* m * x_dim */
    double* vg;    /* m * x_dim */
    int32_t* perr; /* m */
    atomic_size_t next;
} job_t;

static void* worker(void* arg)
{
    job_t* J = (job_t*)arg;
    const kwor_params* p = J->p;
    const int64_t N = p->x_dim, T = p->t_dim;
    double* buf = (double*)malloc(sizeof(double) * (size_t)(6 * N + T));
    scratch_t s = {buf, buf + N, buf + 2 * N, buf + 3 * N, buf + 4 * N};
    double* payoff = buf + 5 * N;
    double* t = buf + 6 * N;
    for (;;) {
        size_t i = atomic_fetch_add(&J->next, 1);
        if (i >= J->m) break;
        const kwor_option* a = &J->assets[J->pde2asset[i]];
        /* kwFd1d.cpp:79-85 */
        const double a0 = -a->r;
        const double ax = a->r - a->q - a->z * a->z / 2;
        const double axx = a->z * a->z / 2;
        double* x = J->xg + i * (size_t)N;
        double* v = J->vg + i * (size_t)N;
        kwor_t_grid(a->t, T, t);
        kwor_x_grid(a->z, a->t, p->scale, p->density, p->uniform, N, x);
        kwor_payoff(a->w, x, N, payoff);
        memcpy(v, payoff, sizeof(double) * (size_t)N);
        J->perr[i] = kwor_solve_one(a0, ax, axx, a->e != 0, p->theta, t, T, x, N, payoff, v,
                                    p->const_dt, &s);
    }
    free(buf);
    return NULL;
}

/* Prices n assets.  prices[i] = k * V(log(s/k)); an asset whose log-moneyness is
 * outside (x_0, x_{N-1}] gets NaN and status KWOR_OUT_OF_GRID.  Returns 0, or the
 * status of the first failing asset in input order (the reference fails the whole
 * call there, src/Pricer/kwFd1d.cpp:154-155) with its message in err. */
int kwor_fd1d_price(const kwor_option* assets, size_t n, const kwor_params* p, int nthreads,
                    double* prices, int32_t* status, char* err, size_t errlen)
{
    if (err && errlen) err[0] = 0;
    if (n == 0) return 0;
    if (p->x_dim < 3 || p->t_dim < 2) {
        if (err) snprintf(err, errlen, "kwor_fd1d_price: bad grid %lld x %lld",
                          (long long)p->x_dim, (long long)p->t_dim);
        return KWOR_BAD_INPUT;
    }
    uint32_t* asset2pde = (uint32_t*)malloc(n * sizeof(uint32_t));
    uint32_t* pde2asset = (uint32_t*)malloc(n * sizeof(uint32_t));
    size_t m = kwor_dedup(assets, n, asset2pde, pde2asset);
    const int64_t N = p->x_dim;
    job_t J;
    J.assets = assets;
    J.pde2asset = pde2asset;
    J.m = m;
    J.p = p;
    J.xg = (double*)malloc(sizeof(double) * m * (size_t)N);
    J.vg = (double*)malloc(sizeof(double) * m * (size_t)N);
    J.perr = (int32_t*)calloc(m, sizeof(int32_t));
    atomic_init(&J.next, 0);
    if (nthreads < 1) nthreads = 1;
    if ((size_t)nthreads > m) nthreads = (int)m;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
    for (int k = 1; k < nthreads; ++k) pthread_create(&th[k], NULL, worker, &J);
    worker(&J);
    for (int k = 1; k < nthreads; ++k) pthread_join(th[k], NULL);
    free(th);

    int ret = 0;
    for (size_t i = 0; i < n; ++i) {
        const kwor_option* a = &assets[i];
        const size_t pi = asset2pde[i];
        double v;
        const double xs = log(a->s / a->k);
        const double* x = J.xg + pi * (size_t)N;
        if (kwor_value(x, J.vg + pi * (size_t)N, N, xs, &v) != 0) {
            prices[i] = NAN;
            if (status) status[i] = KWOR_OUT_OF_GRID;
            if (!ret) {
                ret = KWOR_OUT_OF_GRID;
                if (err)
                    snprintf(err, errlen,
                             "Fd1d_Pricer::price Fd1d::value: x=%f not in range (%f, %f)", xs,
                             x[0], x[N - 1]);
            }
            continue;
        }
        prices[i] = a->k * v;
        if (status) status[i] = J.perr[pi] ? KWOR_SOLVER_ERROR : KWOR_OK;
    }
    free(J.xg);
    free(J.vg);
    free(J.perr);
    free(asset2pde);
    free(pde2asset);
    return ret;
}

/* Solves one PDE and returns its grids (x and final V), for grid-level parity checks. */
int kwor_fd1d_solve_grid(const kwor_option* a, const kwor_params* p, double* x_out, double* v_out)
{
    const int64_t N = p->x_dim, T = p->t_dim;
    double* buf = (double*)malloc(sizeof(double) * (size_t)(6 * N + T));
    scratch_t s = {buf, buf + N, buf + 2 * N, buf + 3 * N, buf + 4 * N};
    double* payoff = buf + 5 * N;
    double* t = buf + 6 * N;
    const double a0 = -a->r;
    const double ax = a->r - a->q - a->z * a->z / 2;
    const double axx = a->z * a->z / 2;
    kwor_t_grid(a->t, T, t);
    kwor_x_grid(a->z, a->t, p->scale, p->density, p->uniform, N, x_out);
    kwor_payoff(a->w, x_out, N, payoff);
    memcpy(v_out, payoff, sizeof(double) * (size_t)N);
    int e = kwor_solve_one(a0, ax, axx, a->e != 0, p->theta, t, T, x_out, N, payoff, v_out,
                           p->const_dt, &s);
    free(buf);
    return e;
}

/* ---------------------------------------------------------------- Black-Scholes (kwBlackScholes.cpp:27-49) */

static double cdf_normal(double x) { return 0.5 * (1 + erf(x / 1.41421356237309504880)); }

/* European closed form; American options get NaN like the reference. */
void kwor_bs_price(const kwor_option* assets, size_t n, double* prices)
{
    for (size_t i = 0; i < n; ++i) {
        const kwor_option* a = &assets[i];
        if (a->e) {
            prices[i] = NAN;
            continue;
        }
        const double k = a->k, q = a->q, r = a->r, s = a->s, t = a->t, z = a->z;
        const int8_t w = a->w;
        double zt = z * sqrt(t);
        double d1 = 1 / zt * (log(s / k) + (r - q + 0.5 * z * z) * t);
        double d2 = d1 - zt;
        prices[i] = w * (s * cdf_normal(w * d1) * exp(-q * t) - k * cdf_normal(w * d2) * exp(-r * t));
    }
}

/* FD1D-BS control variate (kwFd1d_BlackScholes.cpp:15-42): FD(asset) + BS(euro) - FD(euro). */
int kwor_fd1d_bs_price(const kwor_option* assets, size_t n, const kwor_params* p, int nthreads,
                       double* prices, int32_t* status, char* err, size_t errlen)
{
    int r = kwor_fd1d_price(assets, n, p, nthreads, prices, status, err, errlen);
    if (r) return r;
    kwor_option* euro = (kwor_option*)malloc(sizeof(kwor_option) * (n ? n : 1));
    memcpy(euro, assets, sizeof(kwor_option) * n);
    for (size_t i = 0; i < n; ++i) euro[i].e = 0;
    double* fd = (double*)malloc(sizeof(double) * (n ? n : 1));
    double* bs = (double*)malloc(sizeof(double) * (n ? n : 1));
    r = kwor_fd1d_price(euro, n, p, nthreads, fd, NULL, err, errlen);
    if (!r) {
        kwor_bs_price(euro, n, bs);
        for (size_t i = 0; i < n; ++i) prices[i] += bs[i] - fd[i];
    }
    free(euro);
    free(fd);
    free(bs);
    return r;
}
