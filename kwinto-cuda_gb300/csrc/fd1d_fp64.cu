// fd1d_fp64.cu -- FP64 batched theta-scheme solve, thread per PDE, streaming layout.
//
// Replaces kw::Fd1d::solve / solveOne + kw::solveTridiagonal
// (src/Math/kwFd1d.cpp:11-136, src/Math/kwMath.cpp:16-49) and the grid/payoff build
// of kw::Fd1d_Pricer::price (src/Pricer/kwFd1d.cpp:68-139).
//
// Algorithm.  The reference solves, per time step,  B V' = E V  then projects
// V' = max(V', payoff) on nodes 0..N-2 (src/Math/kwFd1d.cpp:129-132), with
// B = 1 - theta dt A and E = 1 + (1-theta) dt A built row by row from the same
// operator A.  Because B and E come from one A,
//     theta E + (1 - theta) B = 1    =>    B^-1 E = (theta B)^-1 - c,  c = (1-theta)/theta,
// so each step is  y = (theta B)^-1 V,  V' = max(y - c V, payoff).  A, dt and the
// grid do not change between steps, so theta B is factorised once per PDE:
//     LU (eliminate upward):   d_0 = T_0;  l_j = Tl_j/d_{j-1},  d_j = Tm_j - l_j Tu_{j-1}
//     UL (eliminate downward): e_{N-1} = Tm;  m_j = Tu_j/e_{j+1}, e_j = Tm_j - m_j Tl_{j+1}
// and the steps alternate between them, so the back substitution of one step and
// the forward elimination of the next run in ONE sweep over the nodes:
//     UP sweep   (j = 0..N-1):  y_j = k_j - n_j y_{j-1}      (back-substitute UL)
//                               V_j = max(y_j - c V_j, p_j)
//                               f_j = V_j - l_j f_{j-1},  g_j = f_j / d_j   (eliminate LU)
//     DOWN sweep (j = N-1..0):  y_j = g_j - u_j y_{j+1}      (back-substitute LU)
//                               V_j = max(y_j - c V_j, p_j)
//                               h_j = V_j - m_j h_{j+1},  k_j = h_j / e_j   (eliminate UL)
// Four FP64 operations per node and step (the reference does ~40 plus 5 divisions),
// one read and one write of (V, k|g) per node and step, and four coefficients read.
//
// Layout (option-interleaved, one tile = 32 PDEs = one warp, lane = PDE):
//     coef  [tile][node][8][32]: UP block (p, n, l, 1/d), DOWN block (p, u, m, 1/e)
//     state [tile][node][2][32]: (V, k|g)
// so a warp's load of one field at one node is one contiguous 256-byte line.
#include <cstdint>
#include <cuda_runtime.h>

#include "fd1d_common.cuh"
#include "fd1d_kernels.h"

namespace kwg {

namespace {

constexpr int kCoefFields = 8;
constexpr int kStateFields = 2;
// coefficient field slots
constexpr int F_UP_P = 0, F_UP_N = 1, F_UP_L = 2, F_UP_ID = 3;
constexpr int F_DN_P = 4, F_DN_U = 5, F_DN_M = 6, F_DN_IE = 7;

__device__ __forceinline__ size_t coef_idx(int n, int j, int f)
{
    return ((size_t)j * kCoefFields + f) * kTile;
}
__device__ __forceinline__ size_t state_idx(int j, int f) { return ((size_t)j * kStateFields + f) * kTile; }

__device__ __forceinline__ bool finite_nonzero(double v) { return v != 0. && isfinite(v); }

}  // namespace

// One thread per PDE slot.  Builds the grid, payoff and both factorisations of
// theta*B, writes the coefficient records, V = payoff, and runs the first
// (DOWN) elimination on V so that the solve kernel starts with an UP sweep.
__global__ void __launch_bounds__(128) fd1d_setup_fp64(const PdeBatch b, Fd1dShape sh, double* __restrict__ coef,
                                                       double* __restrict__ state, int32_t* __restrict__ pde_status)
{
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= b.m_pad) return;
    const int src = slot < b.m ? slot : b.m - 1;  // padding lanes replicate the last PDE
    const int tile = slot / kTile, lane = slot % kTile;
    const int N = sh.x_dim;
    double* C = coef + (size_t)tile * N * kCoefFields * kTile + lane;
    double* S = state + (size_t)tile * N * kStateFields * kTile + lane;

    const double t = b.t[src], z = b.z[src];
    const int8_t w = b.w[src];
    int32_t st = KWG_STATUS_OK;
    if (!(t > 0.) || !(z > 0.) || !isfinite(t) || !isfinite(z) || !isfinite(b.r[src]) ||
        !isfinite(b.q[src]))
        st = KWG_STATUS_BAD_INPUT;

    Grid g;
    g.init(z, t, sh.scale, sh.density, N, sh.uniform);
    const Coef a = pde_coef(b.r[src], b.q[src], z);
    const double dt = time_step(t, sh.t_dim);
    const double theta = sh.theta;

    // Upward sweep: rows, payoff, LU of theta*B.  Temporarily parks Tl, Tu, Tm in
    // the n, m, 1/e slots for the downward sweep.
    double xm = 0., x0 = g.x(0), xp = g.x(1);
    double d_prev = 1., tu_prev = 0.;
    for (int j = 0; j < N; ++j) {
        if (j > 0) {
            xm = x0;
            x0 = xp;
            xp = (j + 1 < N) ? g.x(j + 1) : 0.;
        }
        const Row r = implicit_row(j, N, xm, x0, xp, theta, dt, a.a0, a.ax, a.axx);
        const double tl = mul(theta, r.bl), tm = mul(theta, r.b), tu = mul(theta, r.bu);
        const double p = payoff(w, x0);
        double l = 0., d = tm;
        if (j > 0) {
            l = dvd(tl, d_prev);
            d = sub(tm, mul(l, tu_prev));
        }
        if (!finite_nonzero(d) && st == KWG_STATUS_OK) st = KWG_STATUS_SOLVER;
        const double id = dvd(1., d);
        C[coef_idx(N, j, F_UP_P)] = p;
        C[coef_idx(N, j, F_UP_N)] = tl;  // parked
        C[coef_idx(N, j, F_UP_L)] = l;
        C[coef_idx(N, j, F_UP_ID)] = id;
        C[coef_idx(N, j, F_DN_P)] = p;
        C[coef_idx(N, j, F_DN_U)] = mul(tu, id);
        C[coef_idx(N, j, F_DN_M)] = tu;   // parked
        C[coef_idx(N, j, F_DN_IE)] = tm;  // parked
        S[state_idx(j, 0)] = p;
        d_prev = d;
        tu_prev = tu;
    }
    // Downward sweep: UL of theta*B, then the first elimination (DOWN) of V = payoff.
    double e_next = 1., tl_next = 0., h_next = 0.;
    for (int j = N - 1; j >= 0; --j) {
        const double tl = C[coef_idx(N, j, F_UP_N)];
        const double tu = C[coef_idx(N, j, F_DN_M)];
        const double tm = C[coef_idx(N, j, F_DN_IE)];
        double m = 0., e = tm;
        if (j < N - 1) {
            m = dvd(tu, e_next);
            e = sub(tm, mul(m, tl_next));
        }
        if (!finite_nonzero(e) && st == KWG_STATUS_OK) st = KWG_STATUS_SOLVER;
        const double ie = dvd(1., e);
        C[coef_idx(N, j, F_UP_N)] = dvd(tl, e);
        C[coef_idx(N, j, F_DN_M)] = m;
        C[coef_idx(N, j, F_DN_IE)] = ie;
        const double p = S[state_idx(j, 0)];
        const double h = fma(-m, h_next, p);
        S[state_idx(j, 1)] = mul(h, ie);
        e_next = e;
        tl_next = tl;
        h_next = h;
    }
    if (slot < b.m) pde_status[slot] = st;
}

namespace {

// UP sweep over one PDE (this lane).  C, S point at the lane's node-0 records.
__device__ __forceinline__ void sweep_up(const double* __restrict__ C, double* __restrict__ S, int N,
                                         double c, bool amer)
{
    double y = 0., f = 0.;
#pragma unroll 4
    for (int j = 0; j < N; ++j) {
        const double* cj = C + coef_idx(N, j, 0);
        double* sj = S + state_idx(j, 0);
        const double p = __ldg(cj + F_UP_P * kTile);
        const double nn = __ldg(cj + F_UP_N * kTile);
        const double l = __ldg(cj + F_UP_L * kTile);
        const double id = __ldg(cj + F_UP_ID * kTile);
        const double v = sj[0];
        const double k = sj[kTile];
        y = fma(-nn, y, k);
        double vn = fma(-c, v, y);
        if (amer && j < N - 1) vn = max_floor(vn, p);
        f = fma(-l, f, vn);
        sj[0] = vn;
        sj[kTile] = f * id;
    }
}

__device__ __forceinline__ void sweep_down(const double* __restrict__ C, double* __restrict__ S, int N,
                                           double c, bool amer)
{
    double y = 0., h = 0.;
#pragma unroll 4
    for (int j = N - 1; j >= 0; --j) {
        const double* cj = C + coef_idx(N, j, 0);
        double* sj = S + state_idx(j, 0);
        const double p = __ldg(cj + F_DN_P * kTile);
        const double u = __ldg(cj + F_DN_U * kTile);
        const double m = __ldg(cj + F_DN_M * kTile);
        const double ie = __ldg(cj + F_DN_IE * kTile);
        const double v = sj[0];
        const double g = sj[kTile];
        y = fma(-u, y, g);
        double vn = fma(-c, v, y);
        if (amer && j < N - 1) vn = max_floor(vn, p);
        h = fma(-m, h, vn);
        sj[0] = vn;
        sj[kTile] = h * ie;
    }
}

}  // namespace

// Persistent: each warp takes tiles from a counter (zeroed by the host before the
// launch) and runs all tDim-1 steps of its 32 PDEs.
__global__ void __launch_bounds__(128) fd1d_solve_fp64(const PdeBatch b, Fd1dShape sh, const double* __restrict__ coef,
                                                       double* __restrict__ state, int* __restrict__ tile_counter)
{
    const int lane = threadIdx.x & 31;
    const int N = sh.x_dim;
    const int ntiles = b.m_pad / kTile;
    const double c = sh.c;
    for (;;) {
        int tile = 0;
        if (lane == 0) tile = atomicAdd(tile_counter, 1);
        tile = __shfl_sync(0xffffffffu, tile, 0);
        if (tile >= ntiles) break;
        const int slot = tile * kTile + lane;
        const int src = slot < b.m ? slot : b.m - 1;
        const bool amer = b.e[src] != 0;
        const double* C = coef + (size_t)tile * N * kCoefFields * kTile + lane;
        double* S = state + (size_t)tile * N * kStateFields * kTile + lane;
        for (int s = 1; s < sh.t_dim; ++s) {
            if (s & 1)
                sweep_up(C, S, N, c, amer);
            else
                sweep_down(C, S, N, c, amer);
        }
    }
}

// One thread per asset: x* = log(s/k), first node x_i >= x* (binary search on the
// grid, the same node the reference's linear search finds, src/Math/kwFd1d.cpp:
// 145-147), linear interpolation (:156), price = k*V (src/Pricer/kwFd1d.cpp:156).
__global__ void fd1d_interp_fp64(const PdeBatch b, const AssetBatch a, Fd1dShape sh,
                                 const double* __restrict__ state, const int32_t* __restrict__ pde_status,
                                 double* __restrict__ prices, int32_t* __restrict__ status)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int slot = a.pde[i];
    const int N = sh.x_dim;
    const double s = a.s[i], k = a.k[i];
    int32_t st = pde_status[slot];
    if (!(s > 0.) || !(k > 0.) || !isfinite(s) || !isfinite(k)) st = KWG_STATUS_BAD_INPUT;
    double price = __longlong_as_double(0x7ff8000000000000ll);
    if (st == KWG_STATUS_OK) {
        Grid g;
        g.init(b.z[slot], b.t[slot], sh.scale, sh.density, N, sh.uniform);
        const double xs = log(dvd(s, k));
        int lo = 0, hi = N;  // first index with x >= xs, in [0, N]
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (g.x(mid) < xs)
                lo = mid + 1;
            else
                hi = mid;
        }
        if (lo == 0 || lo == N) {
            st = KWG_STATUS_OUT_OF_GRID;
        } else {
            const int tile = slot / kTile, lane = slot % kTile;
            const double* S = state + (size_t)tile * N * kStateFields * kTile + lane;
            const double xl = g.x(lo - 1), xh = g.x(lo);
            const double vl = S[state_idx(lo - 1, 0)], vh = S[state_idx(lo, 0)];
            const double v = dvd(add(mul(sub(xh, xs), vl), mul(sub(xs, xl), vh)), sub(xh, xl));
            price = mul(k, v);
        }
    }
    prices[i] = price;
    if (status) status[i] = st;
}

int fd1d_fp64_solve_blocks(int ntiles, int device)
{
    static int cached_dev = -1, cached_max = 0, cached_sms = 0;
    if (cached_dev != device) {
        cudaDeviceGetAttribute(&cached_sms, cudaDevAttrMultiProcessorCount, device);
        cached_max = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&cached_max, fd1d_solve_fp64, 128, 0);
        if (cached_max < 1) cached_max = 1;
        cached_dev = device;
    }
    const int want = (ntiles + 3) / 4;
    return want < cached_sms * cached_max ? (want > 0 ? want : 1) : cached_sms * cached_max;
}

size_t fd1d_fp64_coef_bytes(int m_pad, int x_dim) { return (size_t)m_pad * x_dim * kCoefFields * sizeof(double); }
size_t fd1d_fp64_state_bytes(int m_pad, int x_dim) { return (size_t)m_pad * x_dim * kStateFields * sizeof(double); }

int fd1d_fp64_launch(const PdeBatch& b, const AssetBatch& a, const Fd1dShape& sh, double* coef, double* state,
                     int32_t* pde_status, int* tile_counter, double* prices, int32_t* status, int solve_blocks,
                     cudaStream_t stream, const SolveEvents* ev)
{
    int launches = 0;
    fd1d_setup_fp64<<<(b.m_pad + 127) / 128, 128, 0, stream>>>(b, sh, coef, state, pde_status);
    ++launches;
    cudaMemsetAsync(tile_counter, 0, sizeof(int), stream);
    if (ev) cudaEventRecord(ev->start, stream);
    fd1d_solve_fp64<<<solve_blocks, 128, 0, stream>>>(b, sh, coef, state, tile_counter);
    if (ev) cudaEventRecord(ev->stop, stream);
    ++launches;
    if (a.n > 0) {
        fd1d_interp_fp64<<<(a.n + 127) / 128, 128, 0, stream>>>(b, a, sh, state, pde_status, prices, status);
        ++launches;
    }
    return launches;
}

}  // namespace kwg
