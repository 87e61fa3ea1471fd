// fd1d_pcr64.cu -- FP64 theta-scheme solve, one warp per PDE, the PDE on chip.
//
// Same step as the streaming kernel (fd1d_fp64.cu):  y = T^-1 V (T = theta B),
// V' = max(y - cV, p) on nodes < N-1 (src/Math/kwFd1d.cpp:61-132), but the 32 lanes
// of a warp share one PDE, so a batch of m options keeps m warps busy instead of
// m/32.  This is the variant for small batches, where the thread-per-option kernel
// cannot fill the GPU; the autotuner picks between them.
//
// Solve of T y = V (N_p = 32 M nodes, lane k owns nodes kM .. kM+M-1; the grid is
// padded to N_p with decoupled identity rows):
//   * node kM is a separator s_k; nodes kM+1 .. kM+M-1 are lane k's interior;
//   * interior:  y_I = z - s_k L - s_{k+1} R,  z = T_I^-1 V_I  (local LU; spikes
//     L = T_I^-1 (Tl_first e_1), R = T_I^-1 (Tu_last e_last));
//   * separators: a 32-unknown tridiagonal system, parallel cyclic reduction over
//     the warp (5 shuffle levels).
// Factors, spikes and the reduction multipliers are computed once per PDE in FP64.
// Per node and step: 6 FP64 operations (forward, backward, two spike terms, scale,
// update); the reduced system adds ~15 per lane.
#include <cstdint>
#include <cuda_runtime.h>

#include "fd1d_common.cuh"
#include "fd1d_kernels.h"

namespace kwg {

namespace {

constexpr unsigned kFull64 = 0xffffffffu;
constexpr int kP64Fields = 6;
// table fields per node, layout [node-in-lane][field][lane]
enum { Q_L = 0, Q_U, Q_ID, Q_SL, Q_SR, Q_P };
// kShared (uniform grid, x_dim == 32 M): every interior row of T is the same (built
// from the exact spacing hx), so every lane but the last -- whose block holds the
// boundary row -- has bit-identical factors and spikes.  Those 5 fields are then
// kept once per PDE plus once for the last lane, [node][field][2], read as
// broadcasts; only the payoff stays per lane ([node][lane]).
constexpr int kP64Shared = 5;

template <int M, bool kShared>
constexpr size_t pcr64_smem()
{
    return (kShared ? (size_t)M * 32 + (size_t)M * kP64Shared * 2 : (size_t)M * kP64Fields * 32) * sizeof(double);
}

}  // namespace

template <int M, bool kHalf, bool kShared>
__global__ void __launch_bounds__(32) fd1d_solve_fp64_pcr(const PdeBatch b, Fd1dShape sh, double* __restrict__ vout,
                                                          int32_t* __restrict__ pde_status,
                                                          int* __restrict__ counters)
{
    extern __shared__ double qtab[];  // [M][kP64Fields][32], or (kShared) [M][32] + [M][5][2]
    const int k = threadIdx.x & 31;
    // this lane's copy of the shared factors: +1 for lane 31 only (arithmetic, so
    // that each access stays one load from one base address)
    double* const qshr = qtab + M * 32 + (k + 1) / 32;
    const bool writer = !kShared || k == 0 || k == 31;
    auto Q = [&](int i, int f) -> double& {
        if constexpr (kShared) {
            if (f == Q_P) return qtab[i * 32 + k];
            return qshr[(i * kP64Shared + f) * 2];
        } else {
            return qtab[(i * kP64Fields + f) * 32 + k];
        }
    };
    const int j0 = k * M;

    for (;;) {
        int pde = 0;
        if (k == 0) pde = atomicAdd(&counters[0], 1);
        pde = __shfl_sync(kFull64, pde, 0);
        if (pde >= b.m) break;
        const int N = shape_x(sh, pde);
        const int T = shape_t(sh, pde);

        // ------------------------------------------------------------ setup (FP64)
        const double t = b.t[pde], z = b.z[pde], rr = b.r[pde], qq = b.q[pde];
        const int8_t w = b.w[pde];
        const bool amer = b.e[pde] != 0;
        int32_t st = KWG_STATUS_OK;
        if (!(t > 0.) || !(z > 0.) || !isfinite(t) || !isfinite(z) || !isfinite(rr) || !isfinite(qq))
            st = KWG_STATUS_BAD_INPUT;
        Grid g;
        g.init(z, t, sh.scale, sh.density, N, sh.uniform);
        const Coef a = pde_coef(rr, qq, z);
        const double dt = time_step(t, T);
        const double hx = sh.uniform ? dvd(sub(g.xMax, g.xMin), (double)(N - 1)) : 0.;

        // rows of T = theta B for this lane's nodes; interior LU as we go
        double tla = 0., tma = 1., tua = 0.;  // separator row
        double tl_first = 0., tu_last = 0.;
        {
            double xm = (j0 > 0 && j0 - 1 < N) ? g.x(j0 - 1) : 0.;
            double x0 = (j0 < N) ? g.x(j0) : 0.;
            double d_prev = 1., tu_prev = 0.;
            // Bit-identical shortcuts of this FP64 prologue: on uniform grids theta x the
            // interior row is built once; elsewhere the row comes from reciprocal spacings
            // carried from node to node (two divisions per node instead of three); no exp
            // where the payoff is +0 (x >= 0 for a put, x <= 0 for a call).
            Row t_int{};
            bool have_int = false;
            double r_d = (!sh.uniform && j0 > 0 && j0 < N) ? dvd(1., sub(x0, xm)) : 0.;
#pragma unroll 1
            for (int i = 0; i < M; ++i) {
                const int j = j0 + i;
                const double xp = (j + 1 < N) ? g.x(j + 1) : 0.;
                double tl = 0., tm = 1., tu = 0., p = 0.;
                double r_u = 0.;
                if (j < N) {
                    auto scaled = [&](const Row& r) {
                        return Row{mul(sh.theta, r.bl), mul(sh.theta, r.b), mul(sh.theta, r.bu)};
                    };
                    Row tr;
                    if (!sh.uniform) {
                        if (j + 1 < N) r_u = dvd(1., sub(xp, x0));
                        const double r_m = (j > 0 && j + 1 < N) ? dvd(1., sub(xp, xm)) : 0.;
                        tr = scaled(implicit_row_r(j, N, r_u, r_m, r_d, sh.theta, dt, a.a0, a.ax, a.axx));
                    } else if (j == 0 || j == N - 1) {
                        tr = scaled(implicit_row(j, N, -hx, 0., hx, sh.theta, dt, a.a0, a.ax, a.axx));
                    } else {
                        if (!have_int) t_int = scaled(implicit_row(j, N, -hx, 0., hx, sh.theta, dt, a.a0, a.ax, a.axx));
                        have_int = true;
                        tr = t_int;
                    }
                    tl = tr.bl;
                    tm = tr.b;
                    tu = tr.bu;
                    p = ((w < 0) ? (x0 < 0.) : (x0 > 0.)) ? payoff(w, x0) : 0.;
                }
                Q(i, Q_P) = p;
                if (i == 0) {
                    tla = tl;
                    tma = tm;
                    tua = tu;
                } else {
                    // T_I = L U: l_1 = 0, d_1 = tm_1; l_i = tl_i/d_{i-1}, d_i = tm_i - l_i tu_{i-1}
                    const double l = (i == 1) ? 0. : tl / d_prev;
                    const double d = (i == 1) ? tm : tm - l * tu_prev;
                    if (!(d != 0.) || !isfinite(d)) st = st == KWG_STATUS_OK ? KWG_STATUS_SOLVER : st;
                    if (writer) {
                        Q(i, Q_L) = l;
                        Q(i, Q_ID) = 1. / d;
                        Q(i, Q_U) = tu / d;  // U = diag(d) (1 + u shift): y_i = f_i/d_i - u_i y_{i+1}
                    }
                    if (i == 1) tl_first = tl;
                    if (i == M - 1) tu_last = tu;
                    d_prev = d;
                }
                tu_prev = tu;
                xm = x0;
                x0 = xp;
                r_d = r_u;
            }
        }
        // spikes L = T_I^-1 (tl_first e_1), R = T_I^-1 (tu_last e_{M-1})
        if (writer) {
            double f = tl_first;
#pragma unroll 1
            for (int i = 1; i < M; ++i) {
                if (i > 1) f = -Q(i, Q_L) * f;
                Q(i, Q_SL) = f * Q(i, Q_ID);
            }
            double nxt = 0.;
#pragma unroll 1
            for (int i = M - 1; i >= 1; --i) {
                const double v = (i == M - 1) ? Q(i, Q_SL) : Q(i, Q_SL) - Q(i, Q_U) * nxt;
                Q(i, Q_SL) = v;
                nxt = v;
            }
            double rn = tu_last * Q(M - 1, Q_ID);
            Q(M - 1, Q_SR) = rn;
#pragma unroll 1
            for (int i = M - 2; i >= 1; --i) {
                rn = -Q(i, Q_U) * rn;
                Q(i, Q_SR) = rn;
            }
        }
        if constexpr (kShared) __syncwarp();  // lane 0's and lane 31's factors
        // separator system and its cyclic-reduction multipliers
        double ka[5], kc[5], ib;
        {
            double Lprev = __shfl_up_sync(kFull64, Q(M - 1, Q_SL), 1);
            double Rprev = __shfl_up_sync(kFull64, Q(M - 1, Q_SR), 1);
            if (k == 0) Lprev = Rprev = 0.;
            double al = -tla * Lprev;
            double be = tma - tla * Rprev - tua * Q(1, Q_SL);
            double ga = -tua * Q(1, Q_SR);
#pragma unroll
            for (int lv = 0; lv < 5; ++lv) {
                const int sg = 1 << lv;
                double alm = __shfl_up_sync(kFull64, al, sg), bem = __shfl_up_sync(kFull64, be, sg),
                       gam = __shfl_up_sync(kFull64, ga, sg);
                double alp = __shfl_down_sync(kFull64, al, sg), bep = __shfl_down_sync(kFull64, be, sg),
                       gap = __shfl_down_sync(kFull64, ga, sg);
                if (k - sg < 0) {
                    alm = 0.;
                    bem = 1.;
                    gam = 0.;
                }
                if (k + sg > 31) {
                    alp = 0.;
                    bep = 1.;
                    gap = 0.;
                }
                const double ma = (k - sg < 0) ? 0. : al / bem;
                const double mc = (k + sg > 31) ? 0. : ga / bep;
                ka[lv] = ma;
                kc[lv] = mc;
                const double nal = -ma * alm, nga = -mc * gap;
                be = be - ma * gam - mc * alp;
                al = nal;
                ga = nga;
            }
            if (!(be != 0.) || !isfinite(be)) st = st == KWG_STATUS_OK ? KWG_STATUS_SOLVER : st;
            ib = 1. / be;
        }
        st = __reduce_max_sync(kFull64, st);
        const bool run = st == KWG_STATUS_OK;
        double V[M];
#pragma unroll
        for (int i = 0; i < M; ++i) V[i] = Q(i, Q_P);

        // ------------------------------------------------------------ time steps
        for (int step = 1; run && step < T; ++step) {
            double y[M];
            // interior: z = T_I^-1 V_I (forward with l, backward with u and 1/d)
            {
                double f = 0.;
#pragma unroll
                for (int i = 1; i < M; ++i) {
                    f = fma(-Q(i, Q_L), f, V[i]);
                    y[i] = f * Q(i, Q_ID);
                }
#pragma unroll
                for (int i = M - 2; i >= 1; --i) y[i] = fma(-Q(i, Q_U), y[i + 1], y[i]);
            }
            // separators
            double zlp = __shfl_up_sync(kFull64, y[M - 1], 1);
            if (k == 0) zlp = 0.;
            double rho = V[0] - tla * zlp - tua * y[1];
#pragma unroll
            for (int lv = 0; lv < 5; ++lv) {
                const int sg = 1 << lv;
                const double rm = __shfl_up_sync(kFull64, rho, sg);
                const double rp = __shfl_down_sync(kFull64, rho, sg);
                rho = rho - ka[lv] * rm - kc[lv] * rp;
            }
            const double s = rho * ib;
            double s1 = __shfl_down_sync(kFull64, s, 1);
            if (k == 31) s1 = 0.;
            y[0] = s;
#pragma unroll
            for (int i = 1; i < M; ++i) y[i] = fma(-s1, Q(i, Q_SR), fma(-s, Q(i, Q_SL), y[i]));
            // update and early-exercise floor
#pragma unroll
            for (int i = 0; i < M; ++i) {
                double vn = kHalf ? y[i] - V[i] : fma(-sh.c, V[i], y[i]);
                if (amer && j0 + i < N - 1) vn = max_floor(vn, Q(i, Q_P));
                V[i] = vn;
            }
        }
        // ------------------------------------------------------------ result
        double* out = vout + shape_row(sh, pde);
#pragma unroll
        for (int i = 0; i < M; ++i)
            if (j0 + i < N) out[j0 + i] = V[i];
        if (k == 0) pde_status[pde] = st;
    }
}

namespace {

// Resident blocks per SM of fd1d_solve_fp64_pcr<M, *, kShared>, set by fd1d_pcr64_prepare.
template <int M, bool kShared>
int& per_sm_pcr64()
{
    static int v = 1;
    return v;
}

template <int M, bool kShared>
void prepare_pcr64_variant()
{
    const size_t smem = pcr64_smem<M, kShared>();
    cudaFuncSetAttribute(fd1d_solve_fp64_pcr<M, true, kShared>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    cudaFuncSetAttribute(fd1d_solve_fp64_pcr<M, false, kShared>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fd1d_solve_fp64_pcr<M, true, kShared>, 32, smem);
    per_sm_pcr64<M, kShared>() = per_sm < 1 ? 1 : per_sm;
}

template <int M>
void prepare_pcr64()
{
    prepare_pcr64_variant<M, false>();
    prepare_pcr64_variant<M, true>();
}

template <int M, bool kShared>
int launch_pcr64_variant(const PdeBatch& b, const AssetBatch& a, const Fd1dShape& sh, double* vout,
                         int32_t* pde_status, int* counters, double* prices, int32_t* status, int sms,
                         cudaStream_t stream, const SolveEvents* ev)
{
    const size_t smem = pcr64_smem<M, kShared>();
    auto kern = sh.c == 1. ? fd1d_solve_fp64_pcr<M, true, kShared> : fd1d_solve_fp64_pcr<M, false, kShared>;
    const int per_sm = per_sm_pcr64<M, kShared>();
    const int blocks = b.m < sms * per_sm ? b.m : sms * per_sm;
    cudaMemsetAsync(counters, 0, 4 * sizeof(int), stream);
    if (ev) cudaEventRecord(ev->start, stream);
    kern<<<blocks, 32, smem, stream>>>(b, sh, vout, pde_status, counters);
    if (ev) cudaEventRecord(ev->stop, stream);
    int launches = 1;
    if (a.n > 0) {
        fd1d_interp_rows<<<(a.n + 127) / 128, 128, 0, stream>>>(b, a, sh, vout, pde_status, prices, status);
        ++launches;
    }
    return launches;
}

// Shared factor tables on uniform grids whose PDEs fill every lane (x_dim == 32 M).
template <int M>
int launch_pcr64(const PdeBatch& b, const AssetBatch& a, const Fd1dShape& sh, double* vout, int32_t* pde_status,
                 int* counters, double* prices, int32_t* status, int sms, cudaStream_t stream, const SolveEvents* ev)
{
    const bool full = sh.pde_x ? sh.full_lanes : sh.x_dim == 32 * M;
    if (sh.uniform && full)
        return launch_pcr64_variant<M, true>(b, a, sh, vout, pde_status, counters, prices, status, sms, stream, ev);
    return launch_pcr64_variant<M, false>(b, a, sh, vout, pde_status, counters, prices, status, sms, stream, ev);
}

}  // namespace

void fd1d_pcr64_prepare(int)
{
    prepare_pcr64<2>();
    prepare_pcr64<4>();
    prepare_pcr64<8>();
    prepare_pcr64<16>();
    prepare_pcr64<32>();
}

int fd1d_pcr64_nodes_per_lane(int x_dim)
{
    int m = 2;
    while (32 * m < x_dim) m *= 2;
    return m <= 32 ? m : -1;
}

int fd1d_pcr64_launch(const PdeBatch& b, const AssetBatch& a, const Fd1dShape& sh, double* vout, int32_t* pde_status,
                      int* counters, double* prices, int32_t* status, int device, cudaStream_t stream,
                      const SolveEvents* ev)
{
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    switch (fd1d_pcr64_nodes_per_lane(sh.x_dim)) {
    case 2: return launch_pcr64<2>(b, a, sh, vout, pde_status, counters, prices, status, sms, stream, ev);
    case 4: return launch_pcr64<4>(b, a, sh, vout, pde_status, counters, prices, status, sms, stream, ev);
    case 8: return launch_pcr64<8>(b, a, sh, vout, pde_status, counters, prices, status, sms, stream, ev);
    case 16: return launch_pcr64<16>(b, a, sh, vout, pde_status, counters, prices, status, sms, stream, ev);
    case 32: return launch_pcr64<32>(b, a, sh, vout, pde_status, counters, prices, status, sms, stream, ev);
    default: return -1;
    }
}

}  // namespace kwg
