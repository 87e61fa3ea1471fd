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
// Layout (option-interleaved, one tile = 32 PDEs = one warp, lane = PDE): one record
// of 10 fields x 32 lanes (2.5 KB) per node,
//     [0] p  [1] n  [2] l  [3] 1/d  |  [4] V  [5] k|g  |  [6] p  [7] u  [8] m  [9] 1/e
// so an UP sweep reads fields 0..5 and a DOWN sweep fields 4..9: one contiguous
// 1.5 KB bulk copy per node and warp, and a lane's field is a 256-byte line's slot.
#include <cstdint>
#include <cuda_runtime.h>

#include "fd1d_common.cuh"
#include "fd1d_kernels.h"
#include "tma.cuh"

namespace kwg {

namespace {

constexpr int kFields = 10;
constexpr int F_UP_P = 0, F_UP_N = 1, F_UP_L = 2, F_UP_ID = 3;
constexpr int F_V = 4, F_W = 5;
constexpr int F_DN_P = 6, F_DN_U = 7, F_DN_M = 8, F_DN_IE = 9;
constexpr int kSweepFields = 6;                         // fields one sweep reads
constexpr uint32_t kStageBytes = kSweepFields * kTile * 8;  // 1536 B

__device__ __forceinline__ size_t rec_idx(int j, int f) { return ((size_t)j * kFields + f) * kTile; }

__device__ __forceinline__ bool finite_nonzero(double v) { return v != 0. && isfinite(v); }

}  // namespace

// One thread per PDE slot.  Builds the grid, payoff and both factorisations of
// theta*B, writes the node records, V = payoff, and runs the first (DOWN)
// elimination on V so that the solve kernel starts with an UP sweep.
__global__ void __launch_bounds__(128) fd1d_setup_fp64(const PdeBatch b, Fd1dShape sh, double* __restrict__ rec,
                                                       int32_t* __restrict__ pde_status)
{
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= b.m_pad) return;
    const int src = slot < b.m ? slot : b.m - 1;  // padding lanes replicate the last PDE
    const int tile = slot / kTile, lane = slot % kTile;
    const int N = sh.x_dim;
    double* R = rec + (size_t)tile * N * kFields * kTile + lane;

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

    // Upward sweep: rows, payoff, LU of theta*B.  Tl, Tu, Tm are parked in the
    // n, m, 1/e slots for the downward sweep.
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
        R[rec_idx(j, F_UP_P)] = p;
        R[rec_idx(j, F_UP_N)] = tl;  // parked
        R[rec_idx(j, F_UP_L)] = l;
        R[rec_idx(j, F_UP_ID)] = id;
        R[rec_idx(j, F_V)] = p;
        R[rec_idx(j, F_DN_P)] = p;
        R[rec_idx(j, F_DN_U)] = mul(tu, id);
        R[rec_idx(j, F_DN_M)] = tu;   // parked
        R[rec_idx(j, F_DN_IE)] = tm;  // parked
        d_prev = d;
        tu_prev = tu;
    }
    // Downward sweep: UL of theta*B, then the first elimination (DOWN) of V = payoff.
    double e_next = 1., tl_next = 0., h_next = 0.;
    for (int j = N - 1; j >= 0; --j) {
        const double tl = R[rec_idx(j, F_UP_N)];
        const double tu = R[rec_idx(j, F_DN_M)];
        const double tm = R[rec_idx(j, F_DN_IE)];
        double m = 0., e = tm;
        if (j < N - 1) {
            m = dvd(tu, e_next);
            e = sub(tm, mul(m, tl_next));
        }
        if (!finite_nonzero(e) && st == KWG_STATUS_OK) st = KWG_STATUS_SOLVER;
        const double ie = dvd(1., e);
        R[rec_idx(j, F_UP_N)] = dvd(tl, e);
        R[rec_idx(j, F_DN_M)] = m;
        R[rec_idx(j, F_DN_IE)] = ie;
        const double p = R[rec_idx(j, F_V)];
        const double h = fma(-m, h_next, p);
        R[rec_idx(j, F_W)] = mul(h, ie);
        e_next = e;
        tl_next = tl;
        h_next = h;
    }
    if (slot < b.m) pde_status[slot] = st;
}

namespace {

// Ring of node stages in shared memory, filled by one bulk copy each.  Visits are
// numbered globally per warp (q); visit q uses stage q % kRing with mbarrier
// parity (q / kRing) & 1.
constexpr int kRing = 16;
constexpr size_t kSolveSmem = kRing * kStageBytes + kRing * sizeof(uint64_t);

struct Ring {
    double* stage;  // kRing * 6 * 32 doubles
    uint64_t* bar;  // kRing mbarriers
};

__device__ __forceinline__ void issue(const Ring& r, uint64_t q, const double* src)
{
    const int s = (int)(q % kRing);
    mbar_arrive_expect_tx(&r.bar[s], kStageBytes);
    bulk_g2s(r.stage + (size_t)s * kSweepFields * kTile, src, kStageBytes, &r.bar[s]);
}

// Bounded wait for visits [from, to) after a timeout: lets copies in flight land in
// shared memory before the block exits.
__device__ void drain(const Ring& r, uint64_t from, uint64_t to)
{
    for (uint64_t q = from; q < to; ++q) mbar_wait(&r.bar[q % kRing], (uint32_t)((q / kRing) & 1));
}

}  // namespace

// Persistent: each warp takes tiles from tile_counter[0] (zeroed by the host before
// the launch) and runs all tDim-1 steps of its 32 PDEs.  One warp per block so the
// scheduler spreads warps evenly over the SMs.  The node records stream through a
// 16-deep shared-memory ring filled by the TMA engine; V and k|g are written back
// with ordinary stores.  If a ring wait expires, tile_counter[1] is set, the warp
// drains its copies in flight and leaves; the interpolation kernel then marks every
// option with KWG_STATUS_DEVICE_TIMEOUT.
//
//   UP sweep   (j = 0..N-1):  y = k - n y_prev;  V = max(y - cV, p);  f = V - l f_prev;  g = f/d
//   DOWN sweep (j = N-1..0):  y = g - u y_prev;  V = max(y - cV, p);  h = V - m h_prev;  k = h/e
__global__ void __launch_bounds__(32) fd1d_solve_fp64(const PdeBatch b, Fd1dShape sh, double* __restrict__ rec,
                                                      int* __restrict__ tile_counter)
{
    extern __shared__ __align__(128) unsigned char smem[];
    Ring ring;
    ring.stage = reinterpret_cast<double*>(smem);
    ring.bar = reinterpret_cast<uint64_t*>(smem + kRing * kStageBytes);
    const int lane = threadIdx.x & 31;
    if (lane == 0) {
        for (int s = 0; s < kRing; ++s) mbar_init(&ring.bar[s], 1);
        fence_mbar_init();
    }
    __syncwarp();

    const int N = sh.x_dim;
    const int ntiles = b.m_pad / kTile;
    const double c = sh.c;
    const int pre = N < kRing ? N : kRing;
    uint64_t q = 0;  // visits consumed so far
    for (;;) {
        int tile = 0;
        if (lane == 0) tile = atomicAdd(&tile_counter[0], 1);
        tile = __shfl_sync(0xffffffffu, tile, 0);
        if (tile >= ntiles) break;
        const int slot = tile * kTile + lane;
        const int src = slot < b.m ? slot : b.m - 1;
        const bool amer = b.e[src] != 0;
        double* R0 = rec + (size_t)tile * N * kFields * kTile;  // tile base (lane 0)
        double* R = R0 + lane;
        for (int pass = 1; pass < sh.t_dim; ++pass) {
            const bool up = pass & 1;
            const int f0 = up ? F_UP_P : F_V;  // first field this sweep reads
            // the previous sweep's stores must be visible to the bulk-copy engine
            fence_proxy_async_global();
            __syncwarp();
            if (lane == 0)
                for (int d = 0; d < pre; ++d) {
                    const int j = up ? d : N - 1 - d;
                    issue(ring, q + d, R0 + rec_idx(j, f0));
                }
            double y = 0., f = 0.;
            for (int i = 0; i < N; ++i) {
                const uint64_t v = q + i;
                const int s = (int)(v % kRing);
                const bool ok = __all_sync(0xffffffffu, mbar_wait(&ring.bar[s], (uint32_t)((v / kRing) & 1)));
                if (!ok) {
                    if (lane == 0) {
                        atomicExch(&tile_counter[1], 1);
                        const int issued = (i + kRing < N) ? i + kRing : N;
                        drain(ring, v, q + issued);
                    }
                    __syncwarp();
                    return;
                }
                const double* st = ring.stage + (size_t)s * kSweepFields * kTile + lane;
                double p, a, bb, sc, vo, w;
                if (up) {
                    p = st[0 * kTile];
                    a = st[1 * kTile];
                    bb = st[2 * kTile];
                    sc = st[3 * kTile];
                    vo = st[4 * kTile];
                    w = st[5 * kTile];
                } else {
                    vo = st[0 * kTile];
                    w = st[1 * kTile];
                    p = st[2 * kTile];
                    a = st[3 * kTile];
                    bb = st[4 * kTile];
                    sc = st[5 * kTile];
                }
                __syncwarp();  // stage s fully read before it is refilled
                if (lane == 0 && i + kRing < N) {
                    const int jn = up ? i + kRing : N - 1 - i - kRing;
                    issue(ring, v + kRing, R0 + rec_idx(jn, f0));
                }
                const int j = up ? i : N - 1 - i;
                y = fma(-a, y, w);
                double vn = fma(-c, vo, y);
                if (amer && j < N - 1) vn = max_floor(vn, p);
                f = fma(-bb, f, vn);
                R[rec_idx(j, F_V)] = vn;
                R[rec_idx(j, F_W)] = f * sc;
            }
            q += N;
        }
    }
}

// One thread per asset: x* = log(s/k), first node x_i >= x* (binary search on the
// grid, the same node the reference's linear search finds, src/Math/kwFd1d.cpp:
// 145-147), linear interpolation (:156), price = k*V (src/Pricer/kwFd1d.cpp:156).
__global__ void fd1d_interp_fp64(const PdeBatch b, const AssetBatch a, Fd1dShape sh,
                                 const double* __restrict__ rec, const int32_t* __restrict__ pde_status,
                                 const int* __restrict__ device_error, double* __restrict__ prices,
                                 int32_t* __restrict__ status)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int slot = a.pde[i];
    const int N = sh.x_dim;
    const double s = a.s[i], k = a.k[i];
    int32_t st = pde_status[slot];
    if (*device_error) st = KWG_STATUS_DEVICE_TIMEOUT;
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
            const double* R = rec + (size_t)tile * N * kFields * kTile + lane;
            const double xl = g.x(lo - 1), xh = g.x(lo);
            const double vl = R[rec_idx(lo - 1, F_V)], vh = R[rec_idx(lo, F_V)];
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
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&cached_max, fd1d_solve_fp64, 32, kSolveSmem);
        if (cached_max < 1) cached_max = 1;
        cached_dev = device;
    }
    const int cap = cached_sms * cached_max;  // one warp per block, one tile per warp at most
    return ntiles < cap ? (ntiles > 0 ? ntiles : 1) : cap;
}

size_t fd1d_fp64_work_bytes(int m_pad, int x_dim) { return (size_t)m_pad * x_dim * kFields * sizeof(double); }

int fd1d_fp64_launch(const PdeBatch& b, const AssetBatch& a, const Fd1dShape& sh, double* rec, int32_t* pde_status,
                     int* counters, double* prices, int32_t* status, int solve_blocks, cudaStream_t stream,
                     const SolveEvents* ev)
{
    int launches = 0;
    fd1d_setup_fp64<<<(b.m_pad + 127) / 128, 128, 0, stream>>>(b, sh, rec, pde_status);
    ++launches;
    cudaMemsetAsync(counters, 0, 2 * sizeof(int), stream);
    if (ev) cudaEventRecord(ev->start, stream);
    fd1d_solve_fp64<<<solve_blocks, 32, kSolveSmem, stream>>>(b, sh, rec, counters);
    if (ev) cudaEventRecord(ev->stop, stream);
    ++launches;
    if (a.n > 0) {
        fd1d_interp_fp64<<<(a.n + 127) / 128, 128, 0, stream>>>(b, a, sh, rec, pde_status, counters + 1, prices,
                                                                 status);
        ++launches;
    }
    return launches;
}

}  // namespace kwg
