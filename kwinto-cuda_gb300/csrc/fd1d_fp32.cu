// fd1d_fp32.cu -- FP32 stepping with FP64-accurate state: one, two, four or eight warps
// per PDE (tuned; at least two for grids of 1025..2048 nodes), the whole PDE on chip (state in
// registers, coefficient tables in shared memory), a partitioned tridiagonal solve
// with a cyclic reduction of the separator system (warp shuffles; shared memory
// across the warps of a PDE).
//
// Numerics.  The reference step B V' = E V (src/Math/kwFd1d.cpp:61-132) is taken in
// delta form,  V' = max(V + d, p)  with  B d = dt A V  (E = B + dt A), so FP32 only
// ever carries the small increment d.  V and the payoff p are float-float pairs
// (hi + lo, ~48 significant bits).  The residual dt A V is formed from differences
// of the pairs, which are exact in FP32, with the operator written as
//     dt A V_j = c1 S_j + c2 (V_{j+1}-V_j) + c3 (V_j-V_{j-1}) + c4 V_j,
//     S_j = (V_{j+1}-V_j) - (V_j-V_{j-1}),
// c1 = dt axx l2, c2 = dt (axx (u2-l2) + ax im), c3 = dt ax im, c4 = dt a0 (the
// reference's inverse spacings, src/Math/kwFd1d.cpp:87-92), so rounding the
// coefficients to FP32 perturbs the PDE's coefficients by ~1e-7 relatively instead
// of breaking the cancellation of the second difference.  The grid, c1..c4 and the
// payoff are computed in FP64 (src/Pricer/kwFd1d.cpp:110-139); the final
// interpolation reads V = hi + lo in FP64.
//
// Solve of B d = r (N_p = 32 W M nodes, lane k owns nodes kM .. kM+M-1):
//   * node kM is a separator s_k; nodes kM+1 .. kM+M-1 are lane k's interior;
//   * interior:  d_I = y - s_k L - s_{k+1} R,  y = B_I^-1 r_I  (a twisted
//     factorisation: eliminated from both ends towards the lane's pivot node kM+M/2;
//     factors and the spikes L, R precomputed once per PDE);
//   * separators: a 32 W-unknown tridiagonal system, solved by parallel cyclic
//     reduction (5 + log2 W levels, multipliers precomputed).
// B, dt and the grid do not change between steps, so all factors are computed once.
//
// Packed pairs.  Each step runs on float2 values with the packed FP32 instructions
// of sm_100 and later (__fadd2_rn, __fmul2_rn, __ffma2_rn: two FP32 operations per
// issued instruction).  A lane's nodes are paired around its pivot P = M/2: nodes P-k
// and P+k share a float2.  The residual, the spike correction and the update are
// per-node work, so any pairing packs them; this one also packs the twisted solve,
// whose two elimination chains walk P-k and P+k in step.
#include <cstdint>
#include <cuda_runtime.h>

#include "fd1d_common.cuh"
#include "fd1d_kernels.h"

namespace kwg {

namespace {

constexpr unsigned kFull = 0xffffffffu;
// Tables, by slot: a lane's M nodes are paired around its pivot row P = M/2 -- slot k
// (k = 1 .. P-1) holds nodes a = P-k and b = P+k, slot 0 holds node 0 (the lane's
// separator) and node P -- so that each step runs on packed FP32 pairs (below).
//   PP  (hi_a, hi_b, lo_a, lo_b)  the payoff as float-float pairs      per lane
//   F0  (l_a, l_b, id_a, id_b)    twisted elimination, inverse pivots
//   F1  (u_a, u_b, sl_a, sl_b)    back substitution, left spike
//   F2  (sr_a, sr_b)              right spike
//   C0  (c1_a, c1_b, c4_a, c4_b), C1 (c2_a, -c3_b, c3_a, -c2_b)   residual coefficients
// Per-lane groups are laid out [slot][lane] (consecutive lanes, conflict-free).  On a
// uniform grid without padded nodes the interior rows of B are the same at every
// node, so
//   * the residual coefficients c1..c4 live in registers (no C0, C1);
//   * every lane but the last has the same interior block B_I, hence the same
//     factors and spikes: F0, F1, F2 are kept once for the group plus once for the
//     last lane (whose block holds the boundary row), [slot][2], read as broadcasts;
//     only the payoff stays per lane.
template <bool kUni>
__host__ __device__ constexpr int f32_fields() { return kUni ? 2 : 11; }  // per-lane floats per node
constexpr int kSharedFields = 5;                                          // l, id, u, sl, sr

struct FF {
    float hi, lo;
};

// hi + lo of a double, both rounded to nearest.
__device__ __forceinline__ FF split(double v)
{
    FF r;
    r.hi = (float)v;
    r.lo = (float)(v - (double)r.hi);
    return r;
}

// (h, l) += d: h takes the rounded sum and l collects its rounding error, computed
// by Fast2Sum (exact when |h| >= |d| or h == 0 -- the increment of a step is small
// next to the value it updates; where it is not, V is near 0 and the loss is an ulp
// of that tiny sum).  The pair is not renormalised: each step adds at most half an
// ulp of h to l, so over a few thousand steps |l| stays within ~2^11 ulp(h), far
// below h, and the differences of neighbouring h that the residual takes stay exact.
__device__ __forceinline__ void ff_acc(float& h, float& l, float d)
{
    const float s = h + d;
    const float e = d - (s - h);
    h = s;
    l += e;
}

// Packed FP32 pairs (two FP32 operations per instruction on sm_100 and later).
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, neg2(b)); }

// ff_acc on two independent float-float values at once.
__device__ __forceinline__ void ff_acc2(float2& h, float2& l, float2 d)
{
    const float2 s = __fadd2_rn(h, d);
    const float2 e = sub2(d, sub2(s, h));
    h = s;
    l = __fadd2_rn(l, e);
}

}  // namespace

// Shared-memory bytes of the lane-exchange area of a W-warp PDE group (W > 1).
template <int W>
__host__ __device__ constexpr int f32_xchg_bytes()
{
    return W == 1 ? 0 : 32 * W * (8 * 4 + 6 * 8) + 16 * 4;
}

// W warps share one PDE (NL = 32 W lanes, lane K owns nodes KM .. KM+M-1).  W == 1
// exchanges lane-boundary values with warp shuffles; W > 1 through shared memory
// (one block barrier per exchange; the separator reduction runs 5 + log2 W levels).
template <int M, bool kUni, int W>
__global__ void __launch_bounds__(32 * W) fd1d_solve_fp32(const PdeBatch b, Fd1dShape sh, double* __restrict__ vout,
                                                          int32_t* __restrict__ pde_status, int* __restrict__ counters)
{
    constexpr int kF = f32_fields<kUni>();
    constexpr int NL = 32 * W;
    constexpr int kLevels = W == 1 ? 5 : W == 2 ? 6 : W == 4 ? 7 : 8;  // log2 of the lanes
    constexpr int P = M / 2;  // pivot row of the twisted interior factorisation
    static_assert(M % 2 == 0, "an even number of nodes per lane: as many rows above the pivot as below");
    static_assert(W == 1 || W == 2 || W == 4 || W == 8, "1, 2, 4 or 8 warps per PDE");
    // Tables (floats): non-uniform grids C0, C1, F0, F1 [P][NL] float4, F2 [P][NL] float2,
    // PP [P][NL] float4; uniform grids PP [P][NL] float4, F0, F1 [P][2] float4, F2 [P][2]
    // float2; then the exchange area (W > 1).
    extern __shared__ float tab[];
    const int k = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int K = threadIdx.x;  // lane of the PDE group
    constexpr int kTabFloats = M * kF * NL + (kUni ? M * kSharedFields * 2 : 0);
    // per-lane groups at [slot * NL + K]; the uniform grid's shared groups at
    // [slot * 2 + c] with c = 1 for the last lane only, computed arithmetically
    // ((K + 1) / NL with NL a power of two) so that the loads stay single loads
    constexpr int kStride = kUni ? 2 : NL;  // elements per slot of the factor groups
    constexpr int kF0 = kUni ? 2 * M * NL : 4 * M * NL;
    constexpr int kPP = kUni ? 0 : 9 * M * NL;
    const int own = kUni ? (K + 1) / NL : K;
    float4* const C0t = reinterpret_cast<float4*>(tab) + K;
    float4* const C1t = reinterpret_cast<float4*>(tab + 2 * M * NL) + K;
    float4* const F0t = reinterpret_cast<float4*>(tab + kF0) + own;
    float4* const F1t = F0t + P * kStride;
    float2* const F2t = reinterpret_cast<float2*>(tab + kF0 + 4 * M * kStride) + own;
    float4* const PPt = reinterpret_cast<float4*>(tab + kPP) + K;
    // uniform grid: lane 0 writes the group's factors, the last lane its own
    const bool writer = !kUni || K == 0 || K == NL - 1;
    // node i of the lane -> its slot and component (0: node P-k or node 0; 1: P+k or P)
    auto slot_of = [](int i) { return i == 0 ? 0 : (i < P ? P - i : i - P); };
    auto comp_of = [](int i) { return i >= P ? 1 : 0; };
    auto part = [](float4& q, int f) -> float& { return reinterpret_cast<float*>(&q)[f]; };
    auto PH = [&](int i) -> float& { return part(PPt[slot_of(i) * NL], comp_of(i)); };
    auto PL = [&](int i) -> float& { return part(PPt[slot_of(i) * NL], 2 + comp_of(i)); };
    auto L = [&](int i) -> float& { return part(F0t[slot_of(i) * kStride], comp_of(i)); };
    auto ID = [&](int i) -> float& { return part(F0t[slot_of(i) * kStride], 2 + comp_of(i)); };
    auto U = [&](int i) -> float& { return part(F1t[slot_of(i) * kStride], comp_of(i)); };
    auto SL = [&](int i) -> float& { return part(F1t[slot_of(i) * kStride], 2 + comp_of(i)); };
    auto SR = [&](int i) -> float& {
        float2& q = F2t[slot_of(i) * kStride];
        return comp_of(i) ? q.y : q.x;
    };
    // residual coefficients of node i; for the b node of a slot c2 and c3 are stored
    // negated and swapped, which lets one packed FMA serve both components (below)
    auto set_c = [&](int i, float c1, float c2, float c3, float c4) {
        float4& q0 = C0t[slot_of(i) * NL];
        float4& q1 = C1t[slot_of(i) * NL];
        if (comp_of(i) == 0) {
            q0.x = c1;
            q0.z = c4;
            q1.x = c2;
            q1.z = c3;
        } else {
            q0.y = c1;
            q0.w = c4;
            q1.w = -c2;
            q1.y = -c3;
        }
    };
    // B_I^-1 v in place on nodes 1 .. M-1 by a twisted factorisation: eliminate from
    // both ends towards node P (two independent chains), solve that row, then
    // substitute back outward (two chains again).  Factors: rows above the pivot
    // (l, id, u) = (l_i, 1/d_i, bu_i/d_i) of the top-down LU; rows below it
    // (m_i, 1/e_i, bl_i/e_i) of the bottom-up elimination; the pivot row
    // (l_P, 1/gamma, m_P).  Scalar form, used by the setup for the spikes; the steps
    // run the same operations on packed pairs.
    auto interior_solve = [&](float (&v)[M]) {
        float f = 0.f, g = 0.f;
#pragma unroll
        for (int jj = 0; jj < P - 1; ++jj) {
            const int it = 1 + jj, ib = M - 1 - jj;
            f = fmaf(-L(it), f, v[it]);
            v[it] = f;
            g = fmaf(-L(ib), g, v[ib]);
            v[ib] = g;
        }
        v[P] = fmaf(-U(P), g, fmaf(-L(P), f, v[P])) * ID(P);
#pragma unroll
        for (int jj = 0; jj < P - 1; ++jj) {
            const int it = P - 1 - jj, ib = P + 1 + jj;
            v[it] = fmaf(-U(it), v[it + 1], v[it] * ID(it));
            v[ib] = fmaf(-U(ib), v[ib - 1], v[ib] * ID(ib));
        }
    };
    const int j0 = K * M;
    float2* x_last = reinterpret_cast<float2*>(tab + kTabFloats);  // [NL] (H, Lo) of each lane's last node
    float2* x_first = x_last + NL;                                  // [NL] of its first node
    float* x_y = reinterpret_cast<float*>(x_first + NL);            // [NL]
    float* x_p0 = x_y + NL;                                         // [NL] x 2: reduction buffers
    float* x_p1 = x_p0 + NL;
    float* x_s = x_p1 + NL;                                         // [NL]
    double* x_d = reinterpret_cast<double*>(x_s + NL);              // [3][NL] setup exchange
    int* x_i = reinterpret_cast<int*>(x_d + 6 * NL);                // [0] PDE, [1..W] status

    for (;;) {
        int pde = 0;
        if constexpr (W == 1) {
            if (k == 0) pde = atomicAdd(&counters[0], 1);
            pde = __shfl_sync(kFull, pde, 0);
        } else {
            if (K == 0) x_i[0] = atomicAdd(&counters[0], 1);
            __syncthreads();
            pde = x_i[0];
            __syncthreads();
        }
        if (pde >= b.m) break;
        const int N = shape_x(sh, pde);
        const int TL = shape_t(sh, pde);  // time levels of this PDE

        // ------------------------------------------------------------ setup
        const double t = b.t[pde], z = b.z[pde], rr = b.r[pde], qq = b.q[pde];
        const int8_t w = b.w[pde];
        const bool amer = b.e[pde] != 0;
        int32_t st = KWG_STATUS_OK;
        if (!(t > 0.) || !(z > 0.) || !isfinite(t) || !isfinite(z) || !isfinite(rr) || !isfinite(qq))
            st = KWG_STATUS_BAD_INPUT;
        Grid g;
        g.init(z, t, sh.scale, sh.density, N, sh.uniform);
        const Coef a = pde_coef(rr, qq, z);
        const double dt = time_step(t, TL);

        // One FP64 pass over this lane's nodes: grid, operator row, residual
        // coefficients, payoff, and the LU of the interior block B_I with the four
        // spike end values the separator system needs (L_1, L_{M-1}, R_1, R_{M-1}).
        // The separator system nearly cancels when theta dt sigma^2/dx^2 is large, so
        // its coefficients come from FP64; the per-step arrays are stored in FP32.
        // uniform grid: interior residual coefficients and the two boundary ones
        float c1u = 0.f, c2u = 0.f, c3u = 0.f, c4u = 0.f, c2b = 0.f, c3b = 0.f;
        if (kUni) {
            const double x0 = g.x(0), x1 = g.x(1), x2 = g.x(2);
            const double iu = 1. / (x2 - x1), im = 1. / (x2 - x0), id = 1. / (x1 - x0);
            const double u2 = 2. * iu * im, l2 = 2. * id * im;
            c1u = (float)(dt * a.axx * l2);
            c2u = (float)(dt * (a.axx * (u2 - l2) + a.ax * im));
            c3u = (float)(dt * a.ax * im);
            c4u = (float)(dt * a.a0);
            c2b = (float)(dt * a.ax / (x1 - x0));
            c3b = (float)(dt * a.ax / (g.x(N - 1) - g.x(N - 2)));
        }
        // uniform grids of full lanes (kUni): operator rows from the exact spacing, as the
        // FP64 solvers build them; the interior row is the same at every interior node,
        // so it is built once (three divisions per node fewer in this FP64 prologue).
        // Compile-time only: the other instantiations keep their register budget.
        constexpr bool uni = kUni;
        const double hxu = uni ? dvd(sub(g.xMax, g.xMin), (double)(N - 1)) : 0.;
        Row row_int{};
        bool have_int = false;
        auto row_at = [&](int j, double xm, double x0, double xp) -> Row {
            if (!uni) return implicit_row(j, N, xm, x0, xp, sh.theta, dt, a.a0, a.ax, a.axx);
            if (j == 0 || j == N - 1) return implicit_row(j, N, -hxu, 0., hxu, sh.theta, dt, a.a0, a.ax, a.axx);
            if (!have_int) row_int = implicit_row(j, N, -hxu, 0., hxu, sh.theta, dt, a.a0, a.ax, a.axx);
            have_int = true;
            return row_int;
        };
        double bla = 0., ba = 1., bua = 0.;          // separator row (node kM)
        double L1 = 0., Llast = 0., R1 = 0., Rlast = 0.;
        double bl_first_f = 0., bu_last_f = 0.;   // first interior bl, last interior bu
        // pivot row P of the twisted factorisation: its row and top multiplier
        double bl_piv = 0., b_piv = 1., bu_piv = 0., l_piv = 0., bu_above = 0.;
        {
            double xm = (j0 > 0 && j0 - 1 < N) ? g.x(j0 - 1) : 0.;
            double x0 = (j0 < N) ? g.x(j0) : 0.;
            // uniform grids: e^x of the lane's nodes by one exp and a product per node
            // (the payoff needs ~1e-15 here, the float-float state's precision)
            double ex = 1., ex_step = 1.;
            if (uni && j0 < N) {
                ex = exp(x0);
                ex_step = exp(hxu);
            }
            double d_prev = 1., id_prev = 1., bu_prev = 0.;
            double pu = 1., pl = 1., sum = 0., fL = 0., bl_first = 0., pr = 1.;
#pragma unroll 1
            for (int i = 0; i < M; ++i) {
                const int j = j0 + i;
                const double xp = (j + 1 < N) ? g.x(j + 1) : 0.;
                double bl = 0., bb = 1., bu = 0.;
                float c1 = 0.f, c2 = 0.f, c3 = 0.f, c4 = 0.f;
                FF p = {0.f, 0.f};
                if (j < N) {
                    const Row rw = row_at(j, xm, x0, xp);
                    bl = rw.bl;
                    bb = rw.b;
                    bu = rw.bu;
                    c4 = (float)(dt * a.a0);
                    if (j == 0) {
                        c2 = (float)(dt * a.ax / (xp - x0));
                    } else if (j == N - 1) {
                        c3 = (float)(dt * a.ax / (x0 - xm));
                    } else {
                        const double iu = 1. / (xp - x0), im = 1. / (xp - xm), id = 1. / (x0 - xm);
                        const double u2 = 2. * iu * im, l2 = 2. * id * im;
                        c1 = (float)(dt * a.axx * l2);
                        c2 = (float)(dt * (a.axx * (u2 - l2) + a.ax * im));
                        c3 = (float)(dt * a.ax * im);
                    }
                    if (uni) {
                        const double v = (w < 0) ? 1. - ex : ex - 1.;
                        if (v > 0.) p = split(v);
                        ex *= ex_step;
                    } else if ((w < 0) ? (x0 < 0.) : (x0 > 0.)) {
                        // the payoff is exactly 0 on the out-of-the-money side: skip exp there
                        p = split(payoff(w, x0));
                    }
                }
                if (!kUni) set_c(i, c1, c2, c3, c4);
                PH(i) = p.hi;
                PL(i) = p.lo;
                if (i == 0) {
                    bla = bl;
                    ba = bb;
                    bua = bu;
                } else {
                    // LU of B_I: l_1 = 0, d_1 = b_1; l_i = bl_i/d_{i-1}, d_i = b_i - l_i bu_{i-1}
                    const double l = (i == 1) ? 0. : bl * id_prev;
                    const double d = (i == 1) ? bb : bb - l * bu_prev;
                    if (!(d != 0.) || !isfinite(d)) st = st == KWG_STATUS_OK ? KWG_STATUS_SOLVER : st;
                    const double idd = 1. / d;
                    const double u = bu * idd;
                    if (writer && i < P) {
                        L(i) = (float)l;
                        ID(i) = (float)idd;
                        U(i) = (float)u;
                    }
                    if (i == P) {
                        bl_piv = bl;
                        b_piv = bb;
                        bu_piv = bu;
                        l_piv = l;
                        bu_above = bu_prev;
                    }
                    // spike ends: L = B_I^-1 (bl_1 e_1), R = B_I^-1 (bu_{M-1} e_{M-1}).
                    // L_1 = bl_1 (B_I^-1)_11 = bl_1 sum_k prod_{i<k}(-u_i) / d_k prod_{2<=i<=k}(-l_i)
                    if (i == 1) {
                        bl_first = bl;
                        fL = bl;
                    } else {
                        pl *= -l;
                        fL *= -l;
                    }
                    sum += pu * idd * pl;
                    if (i == M - 1) {
                        pr = pu;  // prod_{1<=i<=M-2} (-u_i)
                        Llast = fL * idd;
                        Rlast = bu * idd;
                        bu_last_f = bu;
                    }
                    pu *= -u;
                    d_prev = d;
                    id_prev = idd;
                }
                bu_prev = bu;
                xm = x0;
                x0 = xp;
            }
            (void)d_prev;
            L1 = bl_first * sum;
            R1 = Rlast * pr;
            bl_first_f = bl_first;
        }
        // Bottom part of the twisted factorisation of B_I (rows M-1 .. P+1,
        // eliminating upward from the lane's last node) and the pivot row P:
        //   e_i = b_i - m_i bl_{i+1},  m_i = bu_i / e_{i+1}  (m_{M-1} = 0),
        //   gamma = b_P - l_P bu_{P-1} - m_P bl_{P+1}.
        if (writer) {
            double e_next = 1., bl_next = 0.;
            const int jt = j0 + M - 1;
            double xp = (jt + 1 < N) ? g.x(jt + 1) : 0., x0 = (jt < N) ? g.x(jt) : 0.;
#pragma unroll 1
            for (int i = M - 1; i > P; --i) {
                const int j = j0 + i;
                const double xm = (j - 1 < N) ? g.x(j - 1) : 0.;
                double bl = 0., bb = 1., bu = 0.;
                if (j < N) {
                    const Row rw = row_at(j, xm, x0, xp);
                    bl = rw.bl;
                    bb = rw.b;
                    bu = rw.bu;
                }
                const double m = (i == M - 1) ? 0. : bu / e_next;
                const double e = (i == M - 1) ? bb : bb - m * bl_next;
                if (!(e != 0.) || !isfinite(e)) st = st == KWG_STATUS_OK ? KWG_STATUS_SOLVER : st;
                const double ie = 1. / e;
                L(i) = (float)m;
                ID(i) = (float)ie;
                U(i) = (float)(bl * ie);
                e_next = e;
                bl_next = bl;
                xp = x0;
                x0 = xm;
            }
            const double m_piv = (P == M - 1) ? 0. : bu_piv / e_next;
            const double gam = b_piv - l_piv * bu_above - m_piv * bl_next;
            if (!(gam != 0.) || !isfinite(gam)) st = st == KWG_STATUS_OK ? KWG_STATUS_SOLVER : st;
            (void)bl_piv;
            L(P) = (float)l_piv;
            ID(P) = (float)(1. / gam);
            U(P) = (float)m_piv;
            // spikes L = B_I^-1 (bl_1 e_1) and R = B_I^-1 (bu_{M-1} e_{M-1}), by the
            // same FP32 solve the steps use
            float v[M];
#pragma unroll
            for (int i = 0; i < M; ++i) v[i] = 0.f;
            v[1] = (float)bl_first_f;
            interior_solve(v);
#pragma unroll
            for (int i = 1; i < M; ++i) SL(i) = v[i];
#pragma unroll
            for (int i = 0; i < M; ++i) v[i] = 0.f;
            v[M - 1] = (float)bu_last_f;
            interior_solve(v);
#pragma unroll
            for (int i = 1; i < M; ++i) SR(i) = v[i];
        }
        // separator system (FP64) and its cyclic-reduction multipliers (stored FP32)
        float ka[kLevels], kc[kLevels], ib;
        {
            double Lprev, Rprev;
            if constexpr (W == 1) {
                Lprev = __shfl_up_sync(kFull, Llast, 1);
                Rprev = __shfl_up_sync(kFull, Rlast, 1);
            } else {
                x_d[K] = Llast;
                x_d[NL + K] = Rlast;
                __syncthreads();
                Lprev = K > 0 ? x_d[K - 1] : 0.;
                Rprev = K > 0 ? x_d[NL + K - 1] : 0.;
                __syncthreads();
            }
            if (K == 0) Lprev = Rprev = 0.;
            double al = -bla * Lprev;
            double be = ba - bla * Rprev - bua * L1;
            double ga = -bua * R1;
#pragma unroll
            for (int lv = 0; lv < kLevels; ++lv) {
                const int sg = 1 << lv;
                double alm, bem, gam, alp, bep, gap;
                if constexpr (W == 1) {
                    alm = __shfl_up_sync(kFull, al, sg);
                    bem = __shfl_up_sync(kFull, be, sg);
                    gam = __shfl_up_sync(kFull, ga, sg);
                    alp = __shfl_down_sync(kFull, al, sg);
                    bep = __shfl_down_sync(kFull, be, sg);
                    gap = __shfl_down_sync(kFull, ga, sg);
                } else {
                    x_d[K] = al;
                    x_d[NL + K] = be;
                    x_d[2 * NL + K] = ga;
                    __syncthreads();
                    const int im = K - sg >= 0 ? K - sg : K, ip = K + sg < NL ? K + sg : K;
                    alm = x_d[im];
                    bem = x_d[NL + im];
                    gam = x_d[2 * NL + im];
                    alp = x_d[ip];
                    bep = x_d[NL + ip];
                    gap = x_d[2 * NL + ip];
                    __syncthreads();
                }
                if (K - sg < 0) {
                    alm = 0.;
                    bem = 1.;
                    gam = 0.;
                }
                if (K + sg > NL - 1) {
                    alp = 0.;
                    bep = 1.;
                    gap = 0.;
                }
                const double ma = (K - sg < 0) ? 0. : al / bem;
                const double mc = (K + sg > NL - 1) ? 0. : ga / bep;
                ka[lv] = (float)ma;
                kc[lv] = (float)mc;
                const double nal = -ma * alm, nga = -mc * gap;
                be = be - ma * gam - mc * alp;
                al = nal;
                ga = nga;
            }
            if (!(be != 0.) || !isfinite(be)) st = st == KWG_STATUS_OK ? KWG_STATUS_SOLVER : st;
            ib = (float)(1. / be);
        }
        const float blaf = (float)bla, buaf = (float)bua;
        st = __reduce_max_sync(kFull, st);
        if constexpr (W > 1) {
            if (k == 0) x_i[1 + warp] = st;
            __syncthreads();
#pragma unroll
            for (int v = 0; v < W; ++v) st = max(st, x_i[1 + v]);
            __syncthreads();
        }
        const bool run = st == KWG_STATUS_OK;
        if constexpr (kUni) {  // the shared factors written by lane 0 and the last lane
            if constexpr (W == 1)
                __syncwarp();
            else
                __syncthreads();
        }
        // ------------------------------------------------------------ time steps
        // V as float-float pairs by slot, starting at the payoff
        float2 H2[P], L2[P];
#pragma unroll
        for (int kk = 0; kk < P; ++kk) {
            const float4 p = PPt[kk * NL];
            H2[kk] = make_float2(p.x, p.y);
            L2[kk] = make_float2(p.z, p.w);
        }
        // Residual coefficients by component.  Slot k's a node (P-k) has the upward
        // difference D_k.x and the downward D_(k+1).x; its b node (P+k) the upward
        // -D_(k+1).y and the downward -D_k.y (D_k = V_(k-1) - V_k of the slots, below),
        // so (c2_a, -c3_b) multiplies D_k and (c3_a, -c2_b) multiplies D_(k+1).
        const float2 c4u2 = make_float2(c4u, c4u), c1u2 = make_float2(c1u, c1u);
        const float2 c23u = make_float2(c2u, -c3u), c32u = make_float2(c3u, -c2u);
        // the early-exercise floor applies on nodes < N-1: on a grid of full lanes every
        // node but the last lane's node M-1 (slot P-1 .y); elsewhere the lane's nodes
        // below lim
        const int lim = N - 1 - j0;
        for (int step = 1; run && step < TL; ++step) {
            // neighbours across lanes: node -1 is lane K-1's node M-1 (slot P-1 .y), node
            // M is lane K+1's node 0 (slot 0 .x)
            float Hm, Lm, Hp, Lp;
            if constexpr (W == 1) {
                Hm = __shfl_up_sync(kFull, H2[P - 1].y, 1);
                Lm = __shfl_up_sync(kFull, L2[P - 1].y, 1);
                Hp = __shfl_down_sync(kFull, H2[0].x, 1);
                Lp = __shfl_down_sync(kFull, L2[0].x, 1);
            } else {
                x_last[K] = make_float2(H2[P - 1].y, L2[P - 1].y);
                x_first[K] = make_float2(H2[0].x, L2[0].x);
                __syncthreads();
                const float2 pm = x_last[K > 0 ? K - 1 : 0], pp = x_first[K < NL - 1 ? K + 1 : 0];
                Hm = pm.x;
                Lm = pm.y;
                Hp = pp.x;
                Lp = pp.y;
            }
            if (K == 0) Hm = Lm = 0.f;
            if (K == NL - 1) Hp = Lp = 0.f;
            // differences of consecutive slots, D_k = V_(k-1) - V_k (k = 1 .. P), with the
            // pivot in both components before slot 1 and (node 0, node M) after slot P-1:
            // .x = V(P-k+1) - V(P-k), .y = V(P+k-1) - V(P+k); hi and lo parts each exact
            auto diff = [&](int kk, float2& dh, float2& dl) {
                const float2 hu = kk == 1 ? make_float2(H2[0].y, H2[0].y) : H2[kk - 1];
                const float2 lu = kk == 1 ? make_float2(L2[0].y, L2[0].y) : L2[kk - 1];
                const float2 hd = kk == P ? make_float2(H2[0].x, Hp) : H2[kk];
                const float2 ld = kk == P ? make_float2(L2[0].x, Lp) : L2[kk];
                dh = sub2(hu, hd);
                dl = sub2(lu, ld);
            };
            // residual r = dt A V on the slots 1 .. P-1, two nodes per operation
            float2 y2[P];
            float2 dh1, dl1;
            diff(1, dh1, dl1);
            float2 dh = dh1, dl = dl1, d = __fadd2_rn(dh1, dl1);
#pragma unroll
            for (int kk = 1; kk < P; ++kk) {
                float2 dhn, dln;
                diff(kk + 1, dhn, dln);
                const float2 dn = __fadd2_rn(dhn, dln);
                const float2 S = __fadd2_rn(sub2(dh, dhn), sub2(dl, dln));
                float2 c1v = c1u2, c4v = c4u2, c23 = c23u, c32 = c32u;
                if constexpr (!kUni) {
                    const float4 q0 = C0t[kk * NL], q1 = C1t[kk * NL];
                    c1v = make_float2(q0.x, q0.y);
                    c4v = make_float2(q0.z, q0.w);
                    c23 = make_float2(q1.x, q1.y);
                    c32 = make_float2(q1.z, q1.w);
                }
                float2 r = __fmul2_rn(c4v, __fadd2_rn(H2[kk], L2[kk]));
                r = __ffma2_rn(c1v, S, r);
                r = __ffma2_rn(c23, d, r);
                y2[kk] = __ffma2_rn(c32, dn, r);
                dh = dhn;
                dl = dln;
                d = dn;
            }
            // ... and on slot 0, node by node: the pivot P and the separator 0
            float c1a = c1u, c2a = c2u, c3a = c3u, c4a = c4u, c1b = c1u, c2b_ = c2u, c3b_ = c3u, c4b = c4u;
            if constexpr (!kUni) {
                const float4 q0 = C0t[0], q1 = C1t[0];
                c1a = q0.x;
                c4a = q0.z;
                c2a = q1.x;
                c3a = q1.z;
                c1b = q0.y;
                c4b = q0.w;
                c2b_ = -q1.w;
                c3b_ = -q1.y;
            }
            float yP, y0;
            {
                const float hdu = -dh1.y, hdd = dh1.x, ldu = -dl1.y, ldd = dl1.x;
                const float Dup = hdu + ldu, Ddn = hdd + ldd, S = (hdu - hdd) + (ldu - ldd);
                float r = c4b * (H2[0].y + L2[0].y);
                r = fmaf(c1b, S, r);
                r = fmaf(c2b_, Dup, r);
                yP = fmaf(c3b_, Ddn, r);
            }
            {
                const float hdu = dh.x, hdd = H2[0].x - Hm, ldu = dl.x, ldd = L2[0].x - Lm;  // dh = D_P
                const float Dup = hdu + ldu, Ddn = hdd + ldd, S = (hdu - hdd) + (ldu - ldd);
                float r = c4a * (H2[0].x + L2[0].x);
                r = fmaf(c1a, S, r);
                r = fmaf(c2a, Dup, r);
                y0 = fmaf(c3a, Ddn, r);
                // uniform grids: the one-sided boundary rows (no second difference) --
                // node 0 of the first lane, node M-1 of the last
                if (kUni && K == 0) y0 = fmaf(c2b, hdu + ldu, c4u * (H2[0].x + L2[0].x));
            }
            if (kUni && K == NL - 1) {
                if constexpr (P == 1) {
                    yP = fmaf(c3b, dh1.x + dl1.x, c4u * (H2[0].y + L2[0].y));  // node 1 = the pivot
                } else {
                    // node M-1 minus node M-2 (slot P-2 .y; for P = 2 the pivot, slot 0 .y)
                    const float2 dm = sub2(H2[P - 1], H2[P - 2]), lm = sub2(L2[P - 1], L2[P - 2]);
                    y2[P - 1].y = fmaf(c3b, dm.y + lm.y, c4u * (H2[P - 1].y + L2[P - 1].y));
                }
            }
            // interior: twisted elimination, the two chains in one packed operation ...
            float2 F = make_float2(0.f, 0.f);
#pragma unroll
            for (int kk = P - 1; kk >= 1; --kk) {
                const float4 f0 = F0t[kk * kStride];
                F = __ffma2_rn(make_float2(-f0.x, -f0.y), F, y2[kk]);
                y2[kk] = F;
            }
            // ... the pivot row (F holds f_(P-1) and g_(P+1); 0 when P = 1) ...
            const float4 fp0 = F0t[0], fp1 = F1t[0];
            const float2 fp2 = F2t[0];
            yP = fmaf(-fp1.y, F.y, fmaf(-fp0.y, F.x, yP)) * fp0.w;
            // ... and the back substitution outward
            float2 X = make_float2(yP, yP);
#pragma unroll
            for (int kk = 1; kk < P; ++kk) {
                const float4 f0 = F0t[kk * kStride], f1 = F1t[kk * kStride];
                X = __ffma2_rn(make_float2(-f1.x, -f1.y), X, __fmul2_rn(y2[kk], make_float2(f0.z, f0.w)));
                y2[kk] = X;
            }
            // separators: right-hand side, cyclic reduction, back to the interior
            const float y_last = P == 1 ? yP : y2[P - 1].y;   // node M-1
            const float y_first = P == 1 ? yP : y2[P - 1].x;  // node 1
            float ylp;
            if constexpr (W == 1) {
                ylp = __shfl_up_sync(kFull, y_last, 1);
            } else {
                x_y[K] = y_last;
                __syncthreads();
                ylp = x_y[K > 0 ? K - 1 : 0];
            }
            if (K == 0) ylp = 0.f;
            float rho = y0 - blaf * ylp - buaf * y_first;
            if constexpr (W == 1) {
#pragma unroll
                for (int lv = 0; lv < kLevels; ++lv) {
                    const int sg = 1 << lv;
                    const float rm = __shfl_up_sync(kFull, rho, sg);
                    const float rp = __shfl_down_sync(kFull, rho, sg);
                    rho = rho - ka[lv] * rm - kc[lv] * rp;
                }
            } else {
                float* cur = x_p0;
                float* nxt = x_p1;
                cur[K] = rho;
                __syncthreads();
#pragma unroll
                for (int lv = 0; lv < kLevels; ++lv) {
                    const int sg = 1 << lv;
                    const float rm = cur[K - sg >= 0 ? K - sg : K];
                    const float rp = cur[K + sg < NL ? K + sg : K];
                    rho = rho - ka[lv] * rm - kc[lv] * rp;  // ka, kc are 0 past the ends
                    if (lv + 1 < kLevels) {
                        nxt[K] = rho;
                        __syncthreads();
                        float* tmp = cur;
                        cur = nxt;
                        nxt = tmp;
                    }
                }
            }
            const float sv = rho * ib;
            float s1;
            if constexpr (W == 1) {
                s1 = __shfl_down_sync(kFull, sv, 1);
            } else {
                x_s[K] = sv;
                __syncthreads();
                s1 = x_s[K < NL - 1 ? K + 1 : K];
            }
            if (K == NL - 1) s1 = 0.f;
            const float2 ms = make_float2(-sv, -sv), ms1 = make_float2(-s1, -s1);
#pragma unroll
            for (int kk = 1; kk < P; ++kk) {
                const float4 f1 = F1t[kk * kStride];
                const float2 f2 = F2t[kk * kStride];
                y2[kk] = __ffma2_rn(ms1, f2, __ffma2_rn(ms, make_float2(f1.z, f1.w), y2[kk]));
            }
            y2[0] = make_float2(sv, fmaf(-s1, fp2.y, fmaf(-sv, fp1.w, yP)));
            // V += d (float-float), then the early-exercise floor
#pragma unroll
            for (int kk = 0; kk < P; ++kk) {
                ff_acc2(H2[kk], L2[kk], y2[kk]);
                if (amer) {
                    const float4 p = PPt[kk * NL];
                    const float2 e =
                        __fadd2_rn(sub2(H2[kk], make_float2(p.x, p.y)), sub2(L2[kk], make_float2(p.z, p.w)));
                    const bool pa = kUni || (kk == 0 ? 0 : P - kk) < lim;
                    const bool pb = kUni ? !(kk == P - 1 && K == NL - 1) : P + kk < lim;
                    if (e.x < 0.f && pa) {
                        H2[kk].x = p.x;
                        L2[kk].x = p.z;
                    }
                    if (e.y < 0.f && pb) {
                        H2[kk].y = p.y;
                        L2[kk].y = p.w;
                    }
                }
            }
        }
        // ------------------------------------------------------------ result
        double* V = vout + shape_row(sh, pde);
#pragma unroll
        for (int kk = 0; kk < P; ++kk) {
            const int na = j0 + (kk == 0 ? 0 : P - kk), nb = j0 + P + kk;
            if (na < N) V[na] = (double)H2[kk].x + (double)L2[kk].x;
            if (nb < N) V[nb] = (double)H2[kk].y + (double)L2[kk].y;
        }
        if (K == 0) pde_status[pde] = st;
    }
}

// One thread per asset, like fd1d_interp_fp64 but over a [pde][x_dim] array of V.
__global__ void fd1d_interp_rows(const PdeBatch b, const AssetBatch a, Fd1dShape sh, const double* __restrict__ vrow,
                                 const int32_t* __restrict__ pde_status, double* __restrict__ prices,
                                 int32_t* __restrict__ status)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int slot = a.pde[i];
    const int N = shape_x(sh, slot);
    const double s = a.s[i], k = a.k[i];
    int32_t st = pde_status[slot];
    if (!(s > 0.) || !(k > 0.) || !isfinite(s) || !isfinite(k)) st = KWG_STATUS_BAD_INPUT;
    double price = __longlong_as_double(0x7ff8000000000000ll);
    if (st == KWG_STATUS_OK) {
        Grid g;
        g.init(b.z[slot], b.t[slot], sh.scale, sh.density, N, sh.uniform);
        const double xs = log(dvd(s, k));
        int lo = 0, hi = N;
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
            const double* V = vrow + shape_row(sh, slot);
            const double xl = g.x(lo - 1), xh = g.x(lo);
            const double v = dvd(add(mul(sub(xh, xs), V[lo - 1]), mul(sub(xs, xl), V[lo])), sub(xh, xl));
            price = mul(k, v);
        }
    }
    // a solve that left a non-finite value where the price is read is a solver failure
    // (the FP32 path's float-float state overflows beyond ~3.4e38 x K)
    if (st == KWG_STATUS_OK && !isfinite(price)) {
        st = KWG_STATUS_SOLVER;
        price = __longlong_as_double(0x7ff8000000000000ll);
    }
    prices[i] = price;
    if (status) status[i] = st;
}

namespace {

// Resident blocks per SM of fd1d_solve_fp32<M, kUni, W>, set by fd1d_fp32_prepare.
template <int M, bool kUni, int W>
int& per_sm_fp32()
{
    static int v = 1;
    return v;
}

template <int M, bool kUni, int W>
constexpr size_t fp32_smem()
{
    return ((size_t)M * f32_fields<kUni>() * 32 * W + (kUni ? (size_t)M * kSharedFields * 2 : 0)) * sizeof(float) +
           f32_xchg_bytes<W>();
}

template <int M, bool kUni, int W>
void prepare_mu()
{
    const size_t smem = fp32_smem<M, kUni, W>();
    cudaFuncSetAttribute(fd1d_solve_fp32<M, kUni, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fd1d_solve_fp32<M, kUni, W>, 32 * W, smem);
    per_sm_fp32<M, kUni, W>() = per_sm < 1 ? 1 : per_sm;
}

template <int M, int W>
void prepare_m()
{
    prepare_mu<M, false, W>();
    prepare_mu<M, true, W>();
}

template <int M, bool kUni, int W>
int launch_mu(const PdeBatch& b, const AssetBatch& a, const Fd1dShape& sh, double* vout, int32_t* pde_status,
              int* counters, double* prices, int32_t* status, int sms, cudaStream_t stream, const SolveEvents* ev)
{
    const size_t smem = fp32_smem<M, kUni, W>();
    const int per_sm = per_sm_fp32<M, kUni, W>();
    const int blocks = b.m < sms * per_sm ? b.m : sms * per_sm;
    cudaMemsetAsync(counters, 0, 4 * sizeof(int), stream);
    if (ev) cudaEventRecord(ev->start, stream);
    fd1d_solve_fp32<M, kUni, W><<<blocks, 32 * W, smem, stream>>>(b, sh, vout, pde_status, counters);
    if (ev) cudaEventRecord(ev->stop, stream);
    int launches = 1;
    if (a.n > 0) {
        fd1d_interp_rows<<<(a.n + 127) / 128, 128, 0, stream>>>(b, a, sh, vout, pde_status, prices, status);
        ++launches;
    }
    return launches;
}

// The 7-field uniform-grid kernel needs a uniform grid and x_dim == 32 W M for every
// PDE (M >= 2 so that the boundary rows sit in different nodes of a lane).
template <int M, int W>
int launch_m(const PdeBatch& b, const AssetBatch& a, const Fd1dShape& sh, double* vout, int32_t* pde_status,
             int* counters, double* prices, int32_t* status, int sms, cudaStream_t stream, const SolveEvents* ev)
{
    const bool full = sh.pde_x ? sh.full_lanes : sh.x_dim == 32 * W * M;
    if (sh.uniform && full)
        return launch_mu<M, true, W>(b, a, sh, vout, pde_status, counters, prices, status, sms, stream, ev);
    return launch_mu<M, false, W>(b, a, sh, vout, pde_status, counters, prices, status, sms, stream, ev);
}

}  // namespace

void fd1d_fp32_prepare(int)
{
    prepare_m<2, 1>();
    prepare_m<4, 1>();
    prepare_m<8, 1>();
    prepare_m<16, 1>();
    prepare_m<32, 1>();
    prepare_m<2, 2>();
    prepare_m<4, 2>();
    prepare_m<8, 2>();
    prepare_m<16, 2>();
    prepare_m<32, 2>();
    prepare_m<2, 4>();
    prepare_m<4, 4>();
    prepare_m<8, 4>();
    prepare_m<16, 4>();
    prepare_m<2, 8>();
    prepare_m<4, 8>();
    prepare_m<8, 8>();
}

int fd1d_fp32_nodes_per_lane(int x_dim)
{
    int m = 2;
    while (32 * m < x_dim) m *= 2;
    return m <= 64 ? m : -1;
}

size_t fd1d_fp32_work_bytes(int m, int x_dim) { return (size_t)m * x_dim * sizeof(double); }

int fd1d_fp32_launch(const PdeBatch& b, const AssetBatch& a, const Fd1dShape& sh, double* vout, int32_t* pde_status,
                     int* counters, double* prices, int32_t* status, int device, cudaStream_t stream,
                     const SolveEvents* ev)
{
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    // W = 1, 2, 4 or 8 warps per PDE (sh.option_warps), each lane owning M = m1 / W nodes,
    // m1 the nodes per lane of the one-warp layout; at least 2 nodes per lane, and
    // grids of 1025..2048 nodes take at least two warps
    const int m1 = fd1d_fp32_nodes_per_lane(sh.x_dim);
    if (m1 < 0) return -1;
    int w = sh.option_warps == 8 ? 8 : sh.option_warps == 4 ? 4 : sh.option_warps == 2 ? 2 : 1;
    if (m1 == 64 && w < 2) w = 2;
    while (w > 1 && m1 / w < 2) w /= 2;
    const int M = m1 / w;
#define KWG_FP32_LAUNCH(MM, WW) \
    if (M == MM && w == WW) return launch_m<MM, WW>(b, a, sh, vout, pde_status, counters, prices, status, sms, stream, ev)
    KWG_FP32_LAUNCH(2, 1);
    KWG_FP32_LAUNCH(4, 1);
    KWG_FP32_LAUNCH(8, 1);
    KWG_FP32_LAUNCH(16, 1);
    KWG_FP32_LAUNCH(32, 1);
    KWG_FP32_LAUNCH(2, 2);
    KWG_FP32_LAUNCH(4, 2);
    KWG_FP32_LAUNCH(8, 2);
    KWG_FP32_LAUNCH(16, 2);
    KWG_FP32_LAUNCH(32, 2);
    KWG_FP32_LAUNCH(2, 4);
    KWG_FP32_LAUNCH(4, 4);
    KWG_FP32_LAUNCH(8, 4);
    KWG_FP32_LAUNCH(16, 4);
    KWG_FP32_LAUNCH(2, 8);
    KWG_FP32_LAUNCH(4, 8);
    KWG_FP32_LAUNCH(8, 8);
#undef KWG_FP32_LAUNCH
    return -1;
}

}  // namespace kwg
