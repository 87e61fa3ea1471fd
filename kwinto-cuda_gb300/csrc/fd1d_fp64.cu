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
// so each step is  y = T^-1 V  (T = theta B),  V' = max(y - cV, p).  A, dt and the
// grid do not change between steps, so T is factorised once per PDE, both ways:
//     LU (eliminate upward):   d_0 = Tm_0,  d_j = Tm_j - Tl_j Tu_{j-1} / d_{j-1}
//     UL (eliminate downward): e_{N-1} = Tm_{N-1},  e_j = Tm_j - Tu_j Tl_{j+1} / e_{j+1}
// and the steps alternate between them, so the back substitution of one step and
// the forward elimination of the next run in ONE sweep over the nodes.  The
// elimination results are kept unscaled and the back substitution carries
// yh = y * pivot, which folds the pivot scaling into the update:
//   UP   (j = 0..N-1):  yh = h - nh*yh_prev    nh = Tl_j/e_{j-1}   (back-substitute UL)
//                       V  = max(yh/e - cV, p)
//                       f  = V - l*f_prev     l  = Tl_j/d_{j-1}   (eliminate LU)
//   DOWN (j = N-1..0):  yh = f - uh*yh_prev    uh = Tu_j/d_{j+1}   (back-substitute LU)
//                       V  = max(yh/d - cV, p)
//                       h  = V - m*h_prev     m  = Tu_j/e_{j+1}   (eliminate UL)
// Three FP64 operations per node and step when theta = 1/2 (c = 1), four otherwise;
// the reference does ~40 plus 5 divisions.  max() runs on the integer pipe.
//
// Uniform grids (density = +inf).  Rows come from the exact spacing h, so interior
// rows are identical; the pivot recurrences d_j, e_j then converge, and once a step
// reproduces its input bit for bit (a fixed point of the rounded recurrence) every
// later pivot equals it: the pivot is frozen with no approximation.  Nodes whose six
// coefficients are all frozen form a middle region where a sweep streams only
// (p, V, state).
//
// Layout (option-interleaved, one tile = 32 PDEs = one warp, lane = PDE), arrays per
// tile and node so that a run of consecutive nodes is contiguous for each sweep:
//     CU [node][3][32]  UP coefficients   (nh, l, 1/e)
//     CD [node][3][32]  DOWN coefficients (uh, m, 1/d)
//     P  [node][32]     payoff
//     S  [node][32][2]  state (V, h|f), one 16-byte load/store per lane
// A sweep streams them in stages of consecutive nodes (one mbarrier, one to three
// bulk copies per stage): 2 G nodes in the middle region, where the coefficients are
// not read, G nodes elsewhere (G = 8, or 16 for launches with few warps per SM).
// Where the payoff of every lane of the tile is exactly +0 (the out-of-the-money side
// of a tile of puts only or calls only; all nodes of European PDEs, which never
// project) the payoff is not read either: the projection there is max(V, +0).
#include <atomic>
#include <cstdint>
#include <mutex>

#include <cuda_runtime.h>

#include "fd1d_common.cuh"
#include "fd1d_kernels.h"
#include "tma.cuh"

namespace kwg {

namespace {

constexpr int kCoef = 3;                                   // coefficients per node and sweep
constexpr int kConsts = 6;                                 // nh l 1/e uh m 1/d in the middle
constexpr uint32_t kNodeCoefBytes = kCoef * kTile * 8;    // 768 B
constexpr uint32_t kNodePBytes = kTile * 8;               // 256 B
constexpr uint32_t kNodeSBytes = 2 * kTile * 8;           // 512 B

__device__ __forceinline__ bool finite_nonzero(double v) { return v != 0. && isfinite(v); }

// Work buffer: CU, CD, P, S (each [tile][node]...), then per-PDE middle constants and
// the middle range.
struct Work {
    double* cu;
    double* cd;
    double* p;
    double* s;
    double* cst;  // [m_pad][6]
    int2* range;  // [m_pad]: first and last node of the middle region (empty: x > y)
    int2* zero;   // [m_pad]: first and last node of the run where the payoff is +0
};

__device__ __forceinline__ Work work_of(double* base, int m_pad, long long node_lanes)
{
    const size_t nodes = (size_t)node_lanes;
    Work w;
    w.cu = base;
    w.cd = w.cu + nodes * kCoef;
    w.p = w.cd + nodes * kCoef;
    w.s = w.p + nodes;
    w.cst = w.s + nodes * 2;
    w.range = reinterpret_cast<int2*>(w.cst + (size_t)m_pad * kConsts);
    w.zero = w.range + m_pad;
    return w;
}

// Per-tile views (lane 0's element of node 0).
struct TileView {
    double* cu;
    double* cd;
    double* p;
    double* s;
};

// Node count and first node-lane of a tile (uniform batches: all tiles alike).
__device__ __forceinline__ void tile_shape(const Fd1dShape& sh, int tile, int& n, long long& off)
{
    if (sh.tiles) {
        n = sh.tiles[tile].n;
        off = sh.tiles[tile].off;
    } else {
        n = sh.x_dim;
        off = (long long)tile * sh.x_dim * kTile;
    }
}

__device__ __forceinline__ TileView tile_view(const Work& w, long long off)
{
    TileView v;
    const size_t base = (size_t)off;
    v.cu = w.cu + base * kCoef;
    v.cd = w.cd + base * kCoef;
    v.p = w.p + base;
    v.s = w.s + base * 2;
    return v;
}

}  // namespace

namespace {

// A correctly rounded division with a one-entry cache: on a uniform grid the frozen
// middle region divides the same operands (by their bits) at every node, and the
// cache returns the quotient the division gave the first time -- the same bits.
struct DivMemo {
    long long x = 0, y = 0;
    double q = 0.;
    bool valid = false;
    __device__ __forceinline__ double operator()(double a, double b)
    {
        const long long xa = __double_as_longlong(a), yb = __double_as_longlong(b);
        if (!valid || xa != x || yb != y) {
            x = xa;
            y = yb;
            q = dvd(a, b);
            valid = true;
        }
        return q;
    }
};

// The setup of one PDE slot.  cw, cl: the width of the tile's coefficient and payoff
// records and this slot's index in them -- kTile and the lane, or in twin tiles 16 and
// lane / 2 (one record per twin pair).
// It is FP64-pipe bound (divisions, the payoff's exp).  On a uniform grid it computes
// the interior row once and divides through one-entry caches; on other grids it builds
// the rows from reciprocal spacings carried from node to node; it skips exp where the
// payoff is +0 (x >= 0 for a put, x <= 0 for a call: 1 - e^x <= 0, e^x - 1 <= 0).  All
// bit-identical to evaluating every node.
__device__ __forceinline__ void setup_slot(const PdeBatch& b, const Fd1dShape& sh, const Work& wk, const TileView& tv,
                                           int slot, int src, int lane, int N, int cw, int cl,
                                           int32_t* __restrict__ pde_status)
{
    auto CU = [&](int j, int f) -> double& { return tv.cu[((size_t)j * kCoef + f) * cw + cl]; };
    auto CD = [&](int j, int f) -> double& { return tv.cd[((size_t)j * kCoef + f) * cw + cl]; };
    auto P = [&](int j) -> double& { return tv.p[(size_t)j * cw + cl]; };
    auto S = [&](int j, int f) -> double& { return tv.s[((size_t)j * kTile + lane) * 2 + f]; };

    const double t = b.t[src], z = b.z[src];
    const int8_t w = b.w[src];
    int32_t st = KWG_STATUS_OK;
    if (!(t > 0.) || !(z > 0.) || !isfinite(t) || !isfinite(z) || !isfinite(b.r[src]) ||
        !isfinite(b.q[src]))
        st = KWG_STATUS_BAD_INPUT;

    Grid g;
    g.init(z, t, sh.scale, sh.density, N, sh.uniform);
    const Coef a = pde_coef(b.r[src], b.q[src], z);
    const double dt = time_step(t, shape_t(sh, src));
    const double theta = sh.theta;
    // uniform grids: rows from the exact spacing, so interior rows are identical
    const double hx = sh.uniform ? dvd(sub(g.xMax, g.xMin), (double)(N - 1)) : 0.;

    // Upward pass: rows, payoff, LU pivots d_j.  Tl is parked in CU.nh; d_j, Tu, Tm
    // in CD (uh, m, 1/d) for the downward pass.
    double xm = 0., x0 = g.x(0), xp = g.x(1);
    double d_prev = 1., tu_prev = 0.;
    bool lu_frozen = false;
    int lu_freeze = N;  // first j whose d_j was frozen
    Row t_int;          // uniform grids: theta x the interior row (the same at every interior node)
    bool have_int = false;
    DivMemo div_l;      // tl / d_prev
    double r_d = 0.;    // other grids: 1 / (x_j - x_{j-1}), the previous node's 1 / (x_{j+1} - x_j)
    for (int j = 0; j < N; ++j) {
        if (j > 0) {
            xm = x0;
            x0 = xp;
            xp = (j + 1 < N) ? g.x(j + 1) : 0.;
        }
        auto scaled = [&](const Row& r) { return Row{mul(theta, r.bl), mul(theta, r.b), mul(theta, r.bu)}; };
        Row tr;
        if (!sh.uniform) {
            const double r_u = j + 1 < N ? dvd(1., sub(xp, x0)) : 0.;
            const double r_m = (j > 0 && j + 1 < N) ? dvd(1., sub(xp, xm)) : 0.;
            tr = scaled(implicit_row_r(j, N, r_u, r_m, r_d, theta, dt, a.a0, a.ax, a.axx));
            r_d = r_u;
        } else if (j == 0 || j == N - 1) {
            tr = scaled(implicit_row(j, N, -hx, 0., hx, theta, dt, a.a0, a.ax, a.axx));
        } else {
            if (!have_int) t_int = scaled(implicit_row(j, N, -hx, 0., hx, theta, dt, a.a0, a.ax, a.axx));
            have_int = true;
            tr = t_int;
        }
        const double tl = tr.bl, tm = tr.b, tu = tr.bu;
        const double p = ((w < 0) ? (x0 < 0.) : (x0 > 0.)) ? payoff(w, x0) : 0.;
        const double l = j > 0 ? div_l(tl, d_prev) : 0.;
        double d = tm;
        if (j > 0) {
            if (lu_frozen && j < N - 1) {
                d = d_prev;  // checked when it was computed
            } else {
                d = sub(tm, mul(l, tu_prev));
                // a fixed point: with identical interior rows every later d_j equals it
                if (sh.uniform && j >= 3 && j < N - 1 && d == d_prev) {
                    lu_frozen = true;
                    lu_freeze = j;
                    d = d_prev;
                }
                if (!finite_nonzero(d) && st == KWG_STATUS_OK) st = KWG_STATUS_SOLVER;
            }
        } else if (!finite_nonzero(d) && st == KWG_STATUS_OK) {
            st = KWG_STATUS_SOLVER;
        }
        CU(j, 0) = tl;  // parked
        CU(j, 1) = l;
        P(j) = p;
        S(j, 0) = p;
        CD(j, 0) = d;   // parked
        CD(j, 1) = tu;  // parked
        CD(j, 2) = tm;  // parked
        d_prev = d;
        tu_prev = tu;
    }
    // Downward pass: UL pivots e_j; final coefficients; first elimination of V = p.
    double e_next = 1., tl_next = 0., h_next = 0., d_next = 1.;
    bool ul_frozen = false;
    int ul_freeze = -1;  // first j (from the top) whose e_j was frozen
    DivMemo div_m, div_nh, div_ie, div_uh, div_id;
    for (int j = N - 1; j >= 0; --j) {
        const double tl = CU(j, 0), d = CD(j, 0), tu = CD(j, 1), tm = CD(j, 2);
        double e = tm, m = 0.;
        bool fresh = true;  // e computed here (not the frozen value, checked before)
        if (j < N - 1) {
            m = div_m(tu, e_next);
            if (ul_frozen && j > 0) {
                e = e_next;
                fresh = false;
            } else {
                e = sub(tm, mul(m, tl_next));
                if (sh.uniform && j <= N - 4 && j > 0 && e == e_next) {
                    ul_frozen = true;
                    ul_freeze = j;
                    e = e_next;
                }
            }
        }
        if (fresh && !finite_nonzero(e) && st == KWG_STATUS_OK) st = KWG_STATUS_SOLVER;
        // row j+1's nh = Tl_{j+1} / e_j, written now that e_j is known
        if (j < N - 1) CU(j + 1, 0) = div_nh(tl_next, e);
        CU(j, 2) = div_ie(1., e);
        CD(j, 0) = j < N - 1 ? div_uh(tu, d_next) : 0.;
        CD(j, 1) = m;
        CD(j, 2) = div_id(1., d);
        const double h = fma(-m, h_next, P(j));
        S(j, 1) = h;
        e_next = e;
        tl_next = tl;
        h_next = h;
        d_next = d;
    }
    CU(0, 0) = 0.;  // Tl_0 = 0

    // Middle region: nodes whose coefficients (built from d and e at j-1..j+1 and
    // interior rows j-1..j+1) are all frozen.
    int lo = N, hi = -1;
    if (sh.uniform && lu_frozen && ul_frozen) {
        lo = max(lu_freeze + 1, 2);
        hi = min(ul_freeze - 1, N - 3);
    }
    if (lo <= hi) {
        const int mid = (lo + hi) / 2;
        double* c = wk.cst + (size_t)slot * kConsts;
        c[0] = CU(mid, 0);
        c[1] = CU(mid, 1);
        c[2] = CU(mid, 2);
        c[3] = CD(mid, 0);
        c[4] = CD(mid, 1);
        c[5] = CD(mid, 2);
    }
    wk.range[slot] = make_int2(lo, hi);
    // payoff-free run: the projection never reads P of a European PDE; an American
    // put's payoff is +0 on a top run of nodes (x >= 0), a call's on a bottom run
    int zl = 0, zh = N - 1;
    if (b.e[src] != 0) {
        if (w < 0) {
            zl = N;
            while (zl > 0 && __double_as_longlong(P(zl - 1)) == 0) --zl;
        } else {
            zh = -1;
            while (zh < N - 1 && __double_as_longlong(P(zh + 1)) == 0) ++zh;
        }
    }
    wk.zero[slot] = make_int2(zl, zh);
    if (slot < b.m) pde_status[slot] = st;
}

}  // namespace

// One thread per PDE slot.  Builds the grid, payoff and both factorisations of
// theta*B, writes CU, CD, P, S (V = payoff), the middle-region constants, and runs
// the first (DOWN) elimination on V so that the solve starts with an UP sweep.
__global__ void __launch_bounds__(128) fd1d_setup_fp64(const PdeBatch b, Fd1dShape sh, double* __restrict__ base,
                                                       int32_t* __restrict__ pde_status)
{
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= b.m_pad) return;  // whole warps: m_pad is a multiple of the tile
    const int src = slot < b.m ? slot : b.m - 1;  // padding lanes replicate the last PDE
    const int tile = slot / kTile, lane = slot % kTile;
    int N;
    long long toff;
    tile_shape(sh, tile, N, toff);
    const Work wk = work_of(base, b.m_pad, sh.node_lanes);
    const TileView tv = tile_view(wk, toff);
    const bool twin = tile < sh.twin_tiles;
    // in a twin tile the odd lane (the European copy) has the same operator, payoff and
    // first elimination as the American PDE before it: it copies them below
    const bool copy = twin && (lane & 1);
    if (!copy) setup_slot(b, sh, wk, tv, slot, src, lane, N, twin ? kTile / 2 : kTile, twin ? lane >> 1 : lane,
                          pde_status);
    if (twin) {
        __syncwarp();
        if (copy) {
            double2* sv = reinterpret_cast<double2*>(tv.s);
            for (int j = 0; j < N; ++j) sv[(size_t)j * kTile + lane] = sv[(size_t)j * kTile + lane - 1];
            for (int c = 0; c < kConsts; ++c) wk.cst[(size_t)slot * kConsts + c] = wk.cst[(size_t)(slot - 1) * kConsts + c];
            wk.range[slot] = wk.range[slot - 1];
            wk.zero[slot] = make_int2(0, N - 1);  // European: never projects
            if (slot < b.m) pde_status[slot] = pde_status[slot - 1];
        }
    }
}

namespace {

// Ring of stage slots in shared memory; a slot holds G consecutive nodes of one sweep
// -- coefficients [G][3][32], payoff [G][32], state [G][32][2] -- or, in the middle
// region, 2 G nodes of payoff and state (wide stages).  Stage visits are numbered per
// warp (q); visit q uses slot q % kRing with mbarrier parity (q / kRing) & 1.
// Small stages (G = 8): 12 KB slots, double-buffered: 24 KB per warp keeps >= 7
// single-warp blocks per SM (the 1024 tiles of a 32768-option batch in one wave).
// Measured on the 32768-option 1024 x 1024 batch with uniform stages (launch ms,
// nodes x ring): 4x4 246, 6x3 236, 7x2 223, 8x2 219, 10x2 401 (6 blocks per SM: a
// second wave), 2x8 314; 16-node middle stages in the same slots then 199.
// Big stages (G = 16): 24 KB slots, 48 KB per warp, for launches that cap the
// residency (one 4-warp block per SM: one warp per scheduler).  Each stage boundary
// (mbarrier wait, fence, warp barrier, refill) stalls the warp's FMA chain, and a
// warp alone on its scheduler has no other warp to fill that time: a lone warp on
// 2048-node grids takes 261 cycles per node-step with big stages against 291 with
// small ones.  The stage is loaded into registers in chunks of 8 (coefficient
// stages) or 16 (wide stages) nodes, so the register arrays stay those of the small
// stages.
constexpr int kRing = 2;
template <bool kBig>
struct Geo {
    static constexpr int kGroup = kBig ? 16 : 8;  // nodes of a coefficient stage
    static constexpr int kWide = 2 * kGroup;      // nodes of a wide (middle-region) stage
    static constexpr int kSubC = 8, kSubW = 16;   // nodes per register chunk
    static constexpr uint32_t kStageCoef = kGroup * kNodeCoefBytes;
    static constexpr uint32_t kStageP = kGroup * kNodePBytes;
    static constexpr uint32_t kStageBytes = kStageCoef + kStageP + kGroup * kNodeSBytes;
    static constexpr uint32_t kWideP = kWide * kNodePBytes;  // wide stage: payoff [0, kWideP), state after it
    // one warp's ring and mbarriers, rounded so the next warp's stages stay aligned
    static constexpr size_t kSolveSmem = (kRing * kStageBytes + kRing * sizeof(uint64_t) + 127) / 128 * 128;
    static_assert(kWideP + kWide * kNodeSBytes == kStageBytes, "a wide stage fills one slot");
    static_assert(kGroup % kSubC == 0 && kWide % kSubW == 0, "whole register chunks");
};
constexpr int kMaxBlockWarps = 4;
// share of the L2 given to the state lines at the sweep ends (evict-last)
constexpr double kKeepShare = 0.5;

struct Ring {
    unsigned char* stage;  // kRing * kStageBytes
    uint64_t* bar;         // kRing mbarriers
};

// A stage skips the coefficients when all its nodes lie in the middle region, and
// the payoff when all its nodes lie in the tile's payoff-free run (same test).
__device__ __forceinline__ bool stage_compact(int first, int count, int lo, int hi)
{
    return first >= lo && first + count - 1 <= hi;
}

// The tile's node ranges: middle region [lo, hi], payoff-free run [zlo, zhi].
struct Ranges {
    int lo, hi, zlo, zhi;
};

// L2 policies of a sweep: the state stores of its last keep_n nodes -- the first the
// next sweep, which runs the other way, reads back -- are kept in L2 (evict-last);
// everything else streams (evict-first).  keep_n == 0: no preference.
struct Hints {
    uint64_t keep, stream;
    int keep_n;
};

// Wide stages: in the middle region a stage needs no coefficients, so the same slot
// holds 2 G nodes -- payoff [0, kWideP), state after it -- instead of G nodes with
// coefficients [0, kStageCoef), payoff, state.  Half the stage overhead (mbarrier
// wait, warp sync, refill) per node where most nodes are.

// A stage of a sweep: nodes [first, first + count), ascending in memory.
struct Stage {
    int first, count;
    bool wide;     // kWide middle-region nodes in the wide layout
    bool compact;  // no coefficients: all nodes in the middle region
    bool pfree;    // no payoff: all nodes in the payoff-free run
};

// The stage starting at cursor `cur` (kUp: its lowest node, else its highest).  Wide
// where kWide nodes from the cursor lie in the middle region; else kGroup nodes, fewer
// only at the sweep's end.  Producer and consumer walk the same sequence.
template <bool kUp, bool kBig>
__device__ __forceinline__ Stage stage_at(int cur, int N, const Ranges& rg)
{
    constexpr int kGroup = Geo<kBig>::kGroup, kWide = Geo<kBig>::kWide;
    Stage s;
    if (kUp) {
        s.wide = cur >= rg.lo && cur + kWide - 1 <= rg.hi;
        s.first = cur;
        s.count = s.wide ? kWide : min(kGroup, N - cur);
    } else {
        s.wide = cur - kWide + 1 >= rg.lo && cur <= rg.hi;
        s.count = s.wide ? kWide : min(kGroup, cur + 1);
        s.first = cur - s.count + 1;
    }
    s.compact = s.wide || stage_compact(s.first, s.count, rg.lo, rg.hi);
    s.pfree = stage_compact(s.first, s.count, rg.zlo, rg.zhi);
    return s;
}

template <bool kUp>
__device__ __forceinline__ int sweep_first(int N)
{
    return kUp ? 0 : N - 1;
}

template <bool kUp>
__device__ __forceinline__ bool sweep_done(int cur, int N)
{
    return kUp ? cur >= N : cur < 0;
}

template <bool kUp>
__device__ __forceinline__ int stage_after(int cur, const Stage& s)
{
    return kUp ? cur + s.count : cur - s.count;
}

// Twin tiles hold one coefficient and payoff record per twin pair: 16 entries per node
// where other tiles hold 32.
template <bool kTwin>
__host__ __device__ constexpr int rec_width() { return kTwin ? kTile / 2 : kTile; }

// Bytes a stage moves: its bulk reads plus the state stores.
__device__ __forceinline__ unsigned long long stage_bytes(const Stage& s, bool twin)
{
    const unsigned long long rec = (s.pfree ? 0 : kNodePBytes) + (s.compact ? 0 : kNodeCoefBytes);
    return (unsigned long long)s.count * (2 * kNodeSBytes + (twin ? rec / 2 : rec));
}

// Issues stage visit q for stage sg of this tile.  Twin tiles copy half-width
// coefficient and payoff records into the front of the same slot areas.
template <bool kUp, bool kTwin, bool kBig>
__device__ __forceinline__ void issue(const Ring& r, uint32_t q, const TileView& tv, const Stage& sg, uint64_t pol)
{
    using G = Geo<kBig>;
    constexpr uint32_t kStageBytes = G::kStageBytes, kStageCoef = G::kStageCoef, kStageP = G::kStageP,
                       kWideP = G::kWideP;
    constexpr int kW = rec_width<kTwin>();
    const int s = (int)(q % kRing);
    unsigned char* st = r.stage + (size_t)s * kStageBytes;
    const uint32_t cb = sg.compact ? 0u : sg.count * (uint32_t)(kCoef * kW * 8);
    const uint32_t pb = sg.pfree ? 0u : sg.count * (uint32_t)(kW * 8), sb = sg.count * kNodeSBytes;
    const uint32_t p_off = sg.wide ? 0u : kStageCoef, s_off = sg.wide ? kWideP : kStageCoef + kStageP;
    mbar_arrive_expect_tx(&r.bar[s], cb + pb + sb);
    if (cb) bulk_g2s_hint(st, (kUp ? tv.cu : tv.cd) + (size_t)sg.first * kCoef * kW, cb, &r.bar[s], pol);
    if (pb) bulk_g2s_hint(st + p_off, tv.p + (size_t)sg.first * kW, pb, &r.bar[s], pol);
    bulk_g2s_hint(st + s_off, tv.s + (size_t)sg.first * kTile * 2, sb, &r.bar[s], pol);
}

// The refilling side of a sweep, run by lane 0: the next stage to issue and its
// visit number.
template <bool kUp, bool kTwin, bool kBig>
struct Producer {
    int cur;
    uint32_t next;
    __device__ __forceinline__ void refill(const Ring& ring, const TileView& tv, int N, const Ranges& rg, uint64_t pol)
    {
        if (sweep_done<kUp>(cur, N)) return;
        const Stage sg = stage_at<kUp, kBig>(cur, N, rg);
        issue<kUp, kTwin, kBig>(ring, next, tv, sg, pol);
        cur = stage_after<kUp>(cur, sg);
        ++next;
    }
};

// Bounded wait for stage visits [from, to) after a timeout: lets copies in flight
// land in shared memory before the block exits.
__device__ void drain(const Ring& r, uint32_t from, uint32_t to)
{
    for (uint32_t q = from; q < to; ++q) mbar_wait(&r.bar[q % kRing], (q / kRing) & 1u);
}

// The node-steps of one stage held in registers (kG nodes, processing order): the
// elimination recurrence yh, the new value with the early-exercise floor, the
// second recurrence f, and the 16-byte (value, f) store of each node.
template <bool kUp, bool kHalf, int kG>
__device__ __forceinline__ void stage_steps(const double* ra, const double* rb, const double* rs, const long long* rp,
                                            const double* rv, const double* rw, int first, double c, bool active,
                                            double2* sout, uint64_t pol, double& yh, double& f)
{
#pragma unroll
    for (int k = 0; k < kG; ++k) {
        const int j = kUp ? first + k : first + kG - 1 - k;
        yh = fma(-ra[k], yh, rw[k]);
        const double vs = kHalf ? fma(rs[k], yh, -rv[k]) : fma(rs[k], yh, -c * rv[k]);
        // the early-exercise floor as one signed 64-bit max (rp: the payoff's bits, or
        // those of -0 where the floor does not apply, which no value falls below)
        const double vn = __longlong_as_double(max(__double_as_longlong(vs), rp[k]));
        f = fma(-rb[k], f, vn);
        if (active) st_global_f64x2_hint(reinterpret_cast<double*>(sout + (size_t)j * kTile), vn, f, pol);
    }
}

// The floor operand of node j: the payoff's bits where the reference projects
// (American PDEs, nodes 0 .. N-2), else those of -0 (the smallest signed 64-bit
// pattern a double has), so that the max leaves the value unchanged.
__device__ __forceinline__ long long floor_bits(double p, bool amer, int j, int N)
{
    return (amer && j < N - 1) ? __double_as_longlong(p) : (long long)0x8000000000000000ull;
}

// The L2 policy of a stage's state stores: evict-last when the stage reaches into the
// sweep's last keep_n nodes (read back first by the next sweep), evict-first otherwise.
template <bool kUp>
__device__ __forceinline__ uint64_t stage_policy(int first, int count, int N, const Hints& hz)
{
    const bool keep = kUp ? first + count - 1 >= N - hz.keep_n : first < hz.keep_n;
    return keep ? hz.keep : hz.stream;
}

// One full G-node stage: loads it into registers (in chunks of kSubC nodes), runs its
// node-steps, then lets lane 0 refill the slot.  The refill is a bulk copy (async proxy) into memory the
// lanes have just read (generic proxy): every lane fences its reads before the warp
// barrier that precedes the refill.  Refilling after the node-steps instead of
// before them also keeps lane 0's issue work off the start of the FMA chain (on the
// 32768-option 1024 x 1024 batch: 186 ms fenced, 187 ms with an unfenced refill
// ahead of the node-steps, which raced).  kCompact: the stage lies in the middle
// region (coefficients ca, cb, cs).  No per-node guard: the unrolled stage is one
// block the scheduler interleaves across nodes.
template <bool kUp, bool kHalf, bool kCompact, bool kTwin, bool kBig>
__device__ __forceinline__ void stage_body(const Ring& ring, const TileView& tv, Producer<kUp, kTwin, kBig>& prod,
                                           int N, const Ranges& rg, int first, bool pfree, const unsigned char* st,
                                           int lane, double ca, double cb, double cs, double c, bool amer,
                                           bool active, double2* sout, const Hints& hz, double& yh, double& f)
{
    using G = Geo<kBig>;
    constexpr int kGroup = G::kGroup, kSub = G::kSubC;
    constexpr int kW = rec_width<kTwin>();
    const int rl = kTwin ? lane >> 1 : lane;  // this lane's entry of the records
    const double* sc_ = reinterpret_cast<const double*>(st) + rl;
    const double* sp_ = reinterpret_cast<const double*>(st + G::kStageCoef) + rl;
    const double2* ss_ = reinterpret_cast<const double2*>(st + G::kStageCoef + G::kStageP) + lane;
#pragma unroll
    for (int h = 0; h < kGroup / kSub; ++h) {
        // chunk h in processing order: nodes [cf, cf + kSub)
        const int cf = kUp ? first + h * kSub : first + kGroup - kSub - h * kSub;
        double ra[kSub], rb[kSub], rs[kSub], rv[kSub], rw[kSub];
        long long rp[kSub];
#pragma unroll
        for (int k = 0; k < kSub; ++k) {
            const int idx = (cf - first) + (kUp ? k : kSub - 1 - k);  // node within the stage
            rp[k] = floor_bits(pfree ? 0. : sp_[idx * kW], amer, first + idx, N);
            const double2 sv = ss_[idx * kTile];
            rv[k] = sv.x;
            rw[k] = sv.y;
            ra[k] = kCompact ? ca : sc_[(idx * kCoef + 0) * kW];
            rb[k] = kCompact ? cb : sc_[(idx * kCoef + 1) * kW];
            rs[k] = kCompact ? cs : sc_[(idx * kCoef + 2) * kW];
        }
        stage_steps<kUp, kHalf, kSub>(ra, rb, rs, rp, rv, rw, cf, c, active, sout,
                                      stage_policy<kUp>(cf, kSub, N, hz), yh, f);
    }
    fence_proxy_async_shared();  // this lane's reads of the slot precede the refill
    __syncwarp();
    if (lane == 0) prod.refill(ring, tv, N, rg, hz.stream);
}

// One wide stage (kWide middle-region nodes, wide layout, chunks of kSubW nodes).
template <bool kUp, bool kHalf, bool kTwin, bool kBig>
__device__ __forceinline__ void stage_body_wide(const Ring& ring, const TileView& tv,
                                                Producer<kUp, kTwin, kBig>& prod, int N, const Ranges& rg, int first,
                                                bool pfree, const unsigned char* st, int lane, double ca, double cb,
                                                double cs, double c, bool amer, bool active, double2* sout,
                                                const Hints& hz, double& yh, double& f)
{
    using G = Geo<kBig>;
    constexpr int kWide = G::kWide, kSub = G::kSubW;
    constexpr int kW = rec_width<kTwin>();
    const double* sp_ = reinterpret_cast<const double*>(st) + (kTwin ? lane >> 1 : lane);
    const double2* ss_ = reinterpret_cast<const double2*>(st + G::kWideP) + lane;
#pragma unroll
    for (int h = 0; h < kWide / kSub; ++h) {
        const int cf = kUp ? first + h * kSub : first + kWide - kSub - h * kSub;
        double ra[kSub], rb[kSub], rs[kSub], rv[kSub], rw[kSub];
        long long rp[kSub];
#pragma unroll
        for (int k = 0; k < kSub; ++k) {
            const int idx = (cf - first) + (kUp ? k : kSub - 1 - k);
            rp[k] = floor_bits(pfree ? 0. : sp_[idx * kW], amer, first + idx, N);
            const double2 sv = ss_[idx * kTile];
            rv[k] = sv.x;
            rw[k] = sv.y;
            ra[k] = ca;
            rb[k] = cb;
            rs[k] = cs;
        }
        stage_steps<kUp, kHalf, kSub>(ra, rb, rs, rp, rv, rw, cf, c, active, sout,
                                      stage_policy<kUp>(cf, kSub, N, hz), yh, f);
    }
    fence_proxy_async_shared();
    __syncwarp();
    if (lane == 0) prod.refill(ring, tv, N, rg, hz.stream);
}

// A sweep's last stage when it holds fewer than G nodes.  It refills no ring slot (no
// later stage), so it reads shared memory node by node in a rolled loop and holds no
// stage in registers.
template <bool kUp, bool kHalf, bool kTwin, bool kBig>
__device__ __forceinline__ void tail_stage(int first, int count, bool compact, bool pfree, const unsigned char* st,
                                           int lane, double ca, double cb, double cs, double c, bool amer,
                                           bool active, int N, double2* sout, const Hints& hz, double& yh,
                                           double& f)
{
    using G = Geo<kBig>;
    constexpr int kW = rec_width<kTwin>();
    const int rl = kTwin ? lane >> 1 : lane;
    const double* sc_ = reinterpret_cast<const double*>(st) + rl;
    const double* sp_ = reinterpret_cast<const double*>(st + G::kStageCoef) + rl;
    const double2* ss_ = reinterpret_cast<const double2*>(st + G::kStageCoef + G::kStageP) + lane;
#pragma unroll 1
    for (int k = 0; k < count; ++k) {
        const int idx = kUp ? k : count - 1 - k;
        const int j = first + idx;
        const double2 sv = ss_[idx * kTile];
        const double a = compact ? ca : sc_[(idx * kCoef + 0) * kW];
        const double bb = compact ? cb : sc_[(idx * kCoef + 1) * kW];
        const double sg = compact ? cs : sc_[(idx * kCoef + 2) * kW];
        yh = fma(-a, yh, sv.y);
        double vn = kHalf ? fma(sg, yh, -sv.x) : fma(sg, yh, -c * sv.x);
        if (amer && j < N - 1) vn = max_floor(vn, pfree ? 0. : sp_[idx * kW]);
        f = fma(-bb, f, vn);
        if (active)
            st_global_f64x2_hint(reinterpret_cast<double*>(sout + (size_t)j * kTile), vn, f,
                                 (kUp ? j >= N - hz.keep_n : j < hz.keep_n) ? hz.keep : hz.stream);
    }
}

// One sweep over this warp's tile.  Returns the stage visits it consumed, or -1 on a
// wait timeout (copies in flight already drained).
template <bool kUp, bool kHalf, bool kTwin, bool kBig>
__device__ __forceinline__ int sweep(const Ring& ring, uint32_t q, const TileView& tv, int lane, int N,
                                     const Ranges& rg, const double* cst, double c, bool amer, bool active,
                                     const Hints& hz, int* err)
{
    using G = Geo<kBig>;
    // the previous sweep's stores, and the lanes' reads of the slots its last stages
    // used, are ordered before the bulk copies that refill them
    fence_proxy_async_all();
    __syncwarp();
    Producer<kUp, kTwin, kBig> prod{sweep_first<kUp>(N), q};
    if (lane == 0)
        for (int i = 0; i < kRing; ++i) prod.refill(ring, tv, N, rg, hz.stream);
    // middle-region constants: UP uses (nh, l, 1/e), DOWN (uh, m, 1/d)
    const double ca = kUp ? cst[0] : cst[3], cb = kUp ? cst[1] : cst[4], cs = kUp ? cst[2] : cst[5];
    double2* sout = reinterpret_cast<double2*>(tv.s) + lane;
    double yh = 0., f = 0.;
    uint32_t v = q;
    for (int cur = sweep_first<kUp>(N); !sweep_done<kUp>(cur, N); ++v) {
        const int s = (int)(v % kRing);
        const bool ok = __all_sync(0xffffffffu, mbar_wait(&ring.bar[s], (v / kRing) & 1u));
        if (!ok) {
            if (lane == 0) {
                atomicExch(err, 1);
                drain(ring, v, prod.next);
            }
            __syncwarp();
            return -1;
        }
        const Stage sg = stage_at<kUp, kBig>(cur, N, rg);
        const unsigned char* st = ring.stage + (size_t)s * G::kStageBytes;
        if (sg.wide)
            stage_body_wide<kUp, kHalf, kTwin, kBig>(ring, tv, prod, N, rg, sg.first, sg.pfree, st, lane, ca, cb, cs, c,
                                               amer, active, sout, hz, yh, f);
        else if (sg.count == G::kGroup && sg.compact)
            stage_body<kUp, kHalf, true, kTwin, kBig>(ring, tv, prod, N, rg, sg.first, sg.pfree, st, lane, ca, cb, cs, c,
                                                amer, active, sout, hz, yh, f);
        else if (sg.count == G::kGroup)
            stage_body<kUp, kHalf, false, kTwin, kBig>(ring, tv, prod, N, rg, sg.first, sg.pfree, st, lane, ca, cb, cs, c,
                                                 amer, active, sout, hz, yh, f);
        else
            tail_stage<kUp, kHalf, kTwin, kBig>(sg.first, sg.count, sg.compact, sg.pfree, st, lane, ca, cb, cs, c, amer,
                                          active, N, sout, hz, yh, f);
        cur = stage_after<kUp>(cur, sg);
    }
    return (int)(v - q);
}

}  // namespace

// Persistent: each warp takes tiles from tile_counter[0] (zeroed by the host before
// the launch) and runs all tDim-1 steps of its 32 PDEs.  A block holds 1, 2 or 4
// independent warps (32 options each; each warp has its own ring); the block size is
// a tuned launch parameter.  The sweeps stream through a 2-deep ring of stages in
// shared memory filled by the TMA engine (2 G nodes in the middle region, G with
// coefficients elsewhere; G = 8, or 16 with kBig); V and h|f are
// written back with 16-byte stores, L2 evict-last for the last sh.keep_nodes nodes of a
// sweep (read back first by the next one) and evict-first otherwise.  If a ring wait expires,
// tile_counter[1] is set, the warp drains its copies in flight and leaves; the
// interpolation kernel then marks every option with KWG_STATUS_DEVICE_TIMEOUT.
// tile_counter[2..3] accumulates (64-bit) the bytes the launch reads and writes.
// kHalf: theta = 1/2 (c = 1).  kBig: the big stage geometry (Geo).
template <bool kHalf, bool kBig>
__global__ void __launch_bounds__(32 * kMaxBlockWarps)
    fd1d_solve_fp64(const PdeBatch b, Fd1dShape sh, double* __restrict__ base, int* __restrict__ tile_counter)
{
    using G = Geo<kBig>;
    extern __shared__ __align__(128) unsigned char smem[];
    Ring ring;
    ring.stage = smem + (size_t)(threadIdx.x >> 5) * G::kSolveSmem;
    ring.bar = reinterpret_cast<uint64_t*>(ring.stage + kRing * G::kStageBytes);
    const int lane = threadIdx.x & 31;
    if (lane == 0) {
        for (int s = 0; s < kRing; ++s) mbar_init(&ring.bar[s], 1);
        fence_mbar_init();
    }
    __syncwarp();

    const int ntiles = b.m_pad / kTile;
    const Work wk = work_of(base, b.m_pad, sh.node_lanes);
    Hints hz;
    hz.keep = l2_policy_evict_last();
    hz.stream = sh.keep_nodes > 0 ? l2_policy_evict_first() : l2_policy_evict_normal();
    hz.keep_n = sh.keep_nodes;
    uint32_t q = 0;  // stage visits consumed so far
    for (;;) {
        int tile = 0;
        if (lane == 0) tile = atomicAdd(&tile_counter[0], 1);
        tile = __shfl_sync(0xffffffffu, tile, 0);
        if (tile >= ntiles) break;
        const int slot = tile * kTile + lane;
        const int src = slot < b.m ? slot : b.m - 1;
        const bool amer = b.e[src] != 0;
        int N;
        long long toff;
        tile_shape(sh, tile, N, toff);
        const TileView tv = tile_view(wk, toff);
        const bool twin = tile < sh.twin_tiles;  // one coefficient and payoff record per lane pair
        // every lane steps its own PDE tDim-1 times; the tile runs for its longest
        const int t_lane = shape_t(sh, src);
        const int t_max = sh.tiles ? sh.tiles[tile].t_max : sh.t_dim;
        // the tile's middle region is where every lane's coefficients are frozen
        const int2 mr = wk.range[slot], zr = wk.zero[slot];
        Ranges rg;
        rg.lo = __reduce_max_sync(0xffffffffu, mr.x);
        rg.hi = __reduce_min_sync(0xffffffffu, mr.y);
        rg.zlo = __reduce_max_sync(0xffffffffu, zr.x);
        rg.zhi = __reduce_min_sync(0xffffffffu, zr.y);
        const int lo = rg.lo, hi = rg.hi;
        double cst[kConsts] = {0., 0., 0., 0., 0., 0.};
        if (lo <= hi)
            for (int k = 0; k < kConsts; ++k) cst[k] = wk.cst[(size_t)slot * kConsts + k];
        if (lane == 0) {
            // bytes this tile moves per sweep: the stages' bulk reads + the state stores
            unsigned long long per_up = 0, per_dn = 0;
            for (int cur = sweep_first<true>(N); !sweep_done<true>(cur, N);) {
                const Stage sg = stage_at<true, kBig>(cur, N, rg);
                per_up += stage_bytes(sg, twin);
                cur = stage_after<true>(cur, sg);
            }
            for (int cur = sweep_first<false>(N); !sweep_done<false>(cur, N);) {
                const Stage sg = stage_at<false, kBig>(cur, N, rg);
                per_dn += stage_bytes(sg, twin);
                cur = stage_after<false>(cur, sg);
            }
            const unsigned long long n_up = (unsigned long long)(t_max / 2);  // passes 1, 3, 5, ...
            const unsigned long long n_dn = (unsigned long long)((t_max - 1) / 2);
            atomicAdd(reinterpret_cast<unsigned long long*>(tile_counter + 2), per_up * n_up + per_dn * n_dn);
        }
        Hints ht = hz;
        ht.keep_n = min(hz.keep_n, N / 2);
        for (int pass = 1; pass < t_max; ++pass) {
            const bool act = pass < t_lane;
            int used;
            if (twin)
                used = (pass & 1) ? sweep<true, kHalf, true, kBig>(ring, q, tv, lane, N, rg, cst, sh.c, amer, act,
                                                                   ht, &tile_counter[1])
                                  : sweep<false, kHalf, true, kBig>(ring, q, tv, lane, N, rg, cst, sh.c, amer, act,
                                                                    ht, &tile_counter[1]);
            else
                used = (pass & 1) ? sweep<true, kHalf, false, kBig>(ring, q, tv, lane, N, rg, cst, sh.c, amer, act,
                                                                    ht, &tile_counter[1])
                                  : sweep<false, kHalf, false, kBig>(ring, q, tv, lane, N, rg, cst, sh.c, amer, act,
                                                                     ht, &tile_counter[1]);
            if (used < 0) return;
            q += (uint32_t)used;
        }
    }
}

// One thread per asset: x* = log(s/k), first node x_i >= x* (binary search on the
// grid, the same node the reference's linear search finds, src/Math/kwFd1d.cpp:
// 145-147), linear interpolation (:156), price = k*V (src/Pricer/kwFd1d.cpp:156).
__global__ void fd1d_interp_fp64(const PdeBatch b, const AssetBatch a, Fd1dShape sh, double* __restrict__ base,
                                 const int32_t* __restrict__ pde_status, const int* __restrict__ device_error,
                                 double* __restrict__ prices, int32_t* __restrict__ status)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int slot = a.pde[i];
    int N;
    long long toff;
    tile_shape(sh, slot / kTile, N, toff);
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
            const TileView tv = tile_view(work_of(base, b.m_pad, sh.node_lanes), toff);
            const int lane = slot % kTile;
            const double xl = g.x(lo - 1), xh = g.x(lo);
            const double vl = tv.s[((size_t)(lo - 1) * kTile + lane) * 2];
            const double vh = tv.s[((size_t)lo * kTile + lane) * 2];
            const double v = dvd(add(mul(sub(xh, xs), vl), mul(sub(xs, xl), vh)), sub(xh, xl));
            price = mul(k, v);
        }
    }
    // a solve that left a non-finite value where the price is read is a solver failure
    if (st == KWG_STATUS_OK && !isfinite(price)) {
        st = KWG_STATUS_SOLVER;
        price = __longlong_as_double(0x7ff8000000000000ll);
    }
    prices[i] = price;
    if (status) status[i] = st;
}

namespace {
// Per-device launch facts, filled once under a lock by fd1d_prepare_kernels and read
// without one afterwards (the ready flag publishes them).
constexpr int kMaxDevices = 64;
struct DeviceFacts {
    int sms = 0;
    int l2 = 0;  // L2 bytes
    // FP64 streaming solver: resident blocks per SM by block size, small and big stages
    int max_blocks[kMaxBlockWarps + 1] = {};
    int max_blocks_big[kMaxBlockWarps + 1] = {};
};
DeviceFacts g_facts[kMaxDevices];
std::atomic<bool> g_ready[kMaxDevices];
std::mutex g_prepare_mu;
}  // namespace

void fd1d_prepare_kernels(int device)
{
    if (device < 0 || device >= kMaxDevices || g_ready[device].load(std::memory_order_acquire)) return;
    std::lock_guard<std::mutex> lock(g_prepare_mu);
    if (g_ready[device].load(std::memory_order_relaxed)) return;
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != device) cudaSetDevice(device);
    DeviceFacts& f = g_facts[device];
    cudaDeviceGetAttribute(&f.sms, cudaDevAttrMultiProcessorCount, device);
    cudaDeviceGetAttribute(&f.l2, cudaDevAttrL2CacheSize, device);
    constexpr size_t kSmall = Geo<false>::kSolveSmem, kBigSmem = Geo<true>::kSolveSmem;
    cudaFuncSetAttribute(fd1d_solve_fp64<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(kMaxBlockWarps * kSmall));
    cudaFuncSetAttribute(fd1d_solve_fp64<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(kMaxBlockWarps * kSmall));
    cudaFuncSetAttribute(fd1d_solve_fp64<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(kMaxBlockWarps * kBigSmem));
    cudaFuncSetAttribute(fd1d_solve_fp64<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(kMaxBlockWarps * kBigSmem));
    for (int bw = 1; bw <= kMaxBlockWarps; bw *= 2) {
        int mx = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&mx, fd1d_solve_fp64<true, false>, 32 * bw, bw * kSmall);
        f.max_blocks[bw] = mx < 1 ? 1 : mx;
        mx = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&mx, fd1d_solve_fp64<true, true>, 32 * bw, bw * kBigSmem);
        f.max_blocks_big[bw] = mx;  // 0: does not fit
    }
    fd1d_fp32_prepare(device);
    fd1d_pcr64_prepare(device);
    if (prev >= 0 && prev != device) cudaSetDevice(prev);
    g_ready[device].store(true, std::memory_order_release);
}

namespace {
// Big stages when the launch caps the residency (sm_blocks > 0) at a level their
// shared memory allows: then every resident warp gets the bigger ring.
bool use_big_stages(const DeviceFacts& f, int bw, int sm_blocks)
{
    return sm_blocks > 0 && sm_blocks <= f.max_blocks_big[bw];
}
}  // namespace

int fd1d_fp64_solve_blocks(int ntiles, int device, int block_warps, int sm_blocks)
{
    if (device < 0 || device >= kMaxDevices) return 1;
    fd1d_prepare_kernels(device);
    const DeviceFacts& f = g_facts[device];
    const int bw = block_warps == 2 || block_warps == 4 ? block_warps : 1;
    const int want = (ntiles + bw - 1) / bw;  // one tile per warp at most
    const int per_sm = use_big_stages(f, bw, sm_blocks) ? sm_blocks
                       : sm_blocks > 0 && sm_blocks < f.max_blocks[bw] ? sm_blocks
                                                                       : f.max_blocks[bw];
    const int cap = (f.sms > 0 ? f.sms : 1) * per_sm;
    return want < cap ? (want > 0 ? want : 1) : cap;
}

size_t fd1d_fp64_work_bytes_nl(int m_pad, long long node_lanes)
{
    return (size_t)node_lanes * (2 * kCoef + 1 + 2) * sizeof(double) + (size_t)m_pad * kConsts * sizeof(double) +
           2 * (size_t)m_pad * sizeof(int2);
}

size_t fd1d_fp64_work_bytes(int m_pad, int x_dim) { return fd1d_fp64_work_bytes_nl(m_pad, (long long)m_pad * x_dim); }

int fd1d_fp64_launch(const PdeBatch& b, const AssetBatch& a, const Fd1dShape& sh_in, double* work, int32_t* pde_status,
                     int* counters, double* prices, int32_t* status, int solve_blocks, cudaStream_t stream,
                     const SolveEvents* ev)
{
    Fd1dShape sh = sh_in;
    if (!sh.tiles) sh.node_lanes = (long long)b.m_pad * sh.x_dim;
    int launches = 0;
    fd1d_setup_fp64<<<(b.m_pad + 127) / 128, 128, 0, stream>>>(b, sh, work, pde_status);
    ++launches;
    cudaMemsetAsync(counters, 0, 4 * sizeof(int), stream);
    if (ev) cudaEventRecord(ev->start, stream);
    const int bw = sh.block_warps == 2 || sh.block_warps == 4 ? sh.block_warps : 1;
    int dev = 0;
    cudaGetDevice(&dev);
    const bool known = dev >= 0 && dev < kMaxDevices;
    {
        // nodes per sweep end kept in L2: a share of the L2 split over the resident warps
        // (each node is 32 lanes x 16 B of state)
        const long long l2 = known ? g_facts[dev].l2 : 0;
        const long long warps = (long long)solve_blocks * bw;
        sh.keep_nodes = warps > 0 ? (int)((long long)(kKeepShare * (double)l2) / (warps * kTile * 16)) : 0;
    }
    // the same choice fd1d_fp64_solve_blocks made for the grid size
    const bool big = known && use_big_stages(g_facts[dev], bw, sh.sm_blocks);
    const size_t smem = bw * (big ? Geo<true>::kSolveSmem : Geo<false>::kSolveSmem);
    if (sh.c == 1.) {
        if (big)
            fd1d_solve_fp64<true, true><<<solve_blocks, 32 * bw, smem, stream>>>(b, sh, work, counters);
        else
            fd1d_solve_fp64<true, false><<<solve_blocks, 32 * bw, smem, stream>>>(b, sh, work, counters);
    } else {
        if (big)
            fd1d_solve_fp64<false, true><<<solve_blocks, 32 * bw, smem, stream>>>(b, sh, work, counters);
        else
            fd1d_solve_fp64<false, false><<<solve_blocks, 32 * bw, smem, stream>>>(b, sh, work, counters);
    }
    if (ev) {
        cudaEventRecord(ev->stop, stream);
        if (ev->bytes) cudaMemcpyAsync(ev->bytes, counters + 2, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                       stream);
    }
    ++launches;
    if (a.n > 0) {
        fd1d_interp_fp64<<<(a.n + 127) / 128, 128, 0, stream>>>(b, a, sh, work, pde_status, counters + 1, prices,
                                                                 status);
        ++launches;
    }
    return launches;
}

}  // namespace kwg
