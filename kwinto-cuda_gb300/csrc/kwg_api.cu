// kwg_api.cu -- the C ABI of include/kwg.h: context, host-side deduplication,
// staging, launches and error mapping.
//
// Host flow of kwg_fd1d_price, mirroring kw::Fd1d_Pricer::price
// (src/Pricer/kwFd1d.cpp:21-160):
//   1. dedup the options by (t, r, q, z, e, w) like src/Pricer/kwFd1d.cpp:28-65;
//   2. pack PDE and asset arrays into one pinned buffer, one H2D copy;
//   3. setup + solve + interpolation kernels on the context stream;
//   4. one D2H copy of (prices, status); strict mode maps the first bad option to
//      the reference's whole-call error (src/Pricer/kwFd1d.cpp:154-155).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <numeric>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "fd1d_kernels.h"
#include "host_dedup.h"
#include "kwg.h"
#include "kwg_ctx.h"
#include "tma.cuh"

namespace {

using namespace kwgi;


// Device pointers into one packed buffer holding a batch's inputs and outputs.
struct IoLayout {
    size_t t, z, r, q, s, k, pde, w, e, prices, status, pde_status, total;
    size_t in_bytes;   // [0, in_bytes) is copied host -> device
    size_t out_bytes;  // [prices, prices + out_bytes) is copied device -> host
};

IoLayout io_layout(size_t m, size_t m_pad, size_t n)
{
    IoLayout L;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        size_t at = o;
        o = align_up(o + bytes, 256);
        return at;
    };
    L.t = take(m * 8);
    L.z = take(m * 8);
    L.r = take(m * 8);
    L.q = take(m * 8);
    L.s = take(n * 8);
    L.k = take(n * 8);
    L.pde = take(n * 4);
    L.w = take(m);
    L.e = take(m);
    L.in_bytes = o;
    L.prices = take(n * 8);
    L.status = take(n * 4);
    L.out_bytes = o - L.prices;
    L.pde_status = take(m_pad * 4);
    L.total = o;
    return L;
}

// FD1D-BS epilogue (src/Pricer/kwFd1d_BlackScholes.cpp:15-42): asset i < n was solved
// as given (price[i]) and as its European copy (price[n + i]); the result is
// price[i] + BS(European copy) - price[n + i].  The Black-Scholes price follows
// src/Pricer/kwBlackScholes.cpp:27-49 term for term, with the normal CDF as
// 0.5 (1 + erf(x / sqrt 2)) (src/Math/kwMath.cpp).
__global__ void bs_control_variate(int n, const double* __restrict__ s, const double* __restrict__ k,
                                   const int32_t* __restrict__ pde, const double* __restrict__ t,
                                   const double* __restrict__ z, const double* __restrict__ r,
                                   const double* __restrict__ q, const int8_t* __restrict__ w,
                                   double* __restrict__ prices, int32_t* __restrict__ status)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int j = pde[i];
    const double tt = t[j], zz = z[j], rr = r[j], qq = q[j], ww = (double)w[j], ss = s[i], kk = k[i];
    const double zt = zz * sqrt(tt);
    const double d1 = 1 / zt * (log(ss / kk) + (rr - qq + 0.5 * zz * zz) * tt);
    const double d2 = d1 - zt;
    auto cdf = [](double x) { return 0.5 * (1 + erf(x / 1.41421356237309504880)); };
    const double bs = ww * (ss * cdf(ww * d1) * exp(-qq * tt) - kk * cdf(ww * d2) * exp(-rr * tt));
    prices[i] = prices[i] + (bs - prices[n + i]);
    if (status[i] == KWG_STATUS_OK) status[i] = status[n + i];
}

// Exercise / put-call class of a PDE: European puts, European calls, American puts,
// American calls.  Tiles of one class let the streaming FP64 kernel skip the payoff
// where it is zero for every lane (kernels are indifferent to the PDE order).
__host__ __device__ inline int pde_class(uint8_t e, int8_t w) { return (e ? 2 : 0) + (w < 0 ? 0 : 1); }

// Device path, pass 1: PDEs per class (warp-aggregated atomics).
__global__ void count_classes(const kwg_option* __restrict__ o, int n, int* __restrict__ counts)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = i < n ? pde_class(o[i].e, o[i].w) : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, c);
    if (c >= 0 && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&counts[c], __popc(peers));
}

// Device path, pass 2: AoS options -> the SoA arrays of one packed buffer, each PDE
// at its class's offset + a slot taken in arrival order; pde[i] points at it.
__global__ void unpack_options(const kwg_option* __restrict__ o, int n, const int* __restrict__ counts,
                               int* __restrict__ cursor, double* t, double* z, double* r, double* q, double* s,
                               double* k, int32_t* pde, int8_t* w, uint8_t* e)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = i < n ? pde_class(o[i].e, o[i].w) : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, c);
    const int leader = __ffs(peers) - 1, lane = threadIdx.x & 31;
    int base = 0;
    if (c >= 0 && lane == leader) base = atomicAdd(&cursor[c], __popc(peers));
    base = __shfl_sync(peers, base, leader);
    if (c < 0) return;
    int off = 0;
    for (int v = 0; v < c; ++v) off += counts[v];
    const int slot = off + base + __popc(peers & ((1u << lane) - 1u));
    const kwg_option a = o[i];
    t[slot] = a.t;
    z[slot] = a.z;
    r[slot] = a.r;
    q[slot] = a.q;
    w[slot] = a.w;
    e[slot] = a.e;
    s[i] = a.s;
    k[i] = a.k;
    pde[i] = slot;
}

// ---- device-side dedup (kwg_fd1d_price_device with device_dedup): the key of
// src/Pricer/kwFd1d.cpp:28-65 in an open-addressing table of 2^k >= 2n slots, each
// holding 1 + the index of the option that owns a key (0 = empty).  Keys compare by
// value (+0 == -0; a NaN field never matches, so such options stay separate).
__device__ __forceinline__ bool same_key(const kwg_option& a, const kwg_option& b)
{
    return a.t == b.t && a.r == b.r && a.q == b.q && a.z == b.z && a.e == b.e && a.w == b.w;
}

__device__ __forceinline__ uint64_t key_hash(const kwg_option& o)
{
    uint64_t h = 0x9E3779B97F4A7C15ull;
    for (double v : {o.t, o.r, o.q, o.z}) {
        const uint64_t b = v == 0. ? 0ull : (uint64_t)__double_as_longlong(v);
        h = (h ^ b) * 0xBF58476D1CE4E5B9ull;
        h ^= h >> 31;
    }
    h = (h ^ ((uint64_t)o.e << 8 | (uint8_t)o.w)) * 0x94D049BB133111EBull;
    return h ^ (h >> 29);
}

__global__ void dedup_insert(const kwg_option* __restrict__ o, int n, unsigned* __restrict__ table,
                             unsigned mask, int* __restrict__ owner)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const kwg_option a = o[i];
    unsigned p = (unsigned)key_hash(a) & mask;
    int own = i;  // the probe below ends within mask + 1 steps: the table is at most half full
    for (unsigned it = 0; it <= mask; ++it) {
        const unsigned cur = atomicCAS(&table[p], 0u, (unsigned)i + 1u);
        if (cur == 0u) break;
        if (same_key(o[cur - 1u], a)) {
            own = (int)(cur - 1u);
            break;
        }
        p = (p + 1u) & mask;
    }
    owner[i] = own;
}

// Owners per class, like count_classes.
__global__ void dedup_count(const kwg_option* __restrict__ o, int n, const int* __restrict__ owner,
                            int* __restrict__ counts)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = (i < n && owner[i] == i) ? pde_class(o[i].e, o[i].w) : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, c);
    if (c >= 0 && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&counts[c], __popc(peers));
}

// Owners become PDEs at class offset + arrival slot; every option keeps its s, k.
__global__ void dedup_unpack(const kwg_option* __restrict__ o, int n, const int* __restrict__ owner,
                             const int* __restrict__ counts, int* __restrict__ cursor, int* __restrict__ slot_of,
                             double* t, double* z, double* r, double* q, double* s, double* k, int8_t* w,
                             uint8_t* e)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = (i < n && owner[i] == i) ? pde_class(o[i].e, o[i].w) : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, c);
    const int leader = __ffs(peers) - 1, lane = threadIdx.x & 31;
    int base = 0;
    if (c >= 0 && lane == leader) base = atomicAdd(&cursor[c], __popc(peers));
    base = __shfl_sync(peers, base, leader);
    if (i >= n) return;
    const kwg_option a = o[i];
    s[i] = a.s;
    k[i] = a.k;
    if (c < 0) return;
    int off = 0;
    for (int v = 0; v < c; ++v) off += counts[v];
    const int slot = off + base + __popc(peers & ((1u << lane) - 1u));
    slot_of[i] = slot;
    t[slot] = a.t;
    z[slot] = a.z;
    r[slot] = a.r;
    q[slot] = a.q;
    w[slot] = a.w;
    e[slot] = a.e;
}

__global__ void dedup_map(int n, const int* __restrict__ owner, const int* __restrict__ slot_of,
                          int32_t* __restrict__ pde)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) pde[i] = slot_of[owner[i]];
}

// Self-test of the bounded waits every kernel uses: out[0] = 1 when a wait on an
// mbarrier that nothing arrives on gives up after `limit` polls (the timeout path
// the solvers take before setting their error flags); out[1] = 1 when a wait on an
// mbarrier this thread arrived on succeeds.  One thread, nothing in flight.
__global__ void selftest_waits(int32_t* __restrict__ out, uint32_t limit)
{
    __shared__ uint64_t bar[2];
    if (threadIdx.x != 0) return;
    kwg::mbar_init(&bar[0], 1);
    kwg::mbar_init(&bar[1], 1);
    kwg::fence_mbar_init();
    out[0] = kwg::mbar_wait_n(&bar[0], 0, limit) ? 0 : 1;
    kwg::mbar_arrive(&bar[1]);
    out[1] = kwg::mbar_wait_n(&bar[1], 0, limit) ? 1 : 0;
}


// Launch choices for a batch of m PDEs: the explicit ones in p, else what the
// autotuner recorded for the shape, else defaults.  FP64 solver default: a cost
// model -- the thread-per-option kernel runs m/32 warps, the warp-per-option kernel
// m warps at twice the FP64 work per node-step, so the latter wins while m/32 warps
// cannot fill the GPU (a few warps per SM).
kwg_ctx::Tuned choose(kwg_ctx* ctx, const kwg_fd1d_params* p, int m)
{
    kwg_ctx::Tuned t;
    auto it = ctx->tuned.find(tune_key(p->precision, p->x_dim, p->t_dim, m));
    if (it != ctx->tuned.end()) {
        t = it->second;
    } else {
        const bool pcr_ok = kwg::fd1d_pcr64_nodes_per_lane(p->x_dim) > 0;
        t.solver = (pcr_ok && m < 8192) ? KWG_SOLVER_PCR : KWG_SOLVER_THOMAS;
    }
    if (p->precision == KWG_FP32) t.solver = KWG_SOLVER_PCR;
    else if (p->solver != KWG_SOLVER_AUTO) t.solver = p->solver;
    // an explicit block size or residency replaces the recorded pair (the tuner timed
    // every block size at full residency)
    if (p->block_warps || p->sm_blocks) {
        if (p->block_warps) t.block_warps = p->block_warps;
        t.sm_blocks = p->sm_blocks;
    }
    if (p->option_warps) t.option_warps = p->option_warps;
    return t;
}

int run_batch(kwg_ctx* ctx, char* io, const IoLayout& L, int m, int n, const kwg_fd1d_params* p,
              double* prices, int32_t* status, cudaStream_t stream, int twin_tiles = 0)
{
    const int m_pad = (m + kwg::kTile - 1) / kwg::kTile * kwg::kTile;
    kwg::PdeBatch b;
    b.t = (const double*)(io + L.t);
    b.z = (const double*)(io + L.z);
    b.r = (const double*)(io + L.r);
    b.q = (const double*)(io + L.q);
    b.w = (const int8_t*)(io + L.w);
    b.e = (const uint8_t*)(io + L.e);
    b.m = m;
    b.m_pad = m_pad;
    kwg::AssetBatch a;
    a.s = (const double*)(io + L.s);
    a.k = (const double*)(io + L.k);
    a.pde = (const int32_t*)(io + L.pde);
    a.n = n;
    kwg::Fd1dShape sh = make_shape(p);
    sh.twin_tiles = twin_tiles;
    const kwg_ctx::Tuned tn = choose(ctx, p, m);
    const int solver = tn.solver;
    sh.block_warps = tn.block_warps;
    sh.option_warps = tn.option_warps;
    sh.sm_blocks = tn.sm_blocks;
    if (p->precision == KWG_FP64 && solver == KWG_SOLVER_PCR) {
        const size_t wbytes = kwg::fd1d_fp32_work_bytes(m, sh.x_dim);
        if (int rc = ensure_device(ctx, &ctx->d_work, &ctx->work_bytes, wbytes)) return rc;
        const int n_launch = kwg::fd1d_pcr64_launch(b, a, sh, (double*)ctx->d_work, (int32_t*)(io + L.pde_status),
                                                    ctx->d_counter, prices, status, ctx->device, stream,
                                                    ctx->next_events());
        if (n_launch < 0) return set_err(ctx, KWG_ERR_INVALID, "kwg: the FP64 PCR solver supports x_dim <= 1024");
        ctx->launches += n_launch;
    } else if (p->precision == KWG_FP32) {
        const size_t wbytes = kwg::fd1d_fp32_work_bytes(m, sh.x_dim);
        if (int rc = ensure_device(ctx, &ctx->d_work, &ctx->work_bytes, wbytes)) return rc;
        const int n_launch = kwg::fd1d_fp32_launch(b, a, sh, (double*)ctx->d_work, (int32_t*)(io + L.pde_status),
                                                   ctx->d_counter, prices, status, ctx->device, stream,
                                                   ctx->next_events());
        if (n_launch < 0) return set_err(ctx, KWG_ERR_INVALID, "kwg: FP32 stepping supports x_dim <= 2048");
        ctx->launches += n_launch;
    } else {
        const size_t wbytes = kwg::fd1d_fp64_work_bytes(m_pad, sh.x_dim);
        if (int rc = ensure_device(ctx, &ctx->d_work, &ctx->work_bytes, wbytes)) return rc;
        const int blocks = kwg::fd1d_fp64_solve_blocks(m_pad / kwg::kTile, ctx->device, sh.block_warps, sh.sm_blocks);
        ctx->launches += kwg::fd1d_fp64_launch(b, a, sh, (double*)ctx->d_work, (int32_t*)(io + L.pde_status),
                                               ctx->d_counter, prices, status, blocks, stream, ctx->next_events());
    }
    KWG_CUDA(ctx, cudaGetLastError());
    return KWG_OK;
}

// Host-array pricing (kwg_fd1d_price; with `control_variate`, kwg_fd1d_bs_price).
// The control variate prices 2n assets in one batch -- the n given and their
// European copies -- so dedup shares every PDE the two sets have in common, then
// the device epilogue combines them.
int price_host(kwg_ctx* ctx, const kwg_option* user_opts, size_t n_user, const kwg_fd1d_params* p, double* prices,
               int32_t* status, bool control_variate)
{
    if (!ctx) return KWG_ERR_INVALID;
    ctx->err.clear();
    ctx->launches = 0;
    if (int rc = check_params(ctx, p)) return rc;
    if (n_user == 0) return KWG_OK;
    if (!user_opts || !prices) return set_err(ctx, KWG_ERR_INVALID, "kwg: null options or prices");
    if (n_user > (size_t)INT32_MAX / 4) return set_err(ctx, KWG_ERR_INVALID, "kwg: batch too large");
    KWG_CUDA(ctx, cudaSetDevice(ctx->device));
    std::vector<kwg_option> with_euro;
    const kwg_option* opts = user_opts;
    size_t n = n_user;
    if (control_variate) {
        with_euro.assign(user_opts, user_opts + n_user);
        with_euro.resize(2 * n_user);
        for (size_t i = 0; i < n_user; ++i) {
            with_euro[n_user + i] = user_opts[i];
            with_euro[n_user + i].e = 0;
        }
        opts = with_euro.data();
        n = 2 * n_user;
    }

    // 1. dedup by the reference's key (t, r, q, z, e, w), src/Pricer/kwFd1d.cpp:28-65
    std::vector<int32_t> asset2pde;
    std::vector<uint32_t> pde2asset;
    const size_t m = kwg::dedup_host(opts, n, nullptr, nullptr, asset2pde, pde2asset);
    const size_t m_pad = (m + kwg::kTile - 1) / kwg::kTile * kwg::kTile;
    // PDE order.  FD1D-BS: each American PDE and its European copy (the PDE of the
    // asset's European twin, same t, r, q, z, w) go to lanes 2k, 2k+1 of the first
    // tiles -- puts first, then calls -- as many whole tiles of 16 pairs as there are;
    // the streaming FP64 solver then reads one coefficient and payoff record per pair.
    // All other PDEs follow grouped by exercise / put-call class (stable), so tiles are
    // homogeneous.
    int twin_tiles = 0;
    {
        std::vector<int32_t> moved(m, -1);
        std::vector<uint32_t> order2(m);
        size_t placed = 0;
        if (control_variate) {
            std::vector<std::pair<uint32_t, uint32_t>> pairs;
            for (int put_first = 1; put_first >= 0; --put_first)
                for (size_t j = 0; j < m; ++j) {
                    const uint32_t a = pde2asset[j];
                    if (a >= n_user || !opts[a].e || (opts[a].w < 0) != (put_first == 1)) continue;
                    const uint32_t je = (uint32_t)asset2pde[n_user + a];
                    if (je != j) pairs.emplace_back((uint32_t)j, je);
                }
            twin_tiles = (int)(pairs.size() / (kwg::kTile / 2));
            for (size_t k = 0; k < (size_t)twin_tiles * (kwg::kTile / 2); ++k) {
                for (const uint32_t j : {pairs[k].first, pairs[k].second}) {
                    moved[j] = (int32_t)placed;
                    order2[placed++] = pde2asset[j];
                }
            }
        }
        size_t off[5] = {0, 0, 0, 0, 0};
        for (size_t j = 0; j < m; ++j)
            if (moved[j] < 0) ++off[pde_class(opts[pde2asset[j]].e, opts[pde2asset[j]].w) + 1];
        off[0] = placed;
        for (int c = 0; c < 4; ++c) off[c + 1] += off[c];
        for (size_t j = 0; j < m; ++j) {
            if (moved[j] >= 0) continue;
            const uint32_t a = pde2asset[j];
            const size_t to = off[pde_class(opts[a].e, opts[a].w)]++;
            moved[j] = (int32_t)to;
            order2[to] = a;
        }
        pde2asset.swap(order2);
        for (size_t i = 0; i < n; ++i) asset2pde[i] = moved[asset2pde[i]];
    }

    // 2. pack into pinned memory
    const IoLayout L = io_layout(m, m_pad, n);
    if (int rc = ensure_host(ctx, &ctx->h_io, &ctx->h_io_bytes, L.total)) return rc;
    if (int rc = ensure_device(ctx, &ctx->d_io, &ctx->io_bytes, L.total)) return rc;
    char* h = (char*)ctx->h_io;
    double *t = (double*)(h + L.t), *z = (double*)(h + L.z), *r = (double*)(h + L.r), *q = (double*)(h + L.q);
    int8_t* w = (int8_t*)(h + L.w);
    uint8_t* e = (uint8_t*)(h + L.e);
    for (size_t j = 0; j < m; ++j) {
        const kwg_option& o = opts[pde2asset[j]];
        t[j] = o.t;
        z[j] = o.z;
        r[j] = o.r;
        q[j] = o.q;
        w[j] = o.w;
        e[j] = o.e;
    }
    double *s = (double*)(h + L.s), *k = (double*)(h + L.k);
    int32_t* pde = (int32_t*)(h + L.pde);
    for (size_t i = 0; i < n; ++i) {
        s[i] = opts[i].s;
        k[i] = opts[i].k;
        pde[i] = asset2pde[i];
    }
    KWG_CUDA(ctx, cudaMemcpyAsync(ctx->d_io, ctx->h_io, L.in_bytes, cudaMemcpyHostToDevice, ctx->stream));

    // 3. kernels
    char* dio = (char*)ctx->d_io;
    if (int rc = run_batch(ctx, dio, L, (int)m, (int)n, p, (double*)(dio + L.prices), (int32_t*)(dio + L.status),
                           ctx->stream, twin_tiles))
        return rc;
    if (control_variate) {
        bs_control_variate<<<(unsigned)((n_user + 255) / 256), 256, 0, ctx->stream>>>(
            (int)n_user, (const double*)(dio + L.s), (const double*)(dio + L.k), (const int32_t*)(dio + L.pde),
            (const double*)(dio + L.t), (const double*)(dio + L.z), (const double*)(dio + L.r),
            (const double*)(dio + L.q), (const int8_t*)(dio + L.w), (double*)(dio + L.prices),
            (int32_t*)(dio + L.status));
        ctx->launches += 1;
    }

    // 4. results
    KWG_CUDA(ctx, cudaMemcpyAsync(h + L.prices, (char*)ctx->d_io + L.prices, L.out_bytes, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    KWG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const double* hp = (const double*)(h + L.prices);
    const int32_t* hs = (const int32_t*)(h + L.status);
    std::memcpy(prices, hp, n_user * sizeof(double));
    if (status) std::memcpy(status, hs, n_user * sizeof(int32_t));
    if (p->strict) {
        for (size_t i = 0; i < n_user; ++i) {
            if (hs[i] == KWG_STATUS_OK) continue;
            char msg[256];
            if (hs[i] == KWG_STATUS_OUT_OF_GRID) {
                std::snprintf(msg, sizeof msg, "Fd1dGpu_Pricer::price: asset %zu: x=%f not in grid range", i,
                              std::log(opts[i].s / opts[i].k));
                return set_err(ctx, KWG_ERR_OUT_OF_GRID, msg);
            }
            std::snprintf(msg, sizeof msg, "Fd1dGpu_Pricer::price: asset %zu: status %d", i, (int)hs[i]);
            return set_err(ctx, hs[i] == KWG_STATUS_SOLVER ? KWG_ERR_SOLVER : KWG_ERR_INVALID, msg);
        }
    }
    return KWG_OK;
}

// kwg_fd1d_price_device with device_dedup: the packed buffer is laid out for n PDEs
// (the upper bound), the dedup kernels fill m <= n of them, and one synchronisation
// reads m before the solver launches are sized.
int price_device_dedup(kwg_ctx* ctx, const kwg_option* d_opts, size_t n, size_t n_pad, const kwg_fd1d_params* p,
                       double* d_prices, int32_t* d_status, cudaStream_t stream)
{
    const IoLayout L = io_layout(n, n_pad, n);
    unsigned cap = 64;
    while (cap < 2 * n) cap <<= 1;
    const size_t extra = 8 * sizeof(int) + (size_t)cap * sizeof(unsigned) + 2 * n * sizeof(int);
    if (int rc = ensure_device(ctx, &ctx->d_io, &ctx->io_bytes, L.total + extra)) return rc;
    if (int rc = ensure_host(ctx, &ctx->h_io, &ctx->h_io_bytes, 64)) return rc;
    char* io = (char*)ctx->d_io;
    int* counts = (int*)(io + L.total);  // [4] per-class counts, [4] cursors
    unsigned* table = (unsigned*)(counts + 8);
    int* owner = (int*)(table + cap);
    int* slot_of = owner + n;
    KWG_CUDA(ctx, cudaMemsetAsync(counts, 0, 8 * sizeof(int) + (size_t)cap * sizeof(unsigned), stream));
    const unsigned nb = (unsigned)((n + 255) / 256);
    dedup_insert<<<nb, 256, 0, stream>>>(d_opts, (int)n, table, cap - 1, owner);
    dedup_count<<<nb, 256, 0, stream>>>(d_opts, (int)n, owner, counts);
    dedup_unpack<<<nb, 256, 0, stream>>>(d_opts, (int)n, owner, counts, counts + 4, slot_of, (double*)(io + L.t),
                                         (double*)(io + L.z), (double*)(io + L.r), (double*)(io + L.q),
                                         (double*)(io + L.s), (double*)(io + L.k), (int8_t*)(io + L.w),
                                         (uint8_t*)(io + L.e));
    dedup_map<<<nb, 256, 0, stream>>>((int)n, owner, slot_of, (int32_t*)(io + L.pde));
    ctx->launches += 4;
    int* hc = (int*)ctx->h_io;
    KWG_CUDA(ctx, cudaMemcpyAsync(hc, counts, 4 * sizeof(int), cudaMemcpyDeviceToHost, stream));
    KWG_CUDA(ctx, cudaStreamSynchronize(stream));
    const int m = hc[0] + hc[1] + hc[2] + hc[3];
    return run_batch(ctx, io, L, m, (int)n, p, d_prices, d_status, stream);
}

// Synthetic batch of m options for the autotuner: puts and calls, strikes 80..120,
// vols 0.1..0.6, maturities 0.25..2.
std::vector<kwg_option> tuning_batch(size_t m)
{
    std::vector<kwg_option> opts(m);
    for (size_t i = 0; i < m; ++i) {
        const double u = (double)((i * 2654435761u) % 1000) / 1000.;
        const double v = (double)((i * 40503u + 17) % 997) / 997.;
        opts[i] = kwg_option{0.25 + 1.75 * v, 80. + 40. * u, 0.1 + 0.5 * (1. - u), 0.05, 0.02, 100., 1,
                             (int8_t)((i & 1) ? 1 : -1)};
    }
    return opts;
}

}  // namespace

cudaError_t kwg::unpack_by_class(const void* d_opts, int n, int* counts, double* t, double* z, double* r, double* q,
                                 double* s, double* k, int32_t* pde, int8_t* w, uint8_t* e, cudaStream_t stream)
{
    if (cudaError_t ce = cudaMemsetAsync(counts, 0, 8 * sizeof(int), stream); ce != cudaSuccess) return ce;
    const kwg_option* o = (const kwg_option*)d_opts;
    const unsigned nb = (unsigned)((n + 255) / 256);
    count_classes<<<nb, 256, 0, stream>>>(o, n, counts);
    unpack_options<<<nb, 256, 0, stream>>>(o, n, counts, counts + 4, t, z, r, q, s, k, pde, w, e);
    return cudaGetLastError();
}


extern "C" {

void kwg_fd1d_params_default(kwg_fd1d_params* p)
{
    if (!p) return;
    p->t_dim = 512;
    p->x_dim = 512;
    p->theta = 0.5;
    p->scale = 50.;
    p->density = 0.25;
    p->precision = KWG_FP64;
    p->solver = KWG_SOLVER_AUTO;
    p->strict = 0;
    p->device_dedup = 0;
    p->block_warps = 0;
    p->sm_blocks = 0;
    p->option_warps = 0;
}

kwg_ctx* kwg_create(int device)
{
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) return nullptr;
    if (cudaSetDevice(device) != cudaSuccess) return nullptr;
    kwg_ctx* ctx = new kwg_ctx();
    ctx->device = device;
    cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device);
    kwg::fd1d_prepare_kernels(device);
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&ctx->d_counter, 4 * sizeof(int)) != cudaSuccess) {
        kwg_destroy(ctx);
        return nullptr;
    }
    return ctx;
}

void kwg_destroy(kwg_ctx* ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->d_work) cudaFree(ctx->d_work);
    if (ctx->d_io) cudaFree(ctx->d_io);
    if (ctx->d_counter) cudaFree(ctx->d_counter);
    if (ctx->h_io) cudaFreeHost(ctx->h_io);
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    for (auto& e : ctx->events) {
        cudaEventDestroy(e.start);
        cudaEventDestroy(e.stop);
        cudaFreeHost(e.bytes);
    }
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* kwg_last_error(const kwg_ctx* ctx) { return ctx ? ctx->err.c_str() : "kwg: null context"; }

int kwg_last_launch_count(const kwg_ctx* ctx) { return ctx ? ctx->launches : 0; }

int kwg_set_profiling(kwg_ctx* ctx, int enable)
{
    if (!ctx) return KWG_ERR_INVALID;
    ctx->profiling = enable != 0;
    ctx->events_used = 0;
    return KWG_OK;
}

int kwg_profile_read(kwg_ctx* ctx, double* solve_ms, int* solve_launches, double* solve_bytes)
{
    if (!ctx) return KWG_ERR_INVALID;
    double total = 0., bytes = 0.;
    for (size_t i = 0; i < ctx->events_used; ++i) {
        KWG_CUDA(ctx, cudaEventSynchronize(ctx->events[i].stop));
        float ms = 0.f;
        KWG_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->events[i].start, ctx->events[i].stop));
        total += ms;
    }
    KWG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    KWG_CUDA(ctx, cudaDeviceSynchronize());
    for (size_t i = 0; i < ctx->events_used; ++i) bytes += (double)*ctx->events[i].bytes;
    if (solve_ms) *solve_ms = total;
    if (solve_launches) *solve_launches = (int)ctx->events_used;
    if (solve_bytes) *solve_bytes = bytes;
    ctx->events_used = 0;
    return KWG_OK;
}

int kwg_fd1d_price(kwg_ctx* ctx, const kwg_option* opts, size_t n, const kwg_fd1d_params* p, double* prices,
                   int32_t* status)
{
    return price_host(ctx, opts, n, p, prices, status, false);
}

int kwg_fd1d_bs_price(kwg_ctx* ctx, const kwg_option* opts, size_t n, const kwg_fd1d_params* p, double* prices,
                      int32_t* status)
{
    return price_host(ctx, opts, n, p, prices, status, true);
}

int kwg_selftest_waits(kwg_ctx* ctx, int32_t* timed_out, int32_t* completed)
{
    if (!ctx || !timed_out || !completed) return KWG_ERR_INVALID;
    ctx->err.clear();
    KWG_CUDA(ctx, cudaSetDevice(ctx->device));
    if (int rc = ensure_device(ctx, &ctx->d_io, &ctx->io_bytes, 2 * sizeof(int32_t))) return rc;
    int32_t* d = (int32_t*)ctx->d_io;
    KWG_CUDA(ctx, cudaMemsetAsync(d, 0xff, 2 * sizeof(int32_t), ctx->stream));
    selftest_waits<<<1, 32, 0, ctx->stream>>>(d, 4096u);
    KWG_CUDA(ctx, cudaGetLastError());
    int32_t h[2] = {-1, -1};
    KWG_CUDA(ctx, cudaMemcpyAsync(h, d, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
    KWG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *timed_out = h[0];
    *completed = h[1];
    return KWG_OK;
}

size_t kwg_fd1d_dedup(const kwg_option* opts, const int32_t* x_dims, const int32_t* t_dims, size_t n,
                      int32_t* asset2pde, uint32_t* pde2asset)
{
    if (!opts || !asset2pde || n == 0) return 0;
    std::vector<int32_t> a2p;
    std::vector<uint32_t> p2a;
    const size_t m = kwg::dedup_host(opts, n, x_dims && t_dims ? x_dims : nullptr, x_dims && t_dims ? t_dims : nullptr,
                                     a2p, p2a);
    std::memcpy(asset2pde, a2p.data(), n * sizeof(int32_t));
    if (pde2asset) std::memcpy(pde2asset, p2a.data(), m * sizeof(uint32_t));
    return m;
}

int kwg_autotune_ex(kwg_ctx* ctx, const kwg_fd1d_params* p, size_t m, kwg_tuning* out)
{
    if (!ctx) return KWG_ERR_INVALID;
    ctx->err.clear();
    if (int rc = check_params(ctx, p)) return rc;
    if (m == 0 || m > (size_t)INT32_MAX / 4) return set_err(ctx, KWG_ERR_INVALID, "kwg_autotune: bad batch size");
    const std::vector<kwg_option> opts = tuning_batch(m);
    std::vector<double> prices(m);
    const bool pcr_ok = kwg::fd1d_pcr64_nodes_per_lane(p->x_dim) > 0;
    const kwg_ctx::Tuned best = tune(ctx, p, pcr_ok, [&](const kwg_fd1d_params& q) {
        return kwg_fd1d_price(ctx, opts.data(), m, &q, prices.data(), nullptr);
    }, out);
    ctx->tuned[tune_key(p->precision, p->x_dim, p->t_dim, (int)m)] = best;
    ctx->err.clear();
    return KWG_OK;
}

int kwg_autotune(kwg_ctx* ctx, const kwg_fd1d_params* p, size_t m, double* thomas_ms, double* pcr_ms)
{
    if (thomas_ms) *thomas_ms = -1.;
    if (pcr_ms) *pcr_ms = -1.;
    if (!ctx) return KWG_ERR_INVALID;
    if (int rc = check_params(ctx, p)) return rc;
    if (p->precision != KWG_FP64) return KWG_OK;  // FP32 has one solver family
    kwg_tuning t;
    if (int rc = kwg_autotune_ex(ctx, p, m, &t)) return rc;
    double best = -1.;
    for (double v : t.thomas_ms)
        if (v >= 0. && (best < 0. || v < best)) best = v;
    if (t.spread_ms >= 0. && (best < 0. || t.spread_ms < best)) best = t.spread_ms;
    if (thomas_ms) *thomas_ms = best;
    if (pcr_ms) *pcr_ms = t.pcr_ms;
    return KWG_OK;
}

int kwg_fd1d_price_device(kwg_ctx* ctx, const kwg_option* d_opts, size_t n, const kwg_fd1d_params* p,
                          double* d_prices, int32_t* d_status, void* stream_)
{
    if (!ctx) return KWG_ERR_INVALID;
    ctx->err.clear();
    ctx->launches = 0;
    if (int rc = check_params(ctx, p)) return rc;
    if (p->strict)
        return set_err(ctx, KWG_ERR_INVALID,
                       "kwg_fd1d_price_device: strict mode applies to the blocking host calls only; this call is "
                       "asynchronous, so read d_status (or use kwg_fd1d_price)");
    if (n == 0) return KWG_OK;
    if (!d_opts || !d_prices) return set_err(ctx, KWG_ERR_INVALID, "kwg: null options or prices");
    if (n > (size_t)INT32_MAX / 2) return set_err(ctx, KWG_ERR_INVALID, "kwg: batch too large");
    KWG_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t stream = stream_ ? (cudaStream_t)stream_ : ctx->stream;
    const size_t n_pad = (n + kwg::kTile - 1) / kwg::kTile * kwg::kTile;
    if (p->device_dedup) return price_device_dedup(ctx, d_opts, n, n_pad, p, d_prices, d_status, stream);
    const size_t m = n, m_pad = n_pad;
    const IoLayout L = io_layout(m, m_pad, n);
    if (int rc = ensure_device(ctx, &ctx->d_io, &ctx->io_bytes, L.total + 8 * sizeof(int))) return rc;
    char* io = (char*)ctx->d_io;
    int* counts = (int*)(io + L.total);  // [4] per-class counts, [4] cursors
    KWG_CUDA(ctx, kwg::unpack_by_class(d_opts, (int)n, counts, (double*)(io + L.t), (double*)(io + L.z),
                                       (double*)(io + L.r), (double*)(io + L.q), (double*)(io + L.s),
                                       (double*)(io + L.k), (int32_t*)(io + L.pde), (int8_t*)(io + L.w),
                                       (uint8_t*)(io + L.e), stream));
    ctx->launches += 2;
    return run_batch(ctx, io, L, (int)m, (int)n, p, d_prices, d_status, stream);
}

}  // extern "C"
