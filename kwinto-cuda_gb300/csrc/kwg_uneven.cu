// kwg_uneven.cu -- kwg_fd1d_price_uneven: a batch in which every option has its own
// x-grid size and number of time levels.
//
// The reference prices one grid shape per Fd1d_Pricer::init (src/Pricer/kwFd1d.cpp:
// 15-16), so a mixed portfolio needs one call per shape.  Here the whole batch is
// one pass over the device:
//   * dedup by (t, r, q, z, e, w, x_dim, t_dim), like src/Pricer/kwFd1d.cpp:28-65
//     with the grid added to the key;
//   * FP64 (thread per option): PDEs of equal x_dim are packed 32 to a tile, sorted
//     by t_dim so that the lanes of a tile finish together, and all tiles run in ONE
//     persistent launch whose queue hands out the longest tiles first; each lane
//     steps its own t_dim - 1 times;
//   * warp-per-option solvers (FP32, or FP64 with KWG_SOLVER_PCR): one launch per
//     nodes-per-lane bucket, each PDE with its own x_dim and t_dim;
//   * the device sequence (H2D copy, kernels, D2H copy) is captured once into a CUDA
//     graph and replayed while the batch layout stays the same.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <tuple>
#include <vector>

#include <cuda_runtime.h>

#include "fd1d_kernels.h"
#include "host_dedup.h"
#include "kwg.h"
#include "kwg_ctx.h"

using namespace kwgi;

namespace {

struct UnevenLayout {
    size_t t, z, r, q, px, pt, w, e, s, k, pde, tiles, rows, in_bytes;
    size_t prices, status, out_bytes, pde_status, total;
};

UnevenLayout uneven_layout(size_t m, size_t n, size_t ntiles)
{
    UnevenLayout L;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o = align_up(o + bytes, 256);
        return at;
    };
    L.t = take(m * 8);
    L.z = take(m * 8);
    L.r = take(m * 8);
    L.q = take(m * 8);
    L.px = take(m * 4);
    L.pt = take(m * 4);
    L.w = take(m);
    L.e = take(m);
    L.s = take(n * 8);
    L.k = take(n * 8);
    L.pde = take(n * 4);
    L.tiles = take(ntiles * sizeof(kwg::TileDesc));
    L.rows = take(m * sizeof(long long));
    L.in_bytes = o;
    L.prices = take(n * 8);
    L.status = take(n * 4);
    L.out_bytes = o - L.prices;
    L.pde_status = take(m * 4);
    L.total = o;
    return L;
}

uint64_t mix(uint64_t h, uint64_t v)
{
    h ^= v + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
    return h;
}

}  // namespace

extern "C" int kwg_fd1d_price_uneven(kwg_ctx* ctx, const kwg_option* opts, const int32_t* x_dims,
                                     const int32_t* t_dims, size_t n, const kwg_fd1d_params* p, double* prices,
                                     int32_t* status)
{
    if (!ctx) return KWG_ERR_INVALID;
    ctx->err.clear();
    ctx->launches = 0;
    if (!p) return set_err(ctx, KWG_ERR_INVALID, "kwg: null params");
    if (n == 0) return KWG_OK;
    if (!opts || !x_dims || !t_dims || !prices)
        return set_err(ctx, KWG_ERR_INVALID, "kwg: null options, grid sizes or prices");
    if (n > (size_t)INT32_MAX / 4) return set_err(ctx, KWG_ERR_INVALID, "kwg: batch too large");
    int x_max = 0, t_max = 0;
    for (size_t i = 0; i < n; ++i) {
        if (x_dims[i] < 3 || t_dims[i] < 2) {
            char msg[160];
            std::snprintf(msg, sizeof msg, "kwg: option %zu: x_dim must be >= 3 and t_dim >= 2 (got %d, %d)", i,
                          x_dims[i], t_dims[i]);
            return set_err(ctx, KWG_ERR_INVALID, msg);
        }
        x_max = std::max(x_max, (int)x_dims[i]);
        t_max = std::max(t_max, (int)t_dims[i]);
    }
    kwg_fd1d_params q = *p;
    q.x_dim = x_max;
    q.t_dim = t_max;
    if (int rc = check_params(ctx, &q)) return rc;
    // launch choices: the explicit ones, else what kwg_autotune_uneven recorded for
    // uneven batches of this precision and size, else Thomas with one warp per block
    // (FP64) and one warp per option (FP32)
    kwg_ctx::Tuned tn;
    {
        const auto it = ctx->tuned.find(tune_key(q.precision, 0, 0, (long long)n));
        if (it != ctx->tuned.end()) {
            tn = it->second;
            if (q.precision == KWG_FP64 && q.solver == KWG_SOLVER_AUTO &&
                (tn.solver != KWG_SOLVER_PCR || kwg::fd1d_pcr64_nodes_per_lane(x_max) > 0))
                q.solver = tn.solver;
        }
        if (q.block_warps || q.sm_blocks) {
            if (q.block_warps) tn.block_warps = q.block_warps;
            tn.sm_blocks = q.sm_blocks;
        }
        if (q.option_warps) tn.option_warps = q.option_warps;
    }
    const bool pcr = q.precision == KWG_FP32 || q.solver == KWG_SOLVER_PCR;
    KWG_CUDA(ctx, cudaSetDevice(ctx->device));

    // 1. dedup by (t, r, q, z, e, w, x_dim, t_dim)
    std::vector<int32_t> asset2pde;
    std::vector<uint32_t> pde2asset;
    const size_t m = kwg::dedup_host(opts, n, x_dims, t_dims, asset2pde, pde2asset);
    auto xd = [&](size_t pde) { return x_dims[pde2asset[pde]]; };
    auto td = [&](size_t pde) { return t_dims[pde2asset[pde]]; };

    // 2. layout: slot order and (Thomas) tiles or (PCR) nodes-per-lane buckets
    std::vector<uint32_t> slot_pde;          // slot -> PDE (replicas pad Thomas tiles)
    std::vector<int32_t> pde_slot(m, -1);    // PDE -> its first slot
    std::vector<kwg::TileDesc> tiles;
    std::vector<long long> rows;
    std::vector<std::pair<int, int>> buckets;  // PCR: [begin, end) slot ranges per bucket
    std::vector<int> bucket_x;
    std::vector<bool> bucket_full;
    long long node_lanes = 0;
    // PDEs in layout order: sorted on one packed integer key per PDE (ties by PDE
    // number, so the layout is deterministic)
    std::vector<uint32_t> by(m);
    auto sort_by = [&](auto packed_key) {
        std::vector<std::pair<uint64_t, uint32_t>> kv(m);
        for (size_t i = 0; i < m; ++i) kv[i] = {packed_key((uint32_t)i), (uint32_t)i};
        kwg::radix_sort_pairs(kv);
        for (size_t i = 0; i < m; ++i) by[i] = kv[i].second;
    };
    if (!pcr) {
        // x_dim ascending, t_dim descending
        sort_by([&](uint32_t p) { return (uint64_t)(uint32_t)xd(p) << 32 | (uint32_t)(INT32_MAX - td(p)); });
        struct Chunk {
            size_t begin, count;
            int x, tmax;
        };
        std::vector<Chunk> chunks;
        for (size_t i = 0; i < m;) {
            size_t j = i;
            while (j < m && xd(by[j]) == xd(by[i])) ++j;
            for (size_t c = i; c < j; c += kwg::kTile) {
                const size_t cnt = std::min((size_t)kwg::kTile, j - c);
                chunks.push_back({c, cnt, xd(by[c]), td(by[c])});  // sorted: first has the largest t_dim
            }
            i = j;
        }
        std::stable_sort(chunks.begin(), chunks.end(), [](const Chunk& a, const Chunk& b) {
            return (long long)a.x * (a.tmax - 1) > (long long)b.x * (b.tmax - 1);
        });
        for (const Chunk& c : chunks) {
            tiles.push_back(kwg::TileDesc{c.x, c.tmax, node_lanes});
            node_lanes += (long long)kwg::kTile * c.x;
            for (int l = 0; l < kwg::kTile; ++l) {
                const uint32_t pde = by[c.begin + std::min((size_t)l, c.count - 1)];
                if (pde_slot[pde] < 0) pde_slot[pde] = (int32_t)slot_pde.size();
                slot_pde.push_back(pde);
            }
        }
    } else {
        auto mlane = [&](uint32_t pde) {
            return q.precision == KWG_FP32 ? kwg::fd1d_fp32_nodes_per_lane(xd(pde))
                                           : kwg::fd1d_pcr64_nodes_per_lane(xd(pde));
        };
        // nodes per lane ascending, node-steps descending (x_dim <= 2048 here, so
        // node-steps < 2^43)
        sort_by([&](uint32_t p) {
            const uint64_t work = (uint64_t)xd(p) * (uint64_t)(td(p) > 1 ? td(p) - 1 : 0);
            return (uint64_t)(mlane(p) + 1) << 50 | (((1ull << 50) - 1) - work);
        });
        long long off = 0;
        for (size_t i = 0; i < m; ++i) {
            const uint32_t pde = by[i];
            pde_slot[pde] = (int32_t)i;
            slot_pde.push_back(pde);
            rows.push_back(off);
            off += xd(pde);
            const bool full = (int)xd(pde) == kwg::kTile * mlane(pde);
            if (i == 0 || mlane(pde) != mlane(by[i - 1])) {
                buckets.push_back({(int)i, (int)i + 1});
                bucket_x.push_back(xd(pde));
                bucket_full.push_back(full);
            } else {
                buckets.back().second = (int)i + 1;
                bucket_x.back() = std::max(bucket_x.back(), (int)xd(pde));
                bucket_full.back() = bucket_full.back() && full;
            }
        }
        node_lanes = off;  // rows of final values, in doubles
    }
    const size_t ms = slot_pde.size();

    // 3. pack inputs into pinned memory
    const UnevenLayout L = uneven_layout(ms, n, tiles.size());
    if (int rc = ensure_host(ctx, &ctx->h_io, &ctx->h_io_bytes, L.total)) return rc;
    const size_t wbytes = pcr ? (size_t)node_lanes * sizeof(double)
                              : kwg::fd1d_fp64_work_bytes_nl((int)ms, node_lanes);
    // the graph bakes in device addresses: grow buffers before deciding on replay
    if (int rc = ensure_device(ctx, &ctx->d_io, &ctx->io_bytes, L.total)) return rc;
    if (int rc = ensure_device(ctx, &ctx->d_work, &ctx->work_bytes, wbytes)) return rc;
    char* h = (char*)ctx->h_io;
    for (size_t sl = 0; sl < ms; ++sl) {
        const kwg_option& o = opts[pde2asset[slot_pde[sl]]];
        ((double*)(h + L.t))[sl] = o.t;
        ((double*)(h + L.z))[sl] = o.z;
        ((double*)(h + L.r))[sl] = o.r;
        ((double*)(h + L.q))[sl] = o.q;
        ((int32_t*)(h + L.px))[sl] = xd(slot_pde[sl]);
        ((int32_t*)(h + L.pt))[sl] = td(slot_pde[sl]);
        ((int8_t*)(h + L.w))[sl] = o.w;
        ((uint8_t*)(h + L.e))[sl] = o.e;
    }
    for (size_t i = 0; i < n; ++i) {
        ((double*)(h + L.s))[i] = opts[i].s;
        ((double*)(h + L.k))[i] = opts[i].k;
        ((int32_t*)(h + L.pde))[i] = pde_slot[asset2pde[i]];
    }
    if (!tiles.empty()) std::memcpy(h + L.tiles, tiles.data(), tiles.size() * sizeof(kwg::TileDesc));
    if (!rows.empty()) std::memcpy(h + L.rows, rows.data(), rows.size() * sizeof(long long));

    // 4. the device sequence, as a CUDA graph when not profiling
    char* io = (char*)ctx->d_io;
    kwg::PdeBatch b;
    b.t = (const double*)(io + L.t);
    b.z = (const double*)(io + L.z);
    b.r = (const double*)(io + L.r);
    b.q = (const double*)(io + L.q);
    b.w = (const int8_t*)(io + L.w);
    b.e = (const uint8_t*)(io + L.e);
    b.m = (int)ms;
    b.m_pad = (int)ms;
    kwg::AssetBatch a;
    a.s = (const double*)(io + L.s);
    a.k = (const double*)(io + L.k);
    a.pde = (const int32_t*)(io + L.pde);
    a.n = (int)n;
    kwg::Fd1dShape sh = make_shape(&q);
    sh.block_warps = tn.block_warps;
    sh.option_warps = tn.option_warps;
    sh.sm_blocks = tn.sm_blocks;
    sh.pde_x = (const int32_t*)(io + L.px);
    sh.pde_t = (const int32_t*)(io + L.pt);
    if (!pcr) {
        sh.tiles = (const kwg::TileDesc*)(io + L.tiles);
        sh.node_lanes = node_lanes;
    } else {
        sh.row_off = (const long long*)(io + L.rows);
    }
    double* d_prices = (double*)(io + L.prices);
    int32_t* d_status = (int32_t*)(io + L.status);
    int32_t* d_pde_status = (int32_t*)(io + L.pde_status);

    auto enqueue = [&](cudaStream_t st) -> int {
        int launches = 0;
        cudaMemcpyAsync(ctx->d_io, ctx->h_io, L.in_bytes, cudaMemcpyHostToDevice, st);
        if (!pcr) {
            const int blocks = kwg::fd1d_fp64_solve_blocks((int)tiles.size(), ctx->device, sh.block_warps,
                                                         sh.sm_blocks);
            launches += kwg::fd1d_fp64_launch(b, a, sh, (double*)ctx->d_work, d_pde_status, ctx->d_counter, d_prices,
                                              d_status, blocks, st, ctx->next_events());
        } else {
            for (size_t bi = 0; bi < buckets.size(); ++bi) {
                const int beg = buckets[bi].first, end = buckets[bi].second;
                kwg::PdeBatch sb = b;
                sb.t += beg;
                sb.z += beg;
                sb.r += beg;
                sb.q += beg;
                sb.w += beg;
                sb.e += beg;
                sb.m = sb.m_pad = end - beg;
                kwg::Fd1dShape ss = sh;
                ss.x_dim = bucket_x[bi];
                ss.full_lanes = bucket_full[bi];
                ss.pde_x += beg;
                ss.pde_t += beg;
                ss.row_off += beg;
                kwg::AssetBatch none = a;
                none.n = 0;
                const int r = q.precision == KWG_FP32
                                  ? kwg::fd1d_fp32_launch(sb, none, ss, (double*)ctx->d_work, d_pde_status + beg,
                                                          ctx->d_counter, d_prices, d_status, ctx->device, st,
                                                          ctx->next_events())
                                  : kwg::fd1d_pcr64_launch(sb, none, ss, (double*)ctx->d_work, d_pde_status + beg,
                                                           ctx->d_counter, d_prices, d_status, ctx->device, st,
                                                           ctx->next_events());
                if (r < 0) return -1;
                launches += r;
            }
            kwg::fd1d_interp_rows<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(b, a, sh, (double*)ctx->d_work,
                                                                               d_pde_status, d_prices, d_status);
            ++launches;
        }
        cudaMemcpyAsync(h + L.prices, io + L.prices, L.out_bytes, cudaMemcpyDeviceToHost, st);
        return launches;
    };

    uint64_t sig = 0x5eed;
    for (uint64_t v : {(uint64_t)q.precision, (uint64_t)pcr, (uint64_t)sh.block_warps, (uint64_t)sh.option_warps,
                       (uint64_t)sh.sm_blocks,
                       (uint64_t)n, (uint64_t)ms, (uint64_t)tiles.size(),
                       (uint64_t)node_lanes, (uint64_t)(uintptr_t)ctx->d_io, (uint64_t)(uintptr_t)ctx->d_work,
                       (uint64_t)(uintptr_t)ctx->h_io})
        sig = mix(sig, v);
    for (double v : {q.theta, q.scale, q.density}) {
        uint64_t u;
        std::memcpy(&u, &v, 8);
        sig = mix(sig, u);
    }
    for (size_t bi = 0; bi < buckets.size(); ++bi)
        sig = mix(mix(mix(mix(sig, (uint64_t)buckets[bi].first), (uint64_t)buckets[bi].second), (uint64_t)bucket_x[bi]),
                  (uint64_t)bucket_full[bi]);

    if (ctx->profiling) {
        const int r = enqueue(ctx->stream);
        if (r < 0) return set_err(ctx, KWG_ERR_INVALID, "kwg: grid too large for the chosen solver");
        ctx->launches += r;
        KWG_CUDA(ctx, cudaGetLastError());
    } else {
        if (!ctx->graph_exec || ctx->graph_sig != sig) {
            if (ctx->graph_exec) {
                cudaGraphExecDestroy(ctx->graph_exec);
                ctx->graph_exec = nullptr;
            }
            cudaGraph_t graph = nullptr;
            KWG_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
            const int r = enqueue(ctx->stream);
            const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
            if (r < 0) {
                if (graph) cudaGraphDestroy(graph);
                return set_err(ctx, KWG_ERR_INVALID, "kwg: grid too large for the chosen solver");
            }
            if (ce != cudaSuccess) return cuda_err(ctx, ce, "cudaStreamEndCapture");
            const cudaError_t ie = cudaGraphInstantiate(&ctx->graph_exec, graph, 0);
            cudaGraphDestroy(graph);
            if (ie != cudaSuccess) return cuda_err(ctx, ie, "cudaGraphInstantiate");
            ctx->graph_sig = sig;
            ctx->graph_launches = r;
        }
        KWG_CUDA(ctx, cudaGraphLaunch(ctx->graph_exec, ctx->stream));
        ctx->launches += ctx->graph_launches;
    }
    KWG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));

    // 5. results and strict mode
    const double* hp = (const double*)(h + L.prices);
    const int32_t* hs = (const int32_t*)(h + L.status);
    std::memcpy(prices, hp, n * sizeof(double));
    if (status) std::memcpy(status, hs, n * sizeof(int32_t));
    if (p->strict) {
        for (size_t i = 0; i < n; ++i) {
            if (hs[i] == KWG_STATUS_OK) continue;
            char msg[256];
            std::snprintf(msg, sizeof msg, "Fd1dGpu_Pricer::price: asset %zu: %s", i,
                          hs[i] == KWG_STATUS_OUT_OF_GRID ? "not in grid range" : "failed");
            return set_err(ctx, hs[i] == KWG_STATUS_OUT_OF_GRID ? KWG_ERR_OUT_OF_GRID : KWG_ERR_SOLVER, msg);
        }
    }
    return KWG_OK;
}

extern "C" int kwg_autotune_uneven(kwg_ctx* ctx, const kwg_option* opts, const int32_t* x_dims,
                                   const int32_t* t_dims, size_t n, const kwg_fd1d_params* p, kwg_tuning* out)
{
    if (!ctx) return KWG_ERR_INVALID;
    ctx->err.clear();
    if (!p || !opts || !x_dims || !t_dims || n == 0 || n > (size_t)INT32_MAX / 4)
        return set_err(ctx, KWG_ERR_INVALID, "kwg_autotune_uneven: bad arguments");
    int x_max = 0;
    for (size_t i = 0; i < n; ++i) x_max = std::max(x_max, (int)x_dims[i]);
    std::vector<double> prices(n);
    const bool pcr_ok = kwg::fd1d_pcr64_nodes_per_lane(x_max) > 0;
    const kwg_ctx::Tuned best = tune(ctx, p, pcr_ok, [&](const kwg_fd1d_params& q) {
        return kwg_fd1d_price_uneven(ctx, opts, x_dims, t_dims, n, &q, prices.data(), nullptr);
    }, out);
    ctx->tuned[tune_key(p->precision, 0, 0, (long long)n)] = best;
    ctx->err.clear();
    return KWG_OK;
}
