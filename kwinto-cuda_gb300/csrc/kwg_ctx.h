// kwg_ctx.h -- the context behind the C ABI and the host helpers shared by the
// translation units of libkwg.so (not part of the public interface).
#pragma once

#include <cmath>
#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "fd1d_kernels.h"
#include "kwg.h"

struct kwg_ctx {
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    int launches = 0;

    // grow-only device buffers
    void* d_work = nullptr;  // coefficients + state
    size_t work_bytes = 0;
    void* d_io = nullptr;  // packed inputs / outputs
    size_t io_bytes = 0;
    int* d_counter = nullptr;  // [0] tile queue, [1] device-timeout flag, [2..3] 64-bit byte count
    // pinned host staging
    void* h_io = nullptr;
    size_t h_io_bytes = 0;
    // solve-kernel timing (kwg_set_profiling)
    // uneven batches: the captured device sequence and the layout it was built for
    cudaGraphExec_t graph_exec = nullptr;
    uint64_t graph_sig = 0;
    int graph_launches = 0;
    // autotuner decisions: shape key -> solver (KWG_SOLVER_THOMAS or KWG_SOLVER_PCR),
    // warps per block and resident blocks per SM (0: as many as fit) of the streaming
    // solver, warps per option of the FP32 solver
    struct Tuned {
        int solver = KWG_SOLVER_THOMAS;
        int block_warps = 1;
        int option_warps = 1;
        int sm_blocks = 0;
    };
    std::map<uint64_t, Tuned> tuned;
    bool profiling = false;
    std::vector<kwg::SolveEvents> events;  // pool, reused across reads
    size_t events_used = 0;

    const kwg::SolveEvents* next_events()
    {
        if (!profiling) return nullptr;
        if (events_used == events.size()) {
            kwg::SolveEvents e;
            if (cudaEventCreate(&e.start) != cudaSuccess || cudaEventCreate(&e.stop) != cudaSuccess ||
                cudaMallocHost(&e.bytes, sizeof(unsigned long long)) != cudaSuccess)
                return nullptr;
            events.push_back(e);
        }
        *events[events_used].bytes = 0;
        return &events[events_used++];
    }
};

namespace kwgi {


inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

inline int set_err(kwg_ctx* ctx, int code, const std::string& msg)
{
    if (ctx) ctx->err = msg;
    return code;
}

inline int cuda_err(kwg_ctx* ctx, cudaError_t e, const char* what)
{
    return set_err(ctx, KWG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define KWG_CUDA(ctx, call)                                   \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_err(ctx, e_, #call); \
    } while (0)

inline int ensure_device(kwg_ctx* ctx, void** buf, size_t* cap, size_t need)
{
    if (need <= *cap) return KWG_OK;
    if (*buf) cudaFree(*buf);
    *buf = nullptr;
    *cap = 0;
    cudaError_t e = cudaMalloc(buf, need);
    if (e != cudaSuccess) return cuda_err(ctx, e, "cudaMalloc");
    *cap = need;
    return KWG_OK;
}

inline int ensure_host(kwg_ctx* ctx, void** buf, size_t* cap, size_t need)
{
    if (need <= *cap) return KWG_OK;
    if (*buf) cudaFreeHost(*buf);
    *buf = nullptr;
    *cap = 0;
    cudaError_t e = cudaMallocHost(buf, need);
    if (e != cudaSuccess) return cuda_err(ctx, e, "cudaMallocHost");
    *cap = need;
    return KWG_OK;
}

inline int check_params(kwg_ctx* ctx, const kwg_fd1d_params* p)
{
    if (!p) return set_err(ctx, KWG_ERR_INVALID, "kwg: null params");
    if (p->x_dim < 3) return set_err(ctx, KWG_ERR_INVALID, "kwg: x_dim must be >= 3");
    if (p->t_dim < 2) return set_err(ctx, KWG_ERR_INVALID, "kwg: t_dim must be >= 2");
    if (!(p->theta > 0.) || !(p->theta <= 1.))
        return set_err(ctx, KWG_ERR_INVALID, "kwg: theta must be in (0, 1]");
    if (!(p->scale > 0.) || !std::isfinite(p->scale))
        return set_err(ctx, KWG_ERR_INVALID, "kwg: scale must be positive and finite");
    if (!(p->density > 0.)) return set_err(ctx, KWG_ERR_INVALID, "kwg: density must be positive");
    if (p->precision != KWG_FP64 && p->precision != KWG_FP32)
        return set_err(ctx, KWG_ERR_INVALID, "kwg: unknown precision");
    if (p->solver < KWG_SOLVER_AUTO || p->solver > KWG_SOLVER_PCR)
        return set_err(ctx, KWG_ERR_INVALID, "kwg: unknown solver");
    if (p->precision == KWG_FP64 && p->solver == KWG_SOLVER_PCR && kwg::fd1d_pcr64_nodes_per_lane(p->x_dim) < 0)
        return set_err(ctx, KWG_ERR_INVALID, "kwg: the FP64 PCR solver supports x_dim <= 1024");
    if (p->precision == KWG_FP32 && p->solver == KWG_SOLVER_THOMAS)
        return set_err(ctx, KWG_ERR_INVALID, "kwg: FP32 uses the on-chip partitioned solver (KWG_SOLVER_PCR or AUTO)");
    if (p->precision == KWG_FP32 && kwg::fd1d_fp32_nodes_per_lane(p->x_dim) < 0)
        return set_err(ctx, KWG_ERR_INVALID, "kwg: FP32 stepping supports x_dim <= 2048");
    if (p->block_warps != 0 && p->block_warps != 1 && p->block_warps != 2 && p->block_warps != 4)
        return set_err(ctx, KWG_ERR_INVALID, "kwg: block_warps must be 0, 1, 2 or 4");
    if (p->option_warps != 0 && p->option_warps != 1 && p->option_warps != 2 && p->option_warps != 4 &&
        p->option_warps != 8)
        return set_err(ctx, KWG_ERR_INVALID, "kwg: option_warps must be 0, 1, 2, 4 or 8");
    if (p->sm_blocks < 0 || p->sm_blocks > 64)
        return set_err(ctx, KWG_ERR_INVALID, "kwg: sm_blocks must be in [0, 64]");
    return KWG_OK;
}

// Autotuner key: precision, grid and the batch size rounded up to a power of two.
// Uneven batches use x_dim = t_dim = 0.
inline uint64_t tune_key(int precision, int x_dim, int t_dim, long long m)
{
    int mb = 0;
    while ((1ll << mb) < m && mb < 40) ++mb;
    return ((uint64_t)precision << 60) | ((uint64_t)(x_dim & 0xfffff) << 40) | ((uint64_t)(t_dim & 0xfffff) << 20) |
           (uint64_t)mb;
}

// Solve-kernel milliseconds of one call (after a warm-up call), or -1 on error.
template <typename F>
inline double time_solve(kwg_ctx* ctx, F&& call)
{
    if (call() != KWG_OK) return -1.;
    const bool was = ctx->profiling;
    kwg_set_profiling(ctx, 1);
    double ms = 0.;
    int cnt = 0;
    int rc = call();
    if (rc == KWG_OK) rc = kwg_profile_read(ctx, &ms, &cnt, nullptr);
    kwg_set_profiling(ctx, was);
    return rc == KWG_OK ? ms : -1.;
}

// Times every candidate launch shape on fn(params) and returns the fastest: FP64 --
// the streaming solver with 1, 2, 4 warps per block (as many blocks per SM as fit),
// with one 4-warp block per SM (one warp per scheduler), and the warp-per-PDE solver
// (when pcr_ok); FP32 -- 1, 2, 4 and 8 warps per option.
template <typename F>
inline kwg_ctx::Tuned tune(kwg_ctx* ctx, const kwg_fd1d_params* p, bool pcr_ok, F&& fn, kwg_tuning* out)
{
    kwg_tuning r = {};
    for (double& v : r.thomas_ms) v = -1.;
    r.pcr_ms = -1.;
    for (double& v : r.fp32_ms) v = -1.;
    r.spread_ms = -1.;
    r.fp32_8w_ms = -1.;
    kwg_fd1d_params q = *p;
    q.strict = 0;
    kwg_ctx::Tuned best;
    double best_ms = -1.;
    auto consider = [&](double ms, int solver, int bw, int ow, int sb) {
        if (ms >= 0. && (best_ms < 0. || ms < best_ms)) {
            best_ms = ms;
            best.solver = solver;
            best.block_warps = bw;
            best.option_warps = ow;
            best.sm_blocks = sb;
        }
    };
    if (p->precision == KWG_FP64) {
        const int bws[3] = {1, 2, 4};
        for (int i = 0; i < 3; ++i) {
            q.solver = KWG_SOLVER_THOMAS;
            q.block_warps = bws[i];
            q.sm_blocks = 0;
            r.thomas_ms[i] = time_solve(ctx, [&] { return fn(q); });
            consider(r.thomas_ms[i], KWG_SOLVER_THOMAS, bws[i], 1, 0);
        }
        q.block_warps = 4;
        q.sm_blocks = 1;
        r.spread_ms = time_solve(ctx, [&] { return fn(q); });
        consider(r.spread_ms, KWG_SOLVER_THOMAS, 4, 1, 1);
        if (pcr_ok) {
            q.solver = KWG_SOLVER_PCR;
            q.block_warps = 0;
            q.sm_blocks = 0;
            r.pcr_ms = time_solve(ctx, [&] { return fn(q); });
            consider(r.pcr_ms, KWG_SOLVER_PCR, 1, 1, 0);
        }
    } else {
        const int ws[4] = {1, 2, 4, 8};
        for (int i = 0; i < 4; ++i) {
            q.option_warps = ws[i];
            double& ms = i < 3 ? r.fp32_ms[i] : r.fp32_8w_ms;
            ms = time_solve(ctx, [&] { return fn(q); });
            consider(ms, KWG_SOLVER_PCR, 1, ws[i], 0);
        }
    }
    r.solver = best.solver;
    r.block_warps = best.block_warps;
    r.option_warps = best.option_warps;
    r.sm_blocks = best.sm_blocks;
    if (out) *out = r;
    return best;
}


inline kwg::Fd1dShape make_shape(const kwg_fd1d_params* p)
{
    kwg::Fd1dShape sh;
    sh.x_dim = p->x_dim;
    sh.t_dim = p->t_dim;
    sh.theta = p->theta;
    sh.c = (1. - p->theta) / p->theta;
    sh.scale = p->scale;
    sh.uniform = std::isinf(p->density);
    sh.density = sh.uniform ? 1. : p->density;
    return sh;
}

}  // namespace kwgi
