// kwg_static.cu -- the FP64 pricing call for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc.  A pricing step can be embedded in a host
// application whose device memory belongs to another allocator or is held to a
// fixed budget.  Or it can run on a latency-critical path where cudaMalloc's
// implicit device synchronisation is not allowed.  kwg_fd1d_price_device_static
// serves them: it runs the same kernels as kwg_fd1d_price_device with the Thomas
// solver (class-ordered unpack, setup, streaming solve, interpolation), but every
// byte of scratch (unpacked inputs, per-PDE status, counters, node records) lives
// in one file-scope __device__ array of fixed size.  The caller passes only its own
// inputs and outputs; the call allocates nothing and needs no kwg_ctx.
//
// Rules of use:
//   * Every GPU that loads this library holds the array (kStaticScratchBytes) until
//     the process exits.
//   * Set-up: the first call on a device looks up the array's device address with
//     that device current (cudaGetSymbolAddress) and caches it with the id of the
//     device's CUDA context.  A later call whose current context has another id (the
//     device was reset) or none yet (a host thread's first CUDA call) repeats the
//     look-up.  Make the first call on each device, and from each host thread, before
//     any stream capture.
//   * All calls share the array and it keeps the last call's contents.  Each call
//     clears what must start at zero (the class counters, the tile queue and the
//     timeout flag) and rewrites everything else.  Calls that overlap on the GPU (two
//     streams, or two host threads at once) race on the array: serialise them.
#include <cmath>
#include <cstdio>
#include <mutex>

#include <cuda_runtime.h>

#include "fd1d_kernels.h"
#include "kwg.h"

namespace {

// 64 MiB: room for about 800 options of 1024 nodes (80 bytes per option-node plus
// ~64 bytes per option), or about 1600 of 512 nodes.
constexpr size_t kStaticScratchBytes = 64ull << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

std::mutex g_mu;
struct ScratchAddr {
    void* ptr = nullptr;
    unsigned long long ctx_id = 0;  // CUDA context the address belongs to
};
ScratchAddr g_scratch[kMaxDevices];

size_t align256(size_t v) { return (v + 255) / 256 * 256; }

void put(char* err, size_t errlen, const char* msg)
{
    if (err && errlen) std::snprintf(err, errlen, "%s", msg);
}

// cuCtxGetId of the driver API (CUDA 12.0+), reached through the runtime so the
// library needs no link against libcuda; NULL asks for the current context.
using CtxGetIdFn = int (*)(void* ctx, unsigned long long* id);

CtxGetIdFn ctx_get_id()
{
    static CtxGetIdFn fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        return (CtxGetIdFn)f;
    }();
    return fn;
}

// Id of the calling thread's current context; 0 if there is none (or no driver entry).
unsigned long long current_ctx_id()
{
    unsigned long long id = 0;
    const CtxGetIdFn fn = ctx_get_id();
    if (!fn || fn(nullptr, &id) != 0) return 0;
    return id;
}

// The array's device address on the current device.  Looked up (set-up) on the
// first call for a device and again whenever the current context is not the one
// the cached address belongs to.
cudaError_t scratch_address(void** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mu);
    ScratchAddr& c = g_scratch[dev];
    const unsigned long long id = current_ctx_id();
    if (!c.ptr || id == 0 || id != c.ctx_id) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_scratch);  // makes the device's primary context current
        if (e != cudaSuccess) return e;
        c.ptr = p;
        c.ctx_id = current_ctx_id();
    }
    *out = c.ptr;
    return cudaSuccess;
}

}  // namespace

extern "C" int kwg_fd1d_price_device_static(const kwg_option* d_opts, size_t n, const kwg_fd1d_params* p,
                                            double* d_prices, int32_t* d_status, void* stream, char* err,
                                            size_t errlen)
{
    put(err, errlen, "");
    if (!p) return put(err, errlen, "kwg: null params"), KWG_ERR_INVALID;
    if (p->precision != KWG_FP64) return put(err, errlen, "kwg: the static-scratch call is FP64 only"), KWG_ERR_INVALID;
    if (p->solver != KWG_SOLVER_AUTO && p->solver != KWG_SOLVER_THOMAS)
        return put(err, errlen, "kwg: the static-scratch call uses the Thomas solver"), KWG_ERR_INVALID;
    if (p->x_dim < 3 || p->t_dim < 2) return put(err, errlen, "kwg: x_dim must be >= 3 and t_dim >= 2"), KWG_ERR_INVALID;
    if (!(p->theta > 0.) || !(p->theta <= 1.)) return put(err, errlen, "kwg: theta must be in (0, 1]"), KWG_ERR_INVALID;
    if (!(p->scale > 0.) || !std::isfinite(p->scale))
        return put(err, errlen, "kwg: scale must be positive and finite"), KWG_ERR_INVALID;
    if (!(p->density > 0.)) return put(err, errlen, "kwg: density must be positive"), KWG_ERR_INVALID;
    if (p->block_warps != 0 && p->block_warps != 1 && p->block_warps != 2 && p->block_warps != 4)
        return put(err, errlen, "kwg: block_warps must be 0, 1, 2 or 4"), KWG_ERR_INVALID;
    if (p->sm_blocks < 0 || p->sm_blocks > 64)
        return put(err, errlen, "kwg: sm_blocks must be in [0, 64]"), KWG_ERR_INVALID;
    if (p->strict)
        return put(err, errlen,
                   "kwg: strict mode applies to the blocking host calls only; this call is asynchronous, so read "
                   "d_status"),
               KWG_ERR_INVALID;
    if (p->device_dedup)
        return put(err, errlen, "kwg: the static-scratch call solves every option as its own PDE (no device_dedup)"),
               KWG_ERR_INVALID;
    if (n == 0) return KWG_OK;
    if (!d_opts || !d_prices) return put(err, errlen, "kwg: null options or prices"), KWG_ERR_INVALID;

    // scratch layout: SoA inputs | per-PDE status | class counters | solver counters | node records
    const size_t m = n, m_pad = (m + kwg::kTile - 1) / kwg::kTile * kwg::kTile;
    const bool huge = n > kStaticScratchBytes;  // cannot fit; also keeps the sums below from overflowing
    const size_t need = huge ? SIZE_MAX
                             : 6 * align256(n * 8) + align256(n * 4) + 2 * align256(n) + align256(m_pad * 4) +
                                   2 * 256 + kwg::fd1d_fp64_work_bytes((int)m_pad, p->x_dim);
    if (huge || need > kStaticScratchBytes) {
        char msg[256];
        std::snprintf(msg, sizeof msg,
                      "kwg: %zu options x %d nodes need %zu bytes of scratch; the static-scratch call has %zu "
                      "(about 80 bytes per option and node)",
                      n, p->x_dim, need, kStaticScratchBytes);
        put(err, errlen, msg);
        return KWG_ERR_INVALID;
    }
    void* base = nullptr;
    if (cudaError_t e = scratch_address(&base); e != cudaSuccess) {
        put(err, errlen, cudaGetErrorString(e));
        return KWG_ERR_CUDA;
    }
    char* s = (char*)base;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        char* at = s + o;
        o += align256(bytes);
        return at;
    };
    double* t = (double*)take(n * 8);
    double* z = (double*)take(n * 8);
    double* r = (double*)take(n * 8);
    double* q = (double*)take(n * 8);
    double* sp = (double*)take(n * 8);
    double* k = (double*)take(n * 8);
    int32_t* pde = (int32_t*)take(n * 4);
    int8_t* w = (int8_t*)take(n);
    uint8_t* e = (uint8_t*)take(n);
    int32_t* pde_status = (int32_t*)take(m_pad * 4);
    int* classes = (int*)take(8 * sizeof(int));
    int* counters = (int*)take(4 * sizeof(int));
    double* rec = (double*)(s + o);

    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaError_t ce = kwg::unpack_by_class(d_opts, (int)n, classes, t, z, r, q, sp, k, pde, w, e, st);
        ce != cudaSuccess) {
        put(err, errlen, cudaGetErrorString(ce));
        return KWG_ERR_CUDA;
    }

    kwg::PdeBatch b;
    b.t = t;
    b.z = z;
    b.r = r;
    b.q = q;
    b.w = w;
    b.e = e;
    b.m = (int)m;
    b.m_pad = (int)m_pad;
    kwg::AssetBatch a;
    a.s = sp;
    a.k = k;
    a.pde = pde;
    a.n = (int)n;
    kwg::Fd1dShape sh;
    sh.x_dim = p->x_dim;
    sh.t_dim = p->t_dim;
    sh.theta = p->theta;
    sh.c = (1. - p->theta) / p->theta;
    sh.scale = p->scale;
    sh.uniform = std::isinf(p->density);
    sh.density = sh.uniform ? 1. : p->density;
    sh.block_warps = p->block_warps ? p->block_warps : 1;
    sh.sm_blocks = p->sm_blocks;
    const int blocks = kwg::fd1d_fp64_solve_blocks((int)(m_pad / kwg::kTile), dev, sh.block_warps, sh.sm_blocks);
    kwg::fd1d_fp64_launch(b, a, sh, rec, pde_status, counters, d_prices, d_status, blocks, st, nullptr);
    if (cudaError_t ce = cudaGetLastError(); ce != cudaSuccess) {
        put(err, errlen, cudaGetErrorString(ce));
        return KWG_ERR_CUDA;
    }
    return KWG_OK;
}
