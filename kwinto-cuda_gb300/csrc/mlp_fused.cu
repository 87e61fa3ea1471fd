// mlp_fused.cu -- surrogate pricing in one persistent tcgen05 kernel: option in,
// price out, activations never leave the SM.
//
// One CTA per SM (256 threads: two warpgroups over one option row per thread pair)
// keeps the BF16 weights of all layers in shared memory (core-matrix layout, tc.cuh)
// for its whole life and walks 128-option tiles.  Thread t serves row t % 128; the
// first warpgroup handles accumulator columns 0..63 of its rows, the second 64..127
// (a warp reads the TMEM lanes of its rank in the warpgroup):
//   1. the first warpgroup computes each option's features and writes the split BF16
//      row (hi 0..4, lo 5..9) into the 128 x 16 input tile;
//   2. thread 0 issues the layer-1 MMA (K = 16) into a 128-column TMEM accumulator;
//      meanwhile the second warpgroup computes each option's analytic base price
//      (FP64);
//   3. layers 2-4: the epilogue reads the accumulator (tcgen05.ld), adds the bias,
//      applies SiLU and writes the activation as a BF16 pair into the hi and lo
//      128 x 128 tiles, each warpgroup its 64 columns; thread 0 then issues 8 MMAs
//      over hi and 8 over lo with the same weight operand (the GEMM path's K-doubled
//      [W | W] sums the same terms);
//   4. the layer-4 epilogue folds the 128 -> 1 head into an FP32 dot product in
//      column order (the first warpgroup sums columns 0..63, the second continues
//      from its partial over 64..127, as the GEMM path's epilogue does) and writes
//      max(intrinsic, base + K y / y_scale).
// The arithmetic matches the layer-by-layer path (mlp_gemm.cu) step for step.
// Every MMA completion wait is bounded; on a timeout the kernel sets *error, waits
// (bounded) for the MMAs in flight and frees its TMEM.
#include <atomic>
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "mlp.h"
#include "mlp_math.cuh"
#include "tc.cuh"
#include "tma.cuh"

namespace kwg {

namespace {

constexpr int kRows = 128;  // options per tile, one row per thread pair
constexpr int kThreads = 2 * kRows;
constexpr int kHalfCols = kMlpWidth / 2;  // accumulator columns per warpgroup
constexpr int kK1 = 16;     // layer-1 K: features hi 0..4, lo 5..9, zeros
constexpr uint32_t kW1Bytes = kMlpWidth * kK1 * 2;
constexpr uint32_t kWBytes = kMlpWidth * kMlpWidth * 2;
constexpr uint32_t kXBytes = kRows * kK1 * 2;
constexpr uint32_t kABytes = kRows * kMlpWidth * 2;
constexpr uint32_t kOffW1 = 0;
constexpr uint32_t kOffW = kOffW1 + kW1Bytes;  // W2, W3, W4
constexpr uint32_t kOffX = kOffW + 3 * kWBytes;
constexpr uint32_t kOffAhi = kOffX + kXBytes;
constexpr uint32_t kOffAlo = kOffAhi + kABytes;
constexpr uint32_t kOffBias = kOffAlo + kABytes;            // 4 x 128 FP32
constexpr uint32_t kOffHead = kOffBias + 4 * kMlpWidth * 4;  // 128 FP32 (BF16 head weights, widened)
constexpr uint32_t kOffY = kOffHead + kMlpWidth * 4;         // 128 FP32: head partial sums
constexpr uint32_t kOffMisc = kOffY + kRows * 4;             // mbarrier, TMEM address
constexpr uint32_t kSmemBytes = kOffMisc + 64;
constexpr uint32_t kTmemCols = 128;
static_assert(kOffX % 1024 == 0 && kOffAhi % 1024 == 0 && kOffAlo % 1024 == 0, "operand tiles 1 KB aligned");

__device__ __forceinline__ void store_core(unsigned char* base, int kc, int row, int k, const __nv_bfloat16* v8)
{
    *reinterpret_cast<uint4*>(base + tc::core_offset(row, k, kc)) = *reinterpret_cast<const uint4*>(v8);
}

}  // namespace

__global__ void __launch_bounds__(kThreads, 1)
    mlp_price_fused(const kwg_option* __restrict__ opts, int n, MlpBox box, const __nv_bfloat16* __restrict__ wb,
                    const float* __restrict__ params, float y_scale, double* __restrict__ prices,
                    uint8_t* __restrict__ inside, int* __restrict__ error)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    const int tid = threadIdx.x, warp = tid / 32;
    const int row = tid % kRows, half = tid / kRows;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + kOffMisc);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + kOffMisc + 8);
    float* bias = reinterpret_cast<float*>(sm + kOffBias);
    float* head = reinterpret_cast<float*>(sm + kOffHead);
    float* ypart = reinterpret_cast<float*>(sm + kOffY);

    // resident weights: W1 = columns 0..15 of forward slot 0 ([128][64]); W2..W4 =
    // columns 0..127 of slots 1..3 ([128][256]); biases and the head row
    for (int v = tid; v < kMlpWidth * (kK1 / 8); v += blockDim.x) {
        const int row = v / (kK1 / 8), kq = v % (kK1 / 8);
        store_core(sm + kOffW1, kK1, row, kq * 8, wb + (size_t)row * kMlpInK + kq * 8);
    }
    for (int l = 0; l < 3; ++l) {
        const __nv_bfloat16* src = wb + (size_t)(l + 1) * kMlpFwdSlot;
        for (int v = tid; v < kMlpWidth * (kMlpWidth / 8); v += blockDim.x) {
            const int row = v / (kMlpWidth / 8), kq = v % (kMlpWidth / 8);
            store_core(sm + kOffW + l * kWBytes, kMlpWidth, row, kq * 8, src + (size_t)row * kMlpHidK + kq * 8);
        }
    }
    for (int i = tid; i < 4 * kMlpWidth; i += blockDim.x) bias[i] = params[kMlpWeights + i];
    for (int i = tid; i < kMlpWidth; i += blockDim.x) head[i] = __bfloat162float(wb[4 * kMlpFwdSlot + i]);
    const float head_b = params[kMlpWeights + 4 * kMlpWidth];
    if (warp == 0) {
        tc::tmem_alloc(smem_addr(tslot), kTmemCols);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        mbar_init(mbar, 1);
        fence_mbar_init();
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;
    // this warp's 32 lanes (its rank in the warpgroup) and its warpgroup's columns
    const uint32_t tl = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(half * kHalfCols);
    const uint32_t idesc = tc::idesc_bf16_f32(kRows, kMlpWidth);
    const uint32_t sx = smem_addr(sm + kOffX), sw1 = smem_addr(sm + kOffW1), sw = smem_addr(sm + kOffW);
    const uint32_t shi = smem_addr(sm + kOffAhi), slo = smem_addr(sm + kOffAlo);
    uint32_t phase = 0;
    bool ok = true, pending = false;

    for (int tile = blockIdx.x; tile * kRows < n; tile += gridDim.x) {
        const int i = tile * kRows + row;
        const bool real = i < n;
        kwg_option o = {};
        float f[kMlpIn] = {0.f, 0.f, 0.f, 0.f, 0.f};
        bool in = false;
        if (real) {
            o = opts[i];
            features(o, box, f, in);
        }
        if (half == 0) {
            __align__(16) __nv_bfloat16 xr[kK1];
            split_features<kK1>(f, xr);
            store_core(sm + kOffX, kK1, row, 0, xr);
            store_core(sm + kOffX, kK1, row, 8, xr + 8);
        }
        tc::fence_proxy_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            tc::mma_bf16(tmem, tc::smem_desc(sx, 128, (kK1 / 8) * 128), tc::smem_desc(sw1, 128, (kK1 / 8) * 128),
                         idesc, false);
            tc::commit(smem_addr(mbar));
        }
        pending = true;
        const double base = (half == 1 && real) ? base_price(o) : 0.;  // FP64, overlapped with the MMA

        float y = 0.f, a4[kHalfCols];  // layer-4 activations of this warpgroup's columns
        for (int l = 0; l < 4; ++l) {
            ok = mbar_wait(mbar, phase) && ok;
            phase ^= 1u;
            ok = __syncthreads_and(ok);
            if (!ok) break;
            pending = false;
            tc::fence_after_sync();
#pragma unroll
            for (int cc = 0; cc < kHalfCols; cc += 32) {
                const int c = half * kHalfCols + cc;  // the accumulator column
                float v[32];
                tc::tmem_ld32(tl + (uint32_t)cc, v);
                if (l < 3) {
                    __align__(16) __nv_bfloat16 hi[32], lo[32];
#pragma unroll
                    for (int j = 0; j < 32; ++j) {
                        const float a = silu_f(v[j] + bias[l * kMlpWidth + c + j]);
                        hi[j] = __float2bfloat16(a);
                        lo[j] = __float2bfloat16(a - __bfloat162float(hi[j]));
                    }
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        store_core(sm + kOffAhi, kMlpWidth, row, c + 8 * q, hi + 8 * q);
                        store_core(sm + kOffAlo, kMlpWidth, row, c + 8 * q, lo + 8 * q);
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < 32; ++j) a4[cc + j] = silu_f(v[j] + bias[3 * kMlpWidth + c + j]);
                }
            }
            if (l == 3) {
                // the head in column order: columns 0..63, then 64..127 from that partial
                if (half == 0) {
#pragma unroll
                    for (int j = 0; j < kHalfCols; ++j) y = fmaf(head[j], a4[j], y);
                    ypart[row] = y;
                }
                __syncthreads();
                if (half == 1) {
                    y = ypart[row];
#pragma unroll
                    for (int j = 0; j < kHalfCols; ++j) y = fmaf(head[kHalfCols + j], a4[j], y);
                }
                break;
            }
            // layer l + 2: activations (hi, then lo) x W_{l+2}
            tc::fence_proxy_async_smem();
            tc::fence_before_sync();
            __syncthreads();
            if (tid == 0) {
                tc::fence_after_sync();
                const uint32_t swl = sw + (uint32_t)l * kWBytes;
#pragma unroll
                for (int kk = 0; kk < kMlpWidth / 16; ++kk)
                    tc::mma_bf16(tmem, tc::smem_desc(shi + kk * 256, 128, (kMlpWidth / 8) * 128),
                                 tc::smem_desc(swl + kk * 256, 128, (kMlpWidth / 8) * 128), idesc, kk > 0);
#pragma unroll
                for (int kk = 0; kk < kMlpWidth / 16; ++kk)
                    tc::mma_bf16(tmem, tc::smem_desc(slo + kk * 256, 128, (kMlpWidth / 8) * 128),
                                 tc::smem_desc(swl + kk * 256, 128, (kMlpWidth / 8) * 128), idesc, true);
                tc::commit(smem_addr(mbar));
            }
            pending = true;
        }
        if (!ok) break;
        if (half == 1 && real) {
            const double v = base + o.k * (double)((y + head_b) / y_scale);
            prices[i] = o.e ? fmax(v, intrinsic(o)) : v;
            if (inside) inside[i] = in ? 1 : 0;
        }
        tc::fence_before_sync();  // TMEM reads of this tile precede the next tile's MMA
    }
    if (!ok) {
        if (tid == 0 && error) atomicExch(error, 1);
        if (pending) mbar_wait(mbar, phase ^ 1u);  // let the MMAs in flight finish before TMEM is freed
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

cudaError_t mlp_prepare_device()
{
    static std::atomic<unsigned long long> done{0};
    int dev = 0;
    if (const cudaError_t e = cudaGetDevice(&dev); e != cudaSuccess) return e;
    const unsigned long long bit = 1ull << (dev & 63);
    if (done.load() & bit) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(mlp_price_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes);
    if (e == cudaSuccess) e = gemm_set_smem_limit();
    if (e == cudaSuccess) done.fetch_or(bit);
    return e;
}

cudaError_t mlp_launch_price_fused(const kwg_option* opts, int n, const MlpBox& box, const __nv_bfloat16* wb,
                                   const float* params, float y_scale, double* prices, uint8_t* inside, int* error,
                                   int sms, cudaStream_t st)
{
    if (const cudaError_t e = mlp_prepare_device(); e != cudaSuccess) return e;
    const int tiles = (n + kRows - 1) / kRows;
    const int grid = tiles < sms ? tiles : sms;
    mlp_price_fused<<<grid, kThreads, kSmemBytes, st>>>(opts, n, box, wb, params, y_scale, prices, inside, error);
    return cudaGetLastError();
}

}  // namespace kwg
