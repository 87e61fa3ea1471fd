// mlp_gemm.cu -- BF16 x BF16 -> FP32 GEMM on the tcgen05 tensor cores with a fused
// epilogue, the building block of the MLP surrogate's forward and backward passes.
//
//     acc[M][N] = A[M][K] * B[N][K]^T        (A, B row-major BF16: K contiguous)
//     z = acc + bias[n]
//     out_f32[m][n]  = z                      (or atomically += acc, for split-K)
//     out_bf16[m][n] = act(z),  out_bf16_t[n][m] = act(z)
//     out_dact[m][n] = act'(z)               (FP32; SiLU derivative for backward)
//     out_head[m]    = head_bias + sum_n head_w[n] act(z)   (FP32, fused 128 -> 1 layer)
// out_bf16 may hold the activation as a BF16 pair (hi at column n, lo at n + N).
//
// One CTA of 128 threads computes one 128 x 128 tile (blockIdx.x over M, .y over N)
// over the K range of blockIdx.z.  K is staged 64 at a time into shared memory in
// the no-swizzle core-matrix layout (tc.cuh); thread 0 issues four 128x128x16 MMAs
// per stage into a TMEM accumulator of 128 columns and commits to an mbarrier that
// every thread waits on (bounded) before the stage is refilled.  The epilogue reads
// TMEM with tcgen05.ld, 32 columns at a time, one row per thread.
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "mlp.h"
#include "tc.cuh"
#include "tma.cuh"

namespace kwg {

namespace {

constexpr int kTileM = 128, kTileN = 128, kStageK = 64;
constexpr uint32_t kStageABytes = kTileM * kStageK * 2;  // 16 KB
constexpr uint32_t kStageBBytes = kTileN * kStageK * 2;  // 16 KB
constexpr uint32_t kTmemCols = 128;

__device__ __forceinline__ float silu(float z) { return z / (1.f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z)
{
    const float s = 1.f / (1.f + __expf(-z));
    return s * (1.f + z * (1.f - s));
}

// Copies a 128 x 64 BF16 block (rows r0.., cols k0..) of a row-major matrix with
// leading dimension ld into shared memory in core-matrix layout.  Rows >= rows
// are zero-filled.
__device__ __forceinline__ void stage_block(unsigned char* dst, const __nv_bfloat16* __restrict__ src, int ld,
                                            int r0, int rows, int k0)
{
    for (int v = threadIdx.x; v < 128 * (kStageK / 8); v += blockDim.x) {
        const int row = v / (kStageK / 8), kq = v % (kStageK / 8);
        uint4 val = make_uint4(0, 0, 0, 0);
        if (r0 + row < rows) val = *reinterpret_cast<const uint4*>(src + (size_t)(r0 + row) * ld + k0 + kq * 8);
        *reinterpret_cast<uint4*>(dst + tc::core_offset(row, kq * 8, kStageK)) = val;
    }
}

}  // namespace

__global__ void __launch_bounds__(128) gemm_bf16_tn(const GemmArgs g)
{
    extern __shared__ __align__(1024) unsigned char gsm[];
    unsigned char* sa = gsm;
    unsigned char* sb = gsm + kStageABytes;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(gsm + kStageABytes + kStageBBytes);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(gsm + kStageABytes + kStageBBytes + 8);
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int m0 = blockIdx.x * kTileM, n0 = blockIdx.y * kTileN;
    const int kz0 = blockIdx.z * g.k_per_split;
    const int kz1 = min(g.K, kz0 + g.k_per_split);

    if (warp == 0) {
        tc::tmem_alloc(smem_addr(tslot), kTmemCols);
        tc::tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        mbar_init(mbar, 1);
        fence_mbar_init();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;
    const uint32_t idesc = tc::idesc_bf16_f32(kTileM, kTileN);
    bool ok = true;

    uint32_t phase = 0, last = 0;
    for (int k0 = kz0; k0 < kz1; k0 += kStageK) {
        stage_block(sa, g.A, g.lda, m0, g.M, k0);
        stage_block(sb, g.B, g.ldb, n0, g.N, k0);
        tc::fence_proxy_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) {
            tc::fence_after_sync();
#pragma unroll
            for (int kk = 0; kk < kStageK / 16; ++kk) {
                const uint64_t ad = tc::smem_desc(smem_addr(sa) + kk * 256, 128, (kStageK / 8) * 128);
                const uint64_t bd = tc::smem_desc(smem_addr(sb) + kk * 256, 128, (kStageK / 8) * 128);
                tc::mma_bf16(tmem, ad, bd, idesc, (k0 > kz0) || (kk > 0));
            }
            tc::commit(smem_addr(mbar));
        }
        ok = mbar_wait(mbar, phase) && ok;  // the stage is free again, and D is final on the last
        last = phase;
        phase ^= 1u;
        if (!__syncthreads_and(ok)) break;
    }
    if (!__syncthreads_and(ok)) mbar_wait(mbar, last);  // let MMAs in flight finish before TMEM is freed
    tc::fence_after_sync();

    if (__syncthreads_and(ok) && kz1 > kz0) {
        const int row = m0 + warp * 32 + lane;
        float head = 0.f;
        for (int c = 0; c < kTileN; c += 32) {
            float v[32];
            tc::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
            if (row >= g.M) continue;
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                const int n = n0 + c + i;
                if (n >= g.N) continue;
                const float acc = v[i];
                if (g.atomic_f32) {
                    atomicAdd(g.out_f32 + (size_t)row * g.ldo + n, acc);
                    continue;
                }
                const float z = acc + (g.bias ? g.bias[n] : 0.f);
                if (g.out_f32) g.out_f32[(size_t)row * g.ldo + n] = z;
                const float a = g.silu ? silu(z) : z;
                const __nv_bfloat16 hi = __float2bfloat16(a);
                if (g.out_bf16) {
                    g.out_bf16[(size_t)row * g.ldb16 + n] = hi;
                    if (g.split_bf16) g.out_bf16[(size_t)row * g.ldb16 + g.N + n] = __float2bfloat16(a - __bfloat162float(hi));
                }
                if (g.out_bf16_t) g.out_bf16_t[(size_t)n * g.ldt + row] = hi;
                if (g.out_dact) g.out_dact[(size_t)row * g.ldo + n] = g.silu ? dsilu(z) : 1.f;
                if (g.head_w) head = fmaf(__bfloat162float(g.head_w[n]), a, head);
            }
        }
        if (g.head_w && row < g.M) g.out_head[row] = head + *g.head_bias;
    } else if (threadIdx.x == 0 && !ok && g.error) {
        atomicExch(g.error, 1);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

// Each CTA holds 128 of an SM's 512 TMEM columns; asking for a quarter of the shared
// memory caps residency at 4 CTAs per SM, so allocations never wait on each other.
size_t gemm_smem_bytes() { return 56 * 1024; }

cudaError_t gemm_set_smem_limit()
{
    return cudaFuncSetAttribute(gemm_bf16_tn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gemm_smem_bytes());
}

cudaError_t gemm_launch(const GemmArgs& g, int splits, cudaStream_t stream)
{
    if (const cudaError_t e = mlp_prepare_device(); e != cudaSuccess) return e;
    dim3 grid((g.M + kTileM - 1) / kTileM, (g.N + kTileN - 1) / kTileN, splits);
    gemm_bf16_tn<<<grid, 128, gemm_smem_bytes(), stream>>>(g);
    return cudaGetLastError();
}

}  // namespace kwg
