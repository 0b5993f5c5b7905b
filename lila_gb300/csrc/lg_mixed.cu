// lg_mixed.cu -- split-precision (Ozaki-style) FP64-grade products on the
// BF16 tensor cores (tcgen05, FP32 accumulation in TMEM).
#include "lg_common.cuh"
#include "lg_tc.cuh"
#include "../../include/lila_prim.h"

namespace lg {

// One-tile check of the tcgen05 path: D(128 x N) = A(128 x 64) * B(N x 64)^T,
// BF16 in, FP32 out, one CTA of 128 threads.  `swap` exchanges the two
// descriptor strides (used only to diagnose the layout convention).
__global__ void __launch_bounds__(128)
    k_tc_selftest(const __nv_bfloat16 *A, const __nv_bfloat16 *B, float *D, int N, int swap, int *status)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sA = smem;           // 128 x 64 BF16 = 16 KB
    uint8_t *sB = smem + 16384;   // up to 256 x 64 BF16 = 32 KB
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    const uint32_t LBO = 128, SBO = 1024;
    const int tid = threadIdx.x, warp = tid / 32;
    for (int idx = tid; idx < 128 * 64; idx += 128) {
        int r = idx / 64, k = idx % 64;
        *(__nv_bfloat16 *)(sA + tc::kmajor_off(r, k, LBO, SBO)) = A[idx];
    }
    for (int idx = tid; idx < N * 64; idx += 128) {
        int r = idx / 64, k = idx % 64;
        *(__nv_bfloat16 *)(sB + tc::kmajor_off(r, k, LBO, SBO)) = B[idx];
    }
    if (tid == 0) {
        tc::mbar_init(&mbar, 1);
        tc::fence_mbar_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(&tmem_base, 256);
        tc::tmem_relinquish();
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = tmem_base;
    if (tid == 0) {
        const uint32_t idesc = tc::idesc_bf16_f32(128, N);
        const uint32_t lbo = swap ? SBO : LBO, sbo = swap ? LBO : SBO;
        for (int kk = 0; kk < 4; kk++) {
            uint64_t ad = tc::desc_nosw(tc::smem_u32(sA) + kk * 2 * LBO, lbo, sbo);
            uint64_t bd = tc::desc_nosw(tc::smem_u32(sB) + kk * 2 * LBO, lbo, sbo);
            tc::mma_bf16(tbase, ad, bd, idesc, kk > 0 ? 1u : 0u);
        }
        tc::mma_commit(&mbar);
    }
    const bool ok = tc::mbar_wait(&mbar, 0);
    if (!ok && (tid % 32) == 0) atomicOr(status, ST_WAIT_TIMEOUT);
    tc::fence_after_sync();
    if (ok) {
        const int row = warp * 32 + (tid % 32);
        for (int c0 = 0; c0 < N; c0 += 32) {
            uint32_t r[32];
            tc::tmem_ld32(tbase + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, r);
            tc::tmem_ld_wait();
            for (int j = 0; j < 32; j++) D[(size_t)row * N + c0 + j] = __uint_as_float(r[j]);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, 256);
}

}  // namespace lg

using namespace lg;

extern "C" int lila_prim_tc_selftest(const void *A, const void *B, float *D, int N, int swap)
{
    if (N < 16 || N > 256 || (N % 16) != 0) return -4;
    const size_t smem = 16384 + 32768;
    cudaFuncSetAttribute(k_tc_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_tc_selftest<<<1, 128, smem, stream()>>>((const __nv_bfloat16 *)A, (const __nv_bfloat16 *)B, D, N, swap,
                                              status_ptr());
    note_launch("tc_selftest");
    return 0;
}
