// lg_tc.cuh -- Blackwell 5th-generation tensor core (tcgen05) helpers, inline PTX.
//
// Operands live in shared memory in the canonical K-major, no-swizzle layout:
// "core matrices" of 8 rows x 16 bytes (8 BF16 along K), element (r, k) of a
// tile at byte offset (r/8)*SBO + (k/8)*LBO + (r%8)*16 + (k%8)*2, where LBO is
// the byte stride between core matrices adjacent along K and SBO the stride
// between core matrices adjacent along M (or N).  One tcgen05.mma of
// kind::f16 consumes K = 16 (two core matrices along K); the descriptor start
// address advances by 2*LBO per K step.  Accumulators (FP32) live in tensor
// memory (TMEM): for M = 128, row i of D is TMEM lane i, column j is TMEM
// column base + j.
//
// Every wait is bounded (iteration and clock limits); a wait that gives up
// returns false so the caller can flag ST_WAIT_TIMEOUT, free its TMEM and
// return instead of hanging.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace lg {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: no swizzle, K-major.
__device__ __forceinline__ uint64_t desc_nosw(uint32_t saddr, uint32_t lbo_bytes, uint32_t sbo_bytes)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo_bytes >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo_bytes >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version of the sm_100 family
    return d;                // base offset 0, absolute LBO mode, layout type 0 (no swizzle)
}

// Instruction descriptor of kind::f16: BF16 x BF16 -> FP32, both operands K-major.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N)
{
    return (1u << 4)      // D format: F32
           | (1u << 7)    // A format: BF16
           | (1u << 10)   // B format: BF16
           | ((uint32_t)(N >> 3) << 17)
           | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tmem_alloc(uint32_t *smem_dst, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(smem_dst)),
                 "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void tmem_relinquish()
{
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}

// D(tmem) (+)= A(smem) * B(smem)^T-in-K-major; accumulate != 0 keeps D.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate)
{
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrive on an mbarrier once all previously issued MMAs of this thread are done.
__device__ __forceinline__ void mma_commit(uint64_t *mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                     smem_u32(mbar))
                 : "memory");
}

// One arrival on an mbarrier (release at CTA scope).
__device__ __forceinline__ void mbar_arrive(uint64_t *mbar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(mbar)) : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

// Bounded wait for the phase with the given parity to complete.  Each
// try_wait may suspend the thread (up to the hint, 20 us) until the phase
// completes, so a waiting warp takes no issue slots from the working ones.
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t parity)
{
    uint32_t addr = smem_u32(mbar);
    long long t0 = clock64();
    for (uint32_t it = 0; it < (1u << 26); ++it) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
            "selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(addr), "r"(parity), "r"(20000u)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > 4000000000LL) break;  // ~2 s at 2 GHz
    }
    return false;
}

// A bounded wait that, when it gives up, ORs `timeout_bit` into the status
// word and sets the CTA's abort flag; false at once when the flag is set.
__device__ __forceinline__ bool wait_abort(uint64_t *bar, uint32_t parity, volatile int *s_abort, int *status,
                                           int timeout_bit)
{
    if (*s_abort) return false;
    if (mbar_wait(bar, parity)) return true;
    atomicOr(status, timeout_bit);
    *s_abort = 1;
    return false;
}

// The same wait by every lane of a warp, with a warp-uniform result.
__device__ __forceinline__ bool wait_abort_warp(uint64_t *bar, uint32_t parity, volatile int *s_abort, int *status,
                                                int timeout_bit)
{
    return __all_sync(0xffffffffu, wait_abort(bar, parity, s_abort, status, timeout_bit));
}

__device__ __forceinline__ void fence_before_sync()
{
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync()
{
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}
// Make generic-proxy shared-memory writes visible to the tensor core (async proxy).
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

// 32 lanes x 32-bit, 32 consecutive columns per thread (lane = row).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32])
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
          "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
          "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
          "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
}

// 32 lanes x 32-bit, 8 consecutive columns per thread.
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr)
                 : "memory");
}

__device__ __forceinline__ void tmem_ld_wait()
{
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

// ---- TMA (cp.async.bulk.tensor) and transaction-count mbarriers ----------
// One arrival on mbar that also expects `bytes` more bytes of asynchronous
// copies to complete on it before its phase can end.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *mbar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(mbar)), "r"(bytes)
                 : "memory");
}

// 2-D tiled TMA load of the box at coordinates (x, y) of the tensor map (a
// kernel parameter declared __grid_constant__) into shared memory at dst; its
// bytes complete on mbar.  x (the innermost coordinate) times the element
// size must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const void *tmap, int x, int y, uint64_t *mbar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];\n" ::"r"(dst),
        "l"((unsigned long long)(uintptr_t)tmap), "r"(x), "r"(y), "r"(smem_u32(mbar))
        : "memory");
}

__device__ __forceinline__ void prefetch_tmap(const void *tmap)
{
    asm volatile("prefetch.tensormap [%0];\n" ::"l"((unsigned long long)(uintptr_t)tmap) : "memory");
}

// Byte offset of element (r, k) in the canonical no-swizzle K-major layout.
__host__ __device__ __forceinline__ uint32_t kmajor_off(int r, int k, uint32_t lbo, uint32_t sbo)
{
    return (uint32_t)(r >> 3) * sbo + (uint32_t)(k >> 3) * lbo + (uint32_t)(r & 7) * 16u + (uint32_t)(k & 7) * 2u;
}

}  // namespace tc
}  // namespace lg
