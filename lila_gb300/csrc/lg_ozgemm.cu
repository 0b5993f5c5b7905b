// lg_ozgemm.cu -- general FP64-grade GEMM on the BF16 tensor cores (tcgen05),
// C = alpha op(A) op(B) + beta C with the operand masks and epilogue of the
// FP64 GEMM (lg_kernels.cu), used for the large products of the factorizations
// when the library precision is LILA_PRECISION_SPLIT (lila_gpu_set_precision).
//
// Scheme (the one of lg_ozaki.cu): every row of op(A) and every column of
// op(B) is a scaling group over the CTA's K range; each value becomes eight
// balanced base-128 digits (exact BF16); digit products are accumulated per
// digit order d = s + t in eight TMEM blocks of 64 FP32 columns (all 512
// columns); a block stays an exact integer below 2^24 for K <= 128, so every
// 128 K the blocks are folded into int64 registers.  The output tile is the
// exact integer sum assembled once to FP64 (rounded to nearest).  The error of
// an entry is below 2^-50 (max|a| sum|b| + sum|a| max|b|) over its K range.
//
// CTA = 256 threads, output tile 128 x 64, K in stages of 32 through a
// two-stage SMEM ring (96 KB per stage: A digits 8 x 128 x 32 BF16, B digits
// 8 x 64 x 32), so the split of stage k+1 overlaps the MMAs of stage k.
// Split-K (grid z) writes FP64 partial products; a reduction kernel adds them
// and applies the epilogue, as the FP64 GEMM does.
#include <math.h>

#include "lg_common.cuh"
#include "lg_tc.cuh"
#include "lg_ozdigits.cuh"

namespace lg {
namespace ozg {

using oz::NS;
using oz::LBO;
constexpr int BM = 128, BN = 64, KC = 32, NSTAGE = 2, FLUSH = 4;  // fold TMEM every FLUSH * KC = 128 K
constexpr uint32_t SBO = (KC / 8) * 128;           // 512: M/N-adjacent core matrices
constexpr uint32_t A_SLICE = (BM / 8) * SBO;       // 8 KB per digit slice
constexpr uint32_t B_SLICE = (BN / 8) * SBO;       // 4 KB
constexpr uint32_t A_BYTES = NS * A_SLICE;         // 64 KB
constexpr uint32_t B_BYTES = NS * B_SLICE;         // 32 KB
constexpr uint32_t STAGE_BYTES = A_BYTES + B_BYTES;
constexpr size_t SMEM = (size_t)NSTAGE * STAGE_BYTES;  // 192 KB

// Stored element (sr, sc) of X after its structural mask, as IEEE bits.
__device__ __forceinline__ unsigned long long masked_bits(const double *p, int ld, int mask, int sr, int sc)
{
    switch (mask) {
    case M_UNIT_LOWER:
        if (sr < sc) return 0ull;
        if (sr == sc) return 0x3FF0000000000000ull;
        break;
    case M_UPPER:
        if (sr > sc) return 0ull;
        break;
    case M_LOWER:
        if (sr < sc) return 0ull;
        break;
    case M_UNIT_UPPER:
        if (sr > sc) return 0ull;
        if (sr == sc) return 0x3FF0000000000000ull;
        break;
    default:
        break;
    }
    return __double_as_longlong(p[(size_t)sr + (size_t)sc * (size_t)ld]);
}

// op(A)(r, k) and op(B)(k, c) as bits (0 outside the matrix).
__device__ __forceinline__ unsigned long long opa(const Operand &A, int M, int r, int k, int kend)
{
    if (r >= M || k >= kend) return 0ull;
    return A.trans == NT ? masked_bits(A.p, A.ld, A.mask, r, k) : masked_bits(A.p, A.ld, A.mask, k, r);
}
__device__ __forceinline__ unsigned long long opb(const Operand &B, int N, int k, int c, int kend)
{
    if (c >= N || k >= kend) return 0ull;
    return B.trans == NT ? masked_bits(B.p, B.ld, B.mask, k, c) : masked_bits(B.p, B.ld, B.mask, c, k);
}

__device__ __forceinline__ void store_unit(uint8_t *base, uint32_t slice_bytes, int idx, int kg,
                                           const uint32_t (&fl)[8][NS])
{
#pragma unroll
    for (int s = 0; s < NS; s++) {
        uint4 v;
        v.x = oz::pack_hi(fl[0][s], fl[1][s]);
        v.y = oz::pack_hi(fl[2][s], fl[3][s]);
        v.z = oz::pack_hi(fl[4][s], fl[5][s]);
        v.w = oz::pack_hi(fl[6][s], fl[7][s]);
        *(uint4 *)(base + s * slice_bytes + (idx >> 3) * SBO + kg * LBO + (idx & 7) * 16) = v;
    }
}

__device__ __forceinline__ void epi_store(double v, int r, int c, double *C, int ldc, const GemmEpi &e)
{
    if (e.upper_only && r > c) return;
    double out = e.alpha * v;
    if (e.add_diag && r == c) out += 1.0;
    const size_t off = (size_t)r + (size_t)c * (size_t)ldc;
    if (e.beta != 0.0 && r >= e.zero_rows) out += e.beta * C[off];
    C[off] = out;
}

__global__ void __launch_bounds__(256, 1)
    k_ozgemm(int M, int N, int K, int kchunk, Operand A, Operand B, double *C, int ldc, GemmEpi e, double *part,
             int *status)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t mbar[NSTAGE];
    __shared__ uint32_t tmem_base_s;
    __shared__ int s_rexp[BM], s_cexp[BN];
    __shared__ int s_abort;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int row0 = blockIdx.x * BM, col0 = blockIdx.y * BN;
    const int kbeg = blockIdx.z * kchunk;
    const int kend = min(K, kbeg + kchunk);

    if (tid == 0) {
        for (int b = 0; b < NSTAGE; b++) tc::mbar_init(&mbar[b], 1);
        tc::fence_mbar_init();
        s_abort = 0;
    }
    if (tid < BM) s_rexp[tid] = 0;
    if (tid < BN) s_cexp[tid] = 0;
    if (warp == 0) {
        tc::tmem_alloc(&tmem_base_s, 512);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = tmem_base_s;
    const uint32_t sbase = tc::smem_u32(smem);

    // ---- scaling groups over [kbeg, kend): the largest biased exponent of
    // every row of op(A) and every column of op(B); lanes run along the
    // stored contiguous dimension
    if (A.trans == NT) {
        const int r = tid & 127;
        int mx = 0;
        for (int k = kbeg + (tid >> 7); k < kend; k += 2) mx = max(mx, oz::bexp(opa(A, M, row0 + r, k, kend)));
        atomicMax(&s_rexp[r], mx);
    } else {
        for (int r = warp; r < BM; r += 8) {
            int mx = 0;
            for (int k = kbeg + lane; k < kend; k += 32) mx = max(mx, oz::bexp(opa(A, M, row0 + r, k, kend)));
            for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            if (lane == 0) s_rexp[r] = mx;
        }
    }
    if (B.trans == NT) {
        for (int c = warp; c < BN; c += 8) {
            int mx = 0;
            for (int k = kbeg + lane; k < kend; k += 32) mx = max(mx, oz::bexp(opb(B, N, k, col0 + c, kend)));
            for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            if (lane == 0) s_cexp[c] = mx;
        }
    } else {
        const int c = tid & 63;
        int mx = 0;
        for (int k = kbeg + (tid >> 6); k < kend; k += 4) mx = max(mx, oz::bexp(opb(B, N, k, col0 + c, kend)));
        atomicMax(&s_cexp[c], mx);
    }
    __syncthreads();
    if (tid < BM && s_rexp[tid] == 0x7FF) atomicOr(status, ST_NONFINITE);
    if (tid < BN && s_cexp[tid] == 0x7FF) atomicOr(status, ST_NONFINITE);

    // ---- main loop
    const int q = warp & 3, h = warp >> 2;
    long long acc_hi[32], acc_lo[32];
#pragma unroll
    for (int j = 0; j < 32; j++) {
        acc_hi[j] = 0;
        acc_lo[j] = 0;
    }
    const int nch = kend > kbeg ? (kend - kbeg + KC - 1) / KC : 0;
    uint32_t phase_bits = 0, pend = 0;
    for (int ch = 0; ch < nch; ch++) {
        const int buf = ch & 1;
        if ((pend >> buf) & 1u) {
            if (!tc::mbar_wait(&mbar[buf], (phase_bits >> buf) & 1u)) {
                if (tid == 0) atomicOr(status, ST_WAIT_TIMEOUT);
                s_abort = 1;
            }
            phase_bits ^= 1u << buf;
            pend &= ~(1u << buf);
        }
        __syncthreads();
        if (s_abort) break;
        uint8_t *stA = smem + (size_t)buf * STAGE_BYTES;
        uint8_t *stB = stA + A_BYTES;
        const int k0 = kbeg + ch * KC;
        // A: 128 rows x 4 groups of 8 K values = 512 units, two per thread
#pragma unroll 1
        for (int p = 0; p < 2; p++) {
            const int u = tid + 256 * p;
            int r, kg;
            if (A.trans == NT) {
                r = u & 127;
                kg = u >> 7;
            } else {
                kg = u & 3;
                r = u >> 2;
            }
            const int emax = s_rexp[r];
            uint32_t fl[8][NS];
#pragma unroll
            for (int j = 0; j < 8; j++) oz::digit_floats(oz::fixed56(opa(A, M, row0 + r, k0 + kg * 8 + j, kend), emax), fl[j]);
            store_unit(stA, A_SLICE, r, kg, fl);
        }
        // B: 64 columns x 4 groups = 256 units, one per thread
        {
            int c, kg;
            if (B.trans == NT) {
                kg = tid & 3;
                c = tid >> 2;
            } else {
                c = tid & 63;
                kg = tid >> 6;
            }
            const int emax = s_cexp[c];
            uint32_t fl[8][NS];
#pragma unroll
            for (int j = 0; j < 8; j++) oz::digit_floats(oz::fixed56(opb(B, N, k0 + kg * 8 + j, col0 + c, kend), emax), fl[j]);
            store_unit(stB, B_SLICE, c, kg, fl);
        }
        tc::fence_proxy_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (tid == 0) {
            const uint32_t sa = sbase + buf * STAGE_BYTES, sb = sa + A_BYTES;
            const bool window_start = (ch % FLUSH) == 0;
#pragma unroll
            for (int ks = 0; ks < KC / 16; ks++) {
                const uint32_t koff = ks * 2 * LBO;
#pragma unroll
                for (int s = 0; s < NS; s++) {
                    const int ntot = 64 * (NS - s);
                    const uint64_t ad = tc::desc_nosw(sa + s * A_SLICE + koff, LBO, SBO);
                    const uint32_t acc = (window_start && ks == 0 && s == 0) ? 0u : 1u;
                    const int n1 = ntot < 256 ? ntot : 256;
                    tc::mma_bf16(tbase + 64 * s, ad, tc::desc_nosw(sb + koff, LBO, SBO), tc::idesc_bf16_f32(128, n1), acc);
                    if (ntot > 256)
                        tc::mma_bf16(tbase + 64 * s + 256, ad, tc::desc_nosw(sb + 32 * SBO + koff, LBO, SBO),
                                     tc::idesc_bf16_f32(128, ntot - 256), acc);
                }
            }
            tc::mma_commit(&mbar[buf]);
        }
        pend |= 1u << buf;
        if (((ch + 1) % FLUSH) == 0 || ch == nch - 1) {
            // this stage's commit also covers every earlier MMA (in-order issue)
            if (!tc::mbar_wait(&mbar[buf], (phase_bits >> buf) & 1u)) {
                if (tid == 0) atomicOr(status, ST_WAIT_TIMEOUT);
                s_abort = 1;
            }
            phase_bits ^= 1u << buf;
            pend &= ~(1u << buf);
            tc::fence_after_sync();
            if (!s_abort) {
#pragma unroll
                for (int d = 0; d < NS; d++) {
                    uint32_t v[32];
                    tc::tmem_ld32(tbase + ((uint32_t)(32 * q) << 16) + (uint32_t)(64 * d + 32 * h), v);
                    tc::tmem_ld_wait();
#pragma unroll
                    for (int j = 0; j < 32; j++) {
                        const long long iv = (long long)oz::acc_int(v[j]);
                        if (d <= 3)
                            acc_hi[j] += iv << (7 * (3 - d));
                        else
                            acc_lo[j] += iv << (7 * (7 - d));
                    }
                }
            }
            tc::fence_before_sync();
            __syncthreads();
        }
    }
    // ---- epilogue: TMEM lane 32q + lane = output row, columns 32h + j
    if (!s_abort) {
        const int r = 32 * q + lane, gr = row0 + r;
        const int er = s_rexp[r];
        if (gr < M) {
#pragma unroll
            for (int j = 0; j < 32; j++) {
                const int c = 32 * h + j, gc = col0 + c;
                if (gc >= N) continue;
                const int ec = s_cexp[c];
                double v;
                if (er == 0x7FF || ec == 0x7FF)
                    v = __longlong_as_double(0x7FF8000000000000ll);
                else
                    v = (er && ec) ? oz::assemble(acc_hi[j], acc_lo[j], (er - 1022) + (ec - 1022) - 63) : 0.0;
                if (part)
                    part[(size_t)blockIdx.z * M * N + (size_t)gr + (size_t)gc * M] = v;
                else
                    epi_store(v, gr, gc, C, ldc, e);
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, 512);
}

}  // namespace ozg

static inline int cdiv(long long a, long long b) { return (int)((a + b - 1) / b); }

int ozgemm_splits(int M, int N, int K, long long part_len)
{
    if (M <= 0 || N <= 0 || K <= 256) return 1;
    const long long tiles = (long long)cdiv(M, ozg::BM) * cdiv(N, ozg::BN);
    const int sms = sm_count();
    if (tiles >= sms) return 1;
    int s = cdiv(K, 256);
    const int want = cdiv(sms, tiles);
    if (s > want) s = want;
    const long long fit = part_len / ((long long)M * N);
    if (s > fit) s = (int)fit;
    return s < 2 ? 1 : s;
}

void ozgemm(int M, int N, int K, Operand A, Operand B, double *C, int ldc, const GemmEpi &e, double *part,
            long long part_len, const char *tag)
{
    if (M <= 0 || N <= 0) return;
    cudaStream_t st = stream();
    int splits = part ? ozgemm_splits(M, N, K, part_len) : 1;
    int kchunk = K > 0 ? K : 1;
    if (splits > 1) {
        kchunk = cdiv(cdiv(K, splits), ozg::KC) * ozg::KC;
        splits = cdiv(K, kchunk);
    }
    double *p = splits > 1 ? part : nullptr;
    cudaFuncSetAttribute(ozg::k_ozgemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ozg::SMEM);
    dim3 grid(cdiv(M, ozg::BM), cdiv(N, ozg::BN), splits);
    trace_begin();
    ozg::k_ozgemm<<<grid, 256, ozg::SMEM, st>>>(M, N, K, kchunk, A, B, C, ldc, e, p, status_ptr());
    note_launch(tag);
    if (splits > 1) splitk_reduce(M, N, splits, part, C, ldc, e);
}

}  // namespace lg
