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
// 512 threads (16 warps) per CTA: one A unit (8 K values of one row) and half
// a B unit per thread and stage; TMEM lane 32 (warp % 4) + lane and output
// columns 16 (warp / 4) + [0, 16) per thread.
constexpr int OZT = 512;
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

// Digits of 4 consecutive K values (half hf of a unit) -> 8-byte stores.
__device__ __forceinline__ void store_half(uint8_t *base, uint32_t slice_bytes, int idx, int kg, int hf,
                                           const uint32_t (&w01)[NS], const uint32_t (&w23)[NS])
{
#pragma unroll
    for (int s = 0; s < NS; s++)
        *(uint2 *)(base + s * slice_bytes + (idx >> 3) * SBO + kg * LBO + (idx & 7) * 16 + hf * 8) =
            make_uint2(w01[s], w23[s]);
}

// Digit words of 4 FP64 values (bit patterns) scaled by the group exponent.
__device__ __forceinline__ void digits4(const unsigned long long *v, int emax, uint32_t (&w01)[NS],
                                        uint32_t (&w23)[NS])
{
    oz::digit_pair(oz::fixed56(v[0], emax), oz::fixed56(v[1], emax), w01);
    oz::digit_pair(oz::fixed56(v[2], emax), oz::fixed56(v[3], emax), w23);
}

// The epilogue's FP64 decisions, taken once per tile: the FP64 pipe is
// narrow, so per-output FP64 compares and products are avoided.
struct EpiMode {
    int amode;     // 1: alpha = 1, 2: alpha = -1 (a sign flip), 0: general
    bool use_beta;
};
__device__ __forceinline__ EpiMode epi_mode(const GemmEpi &e)
{
    EpiMode m;
    m.amode = e.alpha == 1.0 ? 1 : (e.alpha == -1.0 ? 2 : 0);
    m.use_beta = e.beta != 0.0;
    return m;
}

// FP64 operations the compiler may not speculate: as volatile asm they run
// only on the branch that needs them (an if-converted epilogue would issue
// them for every output on the narrow FP64 pipe).
__device__ __forceinline__ double dmul_nospec(double a, double b)
{
    double r;
    asm volatile("mul.rn.f64 %0, %1, %2;" : "=d"(r) : "d"(a), "d"(b));
    return r;
}
__device__ __forceinline__ double dadd_nospec(double a, double b)
{
    double r;
    asm volatile("add.rn.f64 %0, %1, %2;" : "=d"(r) : "d"(a), "d"(b));
    return r;
}
__device__ __forceinline__ double dfma_nospec(double a, double b, double c)
{
    double r;
    asm volatile("fma.rn.f64 %0, %1, %2, %3;" : "=d"(r) : "d"(a), "d"(b), "d"(c));
    return r;
}

__device__ __forceinline__ void epi_store(double v, int r, int c, double *C, int ldc, const GemmEpi &e,
                                          const EpiMode &md)
{
    if (e.upper_only && r > c) return;
    double out;
    if (md.amode == 1)
        out = v;
    else if (md.amode == 2)
        out = __longlong_as_double(__double_as_longlong(v) ^ (long long)0x8000000000000000ull);
    else
        out = dmul_nospec(e.alpha, v);
    if (e.add_diag && r == c) out = dadd_nospec(out, 1.0);
    const size_t off = (size_t)r + (size_t)c * (size_t)ldc;
    if (md.use_beta && r >= e.zero_rows) out = dfma_nospec(e.beta, C[off], out);
    C[off] = out;
}

// Adds the 8 digit orders of this thread's 16 TMEM columns (lane quarter q,
// column group h) into the int64 accumulators: orders 0-3 into hi, 4-7 into
// lo, four orders combined per value (combine4).  Four 8-column loads are in
// flight per wait.
__device__ __forceinline__ void flush_acc(uint32_t tbase, int q, int h, long long (&acc_hi)[16],
                                          long long (&acc_lo)[16])
{
#pragma unroll
    for (int hc = 0; hc < 2; hc++)
#pragma unroll
        for (int g4 = 0; g4 < 2; g4++) {
            uint32_t v[4][8];
#pragma unroll
            for (int e = 0; e < 4; e++)
                tc::tmem_ld8(tbase + ((uint32_t)(32 * q) << 16) + (uint32_t)(64 * (4 * g4 + e) + 16 * h + 8 * hc), v[e]);
            tc::tmem_ld_wait();
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const long long x = oz::combine4(v[0][j], v[1][j], v[2][j], v[3][j]);
                if (g4 == 0)
                    acc_hi[8 * hc + j] += x;
                else
                    acc_lo[8 * hc + j] += x;
            }
        }
}

// Per-CTA state of the tile loop: TMEM, the stage mbarriers and their phase
// bookkeeping carry over from one tile to the next in the persistent kernel.
struct TileCtx {
    uint8_t *smem;
    uint64_t *empty_b, *full_b, *tfree;
    int *s_rexp, *s_cexp;
    volatile int *s_abort;
    uint32_t tbase, sbase;
    int g;            // stages run by this CTA so far (buffer g & 1, mbarrier parity (g >> 1) & 1)
    int w;            // flush windows completed so far (tfree parity)
    int last_commit;  // global stage index of the issuer's last commit (-1: none)
};

__device__ __forceinline__ void ctx_open(TileCtx &x, uint8_t *smem, uint64_t *bars, uint32_t *tmem_base_s,
                                         int *s_rexp, int *s_cexp, int *s_abort)
{
    const int tid = threadIdx.x, warp = tid >> 5;
    // bars: empty[NSTAGE], full[NSTAGE], tfree
    if (tid == 0) {
        for (int b = 0; b < NSTAGE; b++) {
            tc::mbar_init(&bars[b], 1);
            tc::mbar_init(&bars[NSTAGE + b], OZT / 32);
        }
        tc::mbar_init(&bars[2 * NSTAGE], OZT / 32);
        tc::fence_mbar_init();
        *s_abort = 0;
    }
    if (warp == 0) {
        tc::tmem_alloc(tmem_base_s, 512);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    x.smem = smem;
    x.empty_b = bars;
    x.full_b = bars + NSTAGE;
    x.tfree = bars + 2 * NSTAGE;
    x.s_rexp = s_rexp;
    x.s_cexp = s_cexp;
    x.s_abort = s_abort;
    x.tbase = *tmem_base_s;
    x.sbase = tc::smem_u32(smem);
    x.g = 0;
    x.w = 0;
    x.last_commit = -1;
}

__device__ __forceinline__ void ctx_close(TileCtx &x)
{
    // normally every commit has been waited on by the flushes; after an
    // abort wait (bounded) for the issuer's last MMAs before freeing TMEM
    if (x.last_commit >= 0) tc::mbar_wait(&x.empty_b[x.last_commit & 1], (x.last_commit >> 1) & 1);
    tc::fence_before_sync();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) tc::tmem_dealloc(x.tbase, 512);
}

// One 128 x 64 output tile at (row0, col0) over K range [kbeg, kend); with
// `part` set the FP64 partial product goes there (ld M) instead of C.
// Returns false after a bounded wait gave up (the CTA must stop).
__device__ __forceinline__ bool tile(TileCtx &x, int M, int N, int row0, int col0, int kbeg, int kend,
                                     const Operand &A, const Operand &B, double *C, int ldc, const GemmEpi &e,
                                     double *part, int *status, const int *rexp = nullptr,
                                     const int *cexp = nullptr)
{
    uint8_t *smem = x.smem;
    int *s_rexp = x.s_rexp, *s_cexp = x.s_cexp;
    volatile int *s_abort = x.s_abort;
    const uint32_t tbase = x.tbase, sbase = x.sbase;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // an upper triangular op(B) has no entries below row col0 + BN - 1
    if (B.mask == M_UPPER || B.mask == M_UNIT_UPPER) {
        if (B.trans == NT) kend = min(kend, col0 + BN);
    }
    // ---- per-thread state of the stage loop
    const int q = warp & 3, h = warp >> 2;
    long long acc_hi[16], acc_lo[16];
#pragma unroll
    for (int j = 0; j < 16; j++) {
        acc_hi[j] = 0;
        acc_lo[j] = 0;
    }
    const int nch = kend > kbeg ? (kend - kbeg + KC - 1) / KC : 0;
    // this thread's A unit (row ar, group ak) and B half unit (column bc,
    // group bk, half bh); the values of stage ch + 1 are loaded while stage
    // ch is split.  No block-wide barrier in the stage loop: the warps arrive
    // on full[b] when their part of a stage is written, lane 0 of the last
    // warp issues the MMAs once all have, its commit frees the buffer
    // (empty[b]); after a flush every warp arrives on tfree before the next
    // window's first MMA may overwrite the accumulators.
    int ar, ak, bc, bk;
    const int bh = tid & 1, bu = tid >> 1;
    if (A.trans == NT) {
        ar = tid & 127;
        ak = tid >> 7;
    } else {
        ak = tid & 3;
        ar = tid >> 2;
    }
    if (B.trans == NT) {
        bk = bu & 3;
        bc = bu >> 2;
    } else {
        bc = bu & 63;
        bk = bu >> 6;
    }
    unsigned long long ra[8], rb[4];
    auto load_stage = [&](int ch2) {
        const int k1 = kbeg + ch2 * KC;
        const bool live = ch2 < nch;
#pragma unroll
        for (int j = 0; j < 8; j++) ra[j] = live ? opa(A, M, row0 + ar, k1 + ak * 8 + j, kend) : 0ull;
#pragma unroll
        for (int j = 0; j < 4; j++) rb[j] = live ? opb(B, N, k1 + bk * 8 + 4 * bh + j, col0 + bc, kend) : 0ull;
    };
    // the first stage's operands and the precomputed scales are loaded before
    // the barrier, so their latency overlaps the wait for the previous tile
    load_stage(0);
    const int my_rexp = (tid < BM && rexp && row0 + tid < M) ? rexp[row0 + tid] : 0;
    const int my_cexp = (tid < BN && cexp && col0 + tid < N) ? cexp[col0 + tid] : 0;
    __syncthreads();  // the previous tile's epilogue has read the exponents
    if (tid < BM) s_rexp[tid] = my_rexp;
    if (tid < BN) s_cexp[tid] = my_cexp;
    __syncthreads();

    // ---- scaling groups over [kbeg, kend): the largest biased exponent of
    // every row of op(A) and every column of op(B); lanes run along the
    // stored contiguous dimension
    if (rexp) {
        // precomputed
    } else if (A.trans == NT) {
        const int r = tid & 127;
        int mx = 0;
#pragma unroll 8
        for (int k = kbeg + (tid >> 7); k < kend; k += 4) mx = max(mx, oz::bexp(opa(A, M, row0 + r, k, kend)));
        atomicMax(&s_rexp[r], mx);
    } else {
        for (int r = warp; r < BM; r += OZT / 32) {
            int mx = 0;
#pragma unroll 4
            for (int k = kbeg + lane; k < kend; k += 32) mx = max(mx, oz::bexp(opa(A, M, row0 + r, k, kend)));
            for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            if (lane == 0) s_rexp[r] = mx;
        }
    }
    if (cexp) {
        // precomputed
    } else if (B.trans == NT) {
        for (int c = warp; c < BN; c += OZT / 32) {
            int mx = 0;
#pragma unroll 4
            for (int k = kbeg + lane; k < kend; k += 32) mx = max(mx, oz::bexp(opb(B, N, k, col0 + c, kend)));
            for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            if (lane == 0) s_cexp[c] = mx;
        }
    } else {
        const int c = tid & 63;
        int mx = 0;
#pragma unroll 8
        for (int k = kbeg + (tid >> 6); k < kend; k += 8) mx = max(mx, oz::bexp(opb(B, N, k, col0 + c, kend)));
        atomicMax(&s_cexp[c], mx);
    }
    __syncthreads();
    if (tid < BM && s_rexp[tid] == 0x7FF) atomicOr(status, ST_NONFINITE);
    if (tid < BN && s_cexp[tid] == 0x7FF) atomicOr(status, ST_NONFINITE);

    // ---- main loop
    const bool issuer = warp == OZT / 32 - 1 && lane == 0;
    for (int ch = 0; ch < nch; ch++) {
        const int G = x.g + ch, buf = G & 1;
        if (G >= NSTAGE && !tc::wait_abort_warp(&x.empty_b[buf], ((G - NSTAGE) >> 1) & 1, s_abort, status, ST_WAIT_TIMEOUT)) break;
        uint8_t *stA = smem + (size_t)buf * STAGE_BYTES;
        uint8_t *stB = stA + A_BYTES;
        // A: 128 rows x 4 groups of 8 K values = 512 units, one per thread
        {
            const int emax = s_rexp[ar];
#pragma unroll
            for (int hf = 0; hf < 2; hf++) {
                uint32_t w01[NS], w23[NS];
                digits4(ra + 4 * hf, emax, w01, w23);
                store_half(stA, A_SLICE, ar, ak, hf, w01, w23);
            }
        }
        // B: 64 columns x 4 groups x 2 halves = 512 half units, one per thread
        {
            uint32_t w01[NS], w23[NS];
            digits4(rb, s_cexp[bc], w01, w23);
            store_half(stB, B_SLICE, bc, bk, bh, w01, w23);
        }
        load_stage(ch + 1);  // in flight during the MMA issue and the next wait
        tc::fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&x.full_b[buf]);
        const bool window_start = (ch % FLUSH) == 0;
        if (issuer) {
            bool ok = tc::wait_abort(&x.full_b[buf], (G >> 1) & 1, s_abort, status, ST_WAIT_TIMEOUT);
            if (ok && window_start && x.w > 0) ok = tc::wait_abort(x.tfree, (x.w - 1) & 1, s_abort, status, ST_WAIT_TIMEOUT);
            if (ok) {
                tc::fence_after_sync();
                const uint64_t da = tc::desc_nosw(sbase + buf * STAGE_BYTES, LBO, SBO);
                const uint64_t db = tc::desc_nosw(sbase + buf * STAGE_BYTES + A_BYTES, LBO, SBO);
#pragma unroll
                for (int ks = 0; ks < KC / 16; ks++) {
                    const uint64_t koff = (uint64_t)(ks * 2 * LBO) >> 4;
#pragma unroll
                    for (int sl = 0; sl < NS; sl++) {
                        const int ntot = 64 * (NS - sl);
                        const uint64_t ad = da + koff + ((uint64_t)(sl * A_SLICE) >> 4);
                        const uint32_t acc = (window_start && ks == 0 && sl == 0) ? 0u : 1u;
                        const int n1 = ntot < 256 ? ntot : 256;
                        tc::mma_bf16(tbase + 64 * sl, ad, db + koff, tc::idesc_bf16_f32(128, n1), acc);
                        if (ntot > 256)
                            tc::mma_bf16(tbase + 64 * sl + 256, ad, db + koff + ((uint64_t)(32 * SBO) >> 4),
                                         tc::idesc_bf16_f32(128, ntot - 256), acc);
                    }
                }
                tc::mma_commit(&x.empty_b[buf]);
                x.last_commit = G;
            }
        }
        if (__any_sync(0xffffffffu, *s_abort)) break;
        if (((ch + 1) % FLUSH) == 0 || ch == nch - 1) {
            // this stage's commit also covers every earlier MMA (in-order issue)
            if (!tc::wait_abort_warp(&x.empty_b[buf], (G >> 1) & 1, s_abort, status, ST_WAIT_TIMEOUT)) break;
            tc::fence_after_sync();
            flush_acc(tbase, q, h, acc_hi, acc_lo);
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(x.tfree);
            x.w++;
        }
    }
    x.g += nch;
    __syncthreads();
    // ---- epilogue: TMEM lane 32q + lane = output row, columns 16h + j.
    // Up to 256 K values (two flush windows) |hi| stays below 2^43, where the
    // integer-only assembly keeps every bit down to 2^-54 of the group scale.
    if (!*s_abort) {
        const bool fast = kend - kbeg <= 256;
        const EpiMode md = epi_mode(e);
        const int r = 32 * q + lane, gr = row0 + r;
        const int er = s_rexp[r];
        if (gr < M) {
#pragma unroll
            for (int j = 0; j < 16; j++) {
                const int c = 16 * h + j, gc = col0 + c;
                if (gc >= N) continue;
                const int ec = s_cexp[c];
                double v;
                if (er == 0x7FF || ec == 0x7FF)
                    v = __longlong_as_double(0x7FF8000000000000ll);
                else if (!(er && ec))
                    v = 0.0;
                else if (fast)
                    v = oz::assemble_fast(acc_hi[j], acc_lo[j], (er - 1022) + (ec - 1022) - 63);
                else
                    v = oz::assemble(acc_hi[j], acc_lo[j], (er - 1022) + (ec - 1022) - 63);
                if (part)
                    part[(size_t)gr + (size_t)gc * M] = v;
                else
                    epi_store(v, gr, gc, C, ldc, e, md);
            }
        }
    }
    // the next tile's first MMA waits on tfree, so TMEM needs no barrier
    // here; the next tile's first barrier orders the exponent reads above
    return !*s_abort;
}

#define OZG_SHARED                                          \
    extern __shared__ __align__(1024) uint8_t smem[];      \
    __shared__ __align__(8) uint64_t bars[2 * NSTAGE + 1]; \
    __shared__ uint32_t tmem_base_s;                       \
    __shared__ int s_rexp[BM], s_cexp[BN];                 \
    __shared__ int s_abort;                                \
    TileCtx x;                                             \
    ctx_open(x, smem, bars, &tmem_base_s, s_rexp, s_cexp, &s_abort)

__global__ void __launch_bounds__(OZT, 1)
    k_ozgemm(int M, int N, int K, int kchunk, Operand A, Operand B, double *C, int ldc, GemmEpi e, double *part,
             int *status)
{
    OZG_SHARED;
    const int kbeg = blockIdx.z * kchunk;
    tile(x, M, N, blockIdx.x * BM, blockIdx.y * BN, kbeg, min(K, kbeg + kchunk), A, B, C, ldc, e,
         part ? part + (size_t)blockIdx.z * M * N : nullptr, status);
    ctx_close(x);
}

// Grouped form: CTA b runs tile b - prefix[g] of group g, prefix[g] <= b <
// prefix[g + 1]; a group's tiles are numbered column-major over its 128 x 64
// tile grid.  No split-K.
// tilemap[b] = {group, tile within the group} for every tile b < prefix[ngroups].
__global__ void k_tile_map(const int *prefix, int ngroups, int2 *tilemap)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ngroups) return;
    const int b0 = prefix[g], b1 = prefix[g + 1];
    for (int b = b0; b < b1; b++) tilemap[b] = make_int2(g, b - b0);
}

// Persistent: CTA i takes tiles i, i + grid, ...; the next tile's map entry
// is loaded while the current tile runs.
__global__ void __launch_bounds__(OZT, 1) k_ozgemm_groups(const OzGroup *groups, const int2 *tilemap, int total,
                                                          int *status)
{
    OZG_SHARED;
    int2 cur = blockIdx.x < total ? tilemap[blockIdx.x] : make_int2(0, 0);
    for (int b = blockIdx.x; b < total; b += gridDim.x) {
        const int bn = b + gridDim.x;
        const int2 nxt = bn < total ? tilemap[bn] : make_int2(0, 0);
        const OzGroup g = groups[cur.x];
        const int t = cur.y;
        const int tiles_m = (g.M + BM - 1) / BM;
        if (!tile(x, g.M, g.N, (t % tiles_m) * BM, (t / tiles_m) * BN, 0, g.K, g.A, g.B, g.C, g.ldc, g.e, nullptr,
                  status, g.rexp, g.cexp))
            break;
        cur = nxt;
    }
    ctx_close(x);
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
    ozg::k_ozgemm<<<grid, ozg::OZT, ozg::SMEM, st>>>(M, N, K, kchunk, A, B, C, ldc, e, p, status_ptr());
    note_launch(tag);
    if (splits > 1) splitk_reduce(M, N, splits, part, C, ldc, e);
}

int ozgemm_group_tiles(int M, int N) { return M > 0 && N > 0 ? cdiv(M, ozg::BM) * cdiv(N, ozg::BN) : 0; }

namespace ozg {
// Job j's row scales; threads run along the rows (coalesced column reads).
__global__ void k_row_exponents(const RowExpJob *jobs, int njobs)
{
    const int j = blockIdx.y;
    if (j >= njobs) return;
    const RowExpJob J = jobs[j];
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < J.m; r += gridDim.x * blockDim.x) {
        int mx = 0;
#pragma unroll 8
        for (int c = 0; c < J.n; c++)
            mx = max(mx, oz::bexp(((const unsigned long long *)J.A)[(size_t)r + (size_t)c * J.lda]));
        J.rexp[r] = mx;
    }
}
}  // namespace ozg

void row_exponents(const RowExpJob *d_jobs, int njobs)
{
    if (njobs <= 0) return;
    trace_begin();
    ozg::k_row_exponents<<<dim3(8, njobs), 256, 0, stream()>>>(d_jobs, njobs);
    note_launch("row_exponents");
}

void ozgemm_groups(const OzGroup *d_groups, const int *d_prefix, int ngroups, int total_tiles, int2 *d_tilemap)
{
    if (ngroups <= 0 || total_tiles <= 0) return;
    cudaStream_t st = stream();
    trace_begin();
    ozg::k_tile_map<<<(ngroups + 255) / 256, 256, 0, st>>>(d_prefix, ngroups, d_tilemap);
    note_launch("tile_map");
    cudaFuncSetAttribute(ozg::k_ozgemm_groups, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ozg::SMEM);
    const int grid = total_tiles < sm_count() ? total_tiles : sm_count();
    trace_begin();
    ozg::k_ozgemm_groups<<<grid, ozg::OZT, ozg::SMEM, st>>>(d_groups, d_tilemap, total_tiles, status_ptr());
    note_launch("ozgemm_groups");
}

}  // namespace lg

// ---------------------------------------------------------------------------
// Grouped FP64-grade Grams G = A^T A of many instances (n <= 128): job j is
// instance j's column half h (G columns [64h, 64h + 64)), all rows of A in
// one CTA.  The column scales come from a prepass (k_gram_colexp), so A is
// read once per job; every 32-row stage is split once into the digits of all
// 128 columns (the M side) and those of the job's 64 columns are copied to
// the N side, so the MMA issue is the GEMM's.
// ---------------------------------------------------------------------------
namespace lg {
namespace ozg {

__global__ void k_gram_colexp(const GramW *jobs, int njobs)
{
    const int j = blockIdx.x;
    if (j >= njobs) return;
    const GramW J = jobs[j];
    if (J.half) return;  // one job per instance computes the scales
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int c = warp; c < J.n; c += blockDim.x >> 5) {
        const unsigned long long *col = (const unsigned long long *)(J.A + (size_t)c * J.lda);
        int mx = 0;
        for (int r = lane; r < J.m; r += 32) mx = max(mx, oz::bexp(col[r]));
        for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (lane == 0) J.colexp[c] = mx;
    }
}

// The 16 warps split the FP64 values into digit slices; lane 0 of the last
// warp also issues the MMAs, so no block-wide barrier sits in the stage loop.
// Per shared-memory buffer the warps arrive on full[b] (16 arrivals) once
// their part of a stage is written; the issuer waits for it, issues, and its
// commit arrives on empty[b] when the tensor core has read the buffer.  After
// reading a flush window's accumulators every warp arrives on tfree (16
// arrivals), which the issuer waits for before the next window's first MMA
// overwrites them.  Every wait is bounded; a wait that gives up sets the
// status and the CTA's abort flag, and every party leaves its loop.
constexpr int GW_NT = OZT;
constexpr int GW_ISSUER = OZT / 32 - 1;

__global__ void __launch_bounds__(GW_NT, 1) k_gram_w(const GramW *jobs, int njobs, int *status)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t empty_b[NSTAGE], full_b[NSTAGE], tfree;
    __shared__ uint32_t tmem_base_s;
    __shared__ int s_exp[BM];
    __shared__ int s_bexp[BN];
    __shared__ int s_abort_v;
    volatile int *s_abort = &s_abort_v;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const GramW J = jobs[blockIdx.x];
    const int n = J.n, nm = min(n, BM), m = J.m, c0 = 64 * J.half;
    const bool bsep = c0 + BN > BM;  // the N-side columns are not among the M-side ones
    if (tid == 0) {
        for (int b = 0; b < NSTAGE; b++) {
            tc::mbar_init(&empty_b[b], 1);
            tc::mbar_init(&full_b[b], OZT / 32);
        }
        tc::mbar_init(&tfree, OZT / 32);
        tc::fence_mbar_init();
        s_abort_v = 0;
    }
    if (tid < BM) s_exp[tid] = tid < nm ? J.colexp[tid] : 0;
    if (tid < BN) s_bexp[tid] = c0 + tid < n ? J.colexp[c0 + tid] : 0;
    if (warp == 0) {
        tc::tmem_alloc(&tmem_base_s, 512);
        tc::tmem_relinquish();
    }
    if (nm < BM) {
        // columns nm..127 of the M side stay zero: clear them once, skip them below
        for (int i = tid; i < (int)(NSTAGE * STAGE_BYTES / 16); i += GW_NT) ((uint4 *)smem)[i] = make_uint4(0, 0, 0, 0);
        tc::fence_proxy_async_smem();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = tmem_base_s;
    const uint32_t sbase = tc::smem_u32(smem);
    const int nch = (m + KC - 1) / KC;
    const int q = warp & 3, h = (warp >> 2) & 3;
    long long acc_hi[16], acc_lo[16];
#pragma unroll
    for (int j = 0; j < 16; j++) {
        acc_hi[j] = 0;
        acc_lo[j] = 0;
    }
    {
        // This thread's unit: column tid / 4, rows 8 (tid % 4) .. + 8 of a
        // stage; stage ch + 1 is loaded while stage ch is split.
        const uint64_t dA0 = tc::desc_nosw(sbase, LBO, SBO), dB0 = tc::desc_nosw(sbase + A_BYTES, LBO, SBO);
        const int ukg = tid & 3, ucol = tid >> 2;
        const unsigned long long *ucp = (const unsigned long long *)(J.A + (size_t)ucol * J.lda);
        unsigned long long rv[8];
        auto load_stage = [&](int ch2) {
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const int r = ch2 * KC + ukg * 8 + j;
                rv[j] = (ch2 < nch && ucol < nm && r < m) ? ucp[r] : 0ull;
            }
        };
        int last_commit = -1;
        load_stage(0);
        for (int ch = 0; ch < nch; ch++) {
            const int buf = ch & 1;
            // the buffer's previous stage (ch - 2) has been read by the tensor core
            if (ch >= NSTAGE && !tc::wait_abort_warp(&empty_b[buf], ((ch - NSTAGE) >> 1) & 1, s_abort, status, ST_WAIT_TIMEOUT)) break;
            uint8_t *stA = smem + (size_t)buf * STAGE_BYTES;
            uint8_t *stB = stA + A_BYTES;
            const int k0 = ch * KC;
            if (ucol < nm) {
                const int c = ucol, kg = ukg;
                const int emax = s_exp[c];
#pragma unroll
                for (int hf = 0; hf < 2; hf++) {
                    uint32_t w01[NS], w23[NS];
                    digits4(rv + 4 * hf, emax, w01, w23);
                    store_half(stA, A_SLICE, c, kg, hf, w01, w23);
                    if (!bsep && c >= c0 && c < c0 + BN) store_half(stB, B_SLICE, c - c0, kg, hf, w01, w23);
                }
            }
            load_stage(ch + 1);
            if (bsep) {
                // 64 columns x 4 groups x 2 halves = 512 half units of the N side
                const int hb = tid & 1, kg = (tid >> 1) & 3, c = tid >> 3;
                const int emax = s_bexp[c];
                const unsigned long long *col = (const unsigned long long *)(J.A + (size_t)(c0 + c) * J.lda);
                unsigned long long bv[4];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int r = k0 + kg * 8 + 4 * hb + j;
                    bv[j] = (c0 + c < n && r < m) ? col[r] : 0ull;
                }
                uint32_t w01[NS], w23[NS];
                digits4(bv, emax, w01, w23);
                store_half(stB, B_SLICE, c, kg, hb, w01, w23);
            }
            tc::fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&full_b[buf]);
            if (warp == GW_ISSUER && lane == 0) {
                bool ok = tc::wait_abort(&full_b[buf], (ch >> 1) & 1, s_abort, status, ST_WAIT_TIMEOUT);
                const bool window_start = (ch % FLUSH) == 0;
                if (ok && window_start && ch > 0) ok = tc::wait_abort(&tfree, ((ch / FLUSH) - 1) & 1, s_abort, status, ST_WAIT_TIMEOUT);
                if (ok) {
                    tc::fence_after_sync();
                    const uint64_t da = dA0 + ((uint64_t)(buf * STAGE_BYTES) >> 4);
                    const uint64_t db = dB0 + ((uint64_t)(buf * STAGE_BYTES) >> 4);
#pragma unroll
                    for (int ks = 0; ks < KC / 16; ks++) {
                        const uint64_t koff = (uint64_t)(ks * 2 * LBO) >> 4;
#pragma unroll
                        for (int sl = 0; sl < NS; sl++) {
                            const int ntot = 64 * (NS - sl);
                            const uint64_t ad = da + koff + ((uint64_t)(sl * A_SLICE) >> 4);
                            const uint32_t acc = (window_start && ks == 0 && sl == 0) ? 0u : 1u;
                            const int n1 = ntot < 256 ? ntot : 256;
                            tc::mma_bf16(tbase + 64 * sl, ad, db + koff, tc::idesc_bf16_f32(128, n1), acc);
                            if (ntot > 256)
                                tc::mma_bf16(tbase + 64 * sl + 256, ad, db + koff + ((uint64_t)(32 * SBO) >> 4),
                                             tc::idesc_bf16_f32(128, ntot - 256), acc);
                        }
                    }
                    tc::mma_commit(&empty_b[buf]);
                    last_commit = ch;
                }
            }
            if (__any_sync(0xffffffffu, *s_abort)) break;
            if (((ch + 1) % FLUSH) == 0 || ch == nch - 1) {
                // every MMA of the window is complete once this stage's commit is
                if (!tc::wait_abort_warp(&empty_b[buf], (ch >> 1) & 1, s_abort, status, ST_WAIT_TIMEOUT)) break;
                tc::fence_after_sync();
                flush_acc(tbase, q, h, acc_hi, acc_lo);
                tc::fence_before_sync();
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(&tfree);
            }
        }
        // after an abort the issuer's last MMAs may still run: wait (bounded)
        // for its last commit before the accumulators are released
        if (last_commit >= 0) tc::mbar_wait(&empty_b[last_commit & 1], (last_commit >> 1) & 1);
    }
    __syncthreads();
    if (!*s_abort) {
        const int r = 32 * q + lane;
        const int er = s_exp[r];
        if (r < nm) {
#pragma unroll
            for (int j = 0; j < 16; j++) {
                const int c = c0 + 16 * h + j;
                if (c >= n) continue;
                const int ec = s_bexp[16 * h + j];
                double v;
                if (er == 0x7FF || ec == 0x7FF) {
                    v = __longlong_as_double(0x7FF8000000000000ll);
                    atomicOr(status, ST_NONFINITE);
                } else {
                    v = (er && ec) ? oz::assemble(acc_hi[j], acc_lo[j], (er - 1022) + (ec - 1022) - 63) : 0.0;
                }
                J.G[(size_t)r + (size_t)c * J.ldg] = v;
                // the first block of a wide Gram also fills G(0:64, 64:128) by
                // symmetry: the 64..127 block job computes only its own rows
                if (c0 == 0 && r >= 64) J.G[(size_t)c + (size_t)r * J.ldg] = v;
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, 512);
}

// Gram block G(c0 : c0 + 64, c0 : c0 + 64) of one job from its own 64
// columns only (c0 = 64 half; for n <= 64 the whole Gram, for the second
// block of a wider matrix its diagonal block).  The 8 digit slices of the
// 64 columns sit next to each other, so [slice s; slice s + 1] is a 128-row
// M operand: for s = 0, 2, 4, 6, D[64 s : 512) += [A_s; A_{s+1}] x
// [A_0 .. A_{7-s}], 12 MMAs per 32-row stage instead of 24.  TMEM lanes 0-63
// (column i, even slices) hold order d in block d, lanes 64-127 (column i,
// odd slices) order d + 1; the halves are added through shared memory at
// the end.  Same mbarrier protocol as k_gram_w, four stage buffers.
constexpr int GS_STAGES = 4;
constexpr uint32_t GS_STAGE_BYTES = NS * B_SLICE;  // 32 KB
constexpr size_t GS_SMEM = GS_STAGES * (size_t)GS_STAGE_BYTES;  // 128 KB

__global__ void __launch_bounds__(OZT, 1) k_gram_stacked(const GramW *jobs, int njobs, int *status)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t empty_b[GS_STAGES], full_b[GS_STAGES], tfree;
    __shared__ uint32_t tmem_base_s;
    __shared__ int s_bexp[BN];
    __shared__ int s_abort_v;
    volatile int *s_abort = &s_abort_v;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const GramW J = jobs[blockIdx.x];
    const int n = J.n, m = J.m, c0 = 64 * J.half;
    if (tid == 0) {
        for (int b = 0; b < GS_STAGES; b++) {
            tc::mbar_init(&empty_b[b], 1);
            tc::mbar_init(&full_b[b], OZT / 32);
        }
        tc::mbar_init(&tfree, OZT / 32);
        tc::fence_mbar_init();
        s_abort_v = 0;
    }
    if (tid < BN) s_bexp[tid] = c0 + tid < n ? J.colexp[c0 + tid] : 0;
    if (warp == 0) {
        tc::tmem_alloc(&tmem_base_s, 512);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = tmem_base_s;
    const uint32_t sbase = tc::smem_u32(smem);
    const int nch = (m + KC - 1) / KC;
    const int q = warp & 3, h = (warp >> 2) & 3;
    const bool top = q < 2;  // TMEM lanes 0-63
    long long acc_hi[16], acc_lo[16];
#pragma unroll
    for (int j = 0; j < 16; j++) {
        acc_hi[j] = 0;
        acc_lo[j] = 0;
    }
    {
        // half unit: column uc of the block, rows 8 kg + 4 hb .. + 4 of a stage
        const int hb = tid & 1, kg = (tid >> 1) & 3, uc = tid >> 3;
        const unsigned long long *col = (const unsigned long long *)(J.A + (size_t)(c0 + uc) * J.lda);
        const bool live_c = c0 + uc < n;
        unsigned long long rv[4];
        auto load_stage = [&](int ch2) {
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int r = ch2 * KC + kg * 8 + 4 * hb + j;
                rv[j] = (ch2 < nch && live_c && r < m) ? col[r] : 0ull;
            }
        };
        const bool issuer = warp == OZT / 32 - 1 && lane == 0;
        int last_commit = -1;
        load_stage(0);
        for (int ch = 0; ch < nch; ch++) {
            const int buf = ch % GS_STAGES;
            if (ch >= GS_STAGES &&
                !tc::wait_abort_warp(&empty_b[buf], ((ch - GS_STAGES) / GS_STAGES) & 1, s_abort, status,
                                     ST_WAIT_TIMEOUT))
                break;
            uint8_t *stg = smem + (size_t)buf * GS_STAGE_BYTES;
            {
                uint32_t w01[NS], w23[NS];
                digits4(rv, s_bexp[uc], w01, w23);
                store_half(stg, B_SLICE, uc, kg, hb, w01, w23);
            }
            load_stage(ch + 1);
            tc::fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&full_b[buf]);
            const bool window_start = (ch % FLUSH) == 0;
            if (issuer) {
                bool ok = tc::wait_abort(&full_b[buf], (ch / GS_STAGES) & 1, s_abort, status, ST_WAIT_TIMEOUT);
                if (ok && window_start && ch > 0)
                    ok = tc::wait_abort(&tfree, ((ch / FLUSH) - 1) & 1, s_abort, status, ST_WAIT_TIMEOUT);
                if (ok) {
                    tc::fence_after_sync();
                    const uint64_t d0 = tc::desc_nosw(sbase + buf * GS_STAGE_BYTES, LBO, SBO);
#pragma unroll
                    for (int ks = 0; ks < KC / 16; ks++) {
                        const uint64_t koff = (uint64_t)(ks * 2 * LBO) >> 4;
#pragma unroll
                        for (int sl = 0; sl < NS; sl += 2) {
                            const int ntot = 64 * (NS - sl);
                            const uint64_t ad = d0 + koff + ((uint64_t)(sl * B_SLICE) >> 4);
                            const uint32_t acc = (window_start && ks == 0 && sl == 0) ? 0u : 1u;
                            const int n1 = ntot < 256 ? ntot : 256;
                            tc::mma_bf16(tbase + 64 * sl, ad, d0 + koff, tc::idesc_bf16_f32(128, n1), acc);
                            if (ntot > 256)
                                tc::mma_bf16(tbase + 64 * sl + 256, ad, d0 + koff + ((uint64_t)(32 * SBO) >> 4),
                                             tc::idesc_bf16_f32(128, ntot - 256), acc);
                        }
                    }
                    tc::mma_commit(&empty_b[buf]);
                    last_commit = ch;
                }
            }
            if (__any_sync(0xffffffffu, *s_abort)) break;
            if (((ch + 1) % FLUSH) == 0 || ch == nch - 1) {
                if (!tc::wait_abort_warp(&empty_b[buf], (ch / GS_STAGES) & 1, s_abort, status, ST_WAIT_TIMEOUT))
                    break;
                tc::fence_after_sync();
                // top lanes: order d in block d; bottom lanes: order d in
                // block d - 1 (their order 0 is absent: a zero word)
#pragma unroll
                for (int hc = 0; hc < 2; hc++)
#pragma unroll
                    for (int g4 = 0; g4 < 2; g4++) {
                        uint32_t v[4][8];
#pragma unroll
                        for (int e = 0; e < 4; e++) {
                            const int d = 4 * g4 + e;
                            const int blk = top ? d : d - 1;
                            if (blk >= 0)
                                tc::tmem_ld8(tbase + ((uint32_t)(32 * q) << 16) + (uint32_t)(64 * blk + 16 * h + 8 * hc),
                                             v[e]);
                            else
#pragma unroll
                                for (int j = 0; j < 8; j++) v[e][j] = 0u;
                        }
                        tc::tmem_ld_wait();
#pragma unroll
                        for (int j = 0; j < 8; j++) {
                            const long long x = oz::combine4(v[0][j], v[1][j], v[2][j], v[3][j]);
                            if (g4 == 0)
                                acc_hi[8 * hc + j] += x;
                            else
                                acc_lo[8 * hc + j] += x;
                        }
                    }
                tc::fence_before_sync();
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(&tfree);
            }
        }
        if (last_commit >= 0) tc::mbar_wait(&empty_b[last_commit % GS_STAGES], (last_commit / GS_STAGES) & 1);
    }
    __syncthreads();
    if (!*s_abort) {
        // bottom lanes hand their partial sums to the top lanes of the same column
        long long *xh = (long long *)smem;
        long long *xl = xh + 64 * 64;
        const int L = 32 * q + lane;
        if (!top) {
#pragma unroll
            for (int j = 0; j < 16; j++) {
                xh[(L - 64) * 64 + 16 * h + j] = acc_hi[j];
                xl[(L - 64) * 64 + 16 * h + j] = acc_lo[j];
            }
        }
        __syncthreads();
        if (top && c0 + L < n) {
            const int er = s_bexp[L];
#pragma unroll
            for (int j = 0; j < 16; j++) {
                const int cc = 16 * h + j, c = c0 + cc;
                if (c >= n) continue;
                const int ec = s_bexp[cc];
                double v;
                if (er == 0x7FF || ec == 0x7FF) {
                    v = __longlong_as_double(0x7FF8000000000000ll);
                    atomicOr(status, ST_NONFINITE);
                } else {
                    v = (er && ec) ? oz::assemble(acc_hi[j] + xh[L * 64 + cc], acc_lo[j] + xl[L * 64 + cc],
                                                  (er - 1022) + (ec - 1022) - 63)
                                   : 0.0;
                }
                J.G[(size_t)(c0 + L) + (size_t)c * J.ldg] = v;
            }
        }
    } else {
        __syncthreads();
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, 512);
}

}  // namespace ozg

void ozaki_grams(const GramW *d_jobs, int njobs, int nstacked)
{
    if (njobs <= 0) return;
    cudaStream_t st = stream();
    trace_begin();
    ozg::k_gram_colexp<<<njobs, 256, 0, st>>>(d_jobs, njobs);
    note_launch("gram_colexp");
    if (nstacked > 0) {
        cudaFuncSetAttribute(ozg::k_gram_stacked, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ozg::GS_SMEM);
        trace_begin();
        ozg::k_gram_stacked<<<nstacked, ozg::OZT, ozg::GS_SMEM, st>>>(d_jobs, nstacked, status_ptr());
        note_launch("ozaki_grams");
    }
    if (njobs > nstacked) {
        cudaFuncSetAttribute(ozg::k_gram_w, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ozg::SMEM);
        trace_begin();
        ozg::k_gram_w<<<njobs - nstacked, ozg::GW_NT, ozg::SMEM, st>>>(d_jobs + nstacked, njobs - nstacked,
                                                                       status_ptr());
        note_launch("ozaki_grams");
    }
}


// ---------------------------------------------------------------------------
// Batched row maps out(:, col0 : col0 + ncols) = A X(:, col0 : col0 + ncols)
// for many instances (A m x K, X upper triangular, K <= 128), FP64 grade.
// Persistent CTAs take work items (an instance's 64-column block) from a
// counter.  Per item the block of X is split once into digit chunks that
// stay in shared memory (4 chunks of 32 K, 128 KB); A is streamed through
// two 16-K stage buffers (32 KB each) with the mbarrier protocol of the
// split GEMM tile (full / empty per buffer, tfree per 128-row tile, lane 0
// of the last warp issuing), so each 128-row tile costs its A split, one
// TMEM fold and its epilogue.  The row and column scales are precomputed.
// ---------------------------------------------------------------------------
namespace ozg {

constexpr int MI_KC = 16;                                 // K per A stage
constexpr uint32_t MI_ASBO = (MI_KC / 8) * 128;           // 256
constexpr uint32_t MI_ASLICE = (BM / 8) * MI_ASBO;        // 4 KB per digit slice
constexpr uint32_t MI_ABYTES = NS * MI_ASLICE;            // 32 KB per stage
constexpr uint32_t MI_XCHUNK = NS * B_SLICE;              // 32 KB: 32 K of X, 8 slices
constexpr size_t MI_SMEM = 4 * (size_t)MI_XCHUNK + 2 * (size_t)MI_ABYTES;  // 192 KB

__global__ void __launch_bounds__(OZT, 1) k_map_items(const MapItem *items, int nitems, int *counter, int *status)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t empty_b[2], full_b[2], tfree;
    __shared__ uint32_t tmem_base_s;
    __shared__ int s_cexp[BN];
    __shared__ int s_item;
    __shared__ MapItem s_J;
    __shared__ int s_abort_v;
    volatile int *s_abort = &s_abort_v;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    uint8_t *XB = smem;
    uint8_t *AB = smem + 4 * MI_XCHUNK;
    if (tid == 0) {
        for (int b = 0; b < 2; b++) {
            tc::mbar_init(&empty_b[b], 1);
            tc::mbar_init(&full_b[b], OZT / 32);
        }
        tc::mbar_init(&tfree, OZT / 32);
        tc::fence_mbar_init();
        s_abort_v = 0;
    }
    if (warp == 0) {
        tc::tmem_alloc(&tmem_base_s, 512);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = tmem_base_s;
    const uint32_t xaddr = tc::smem_u32(XB), aaddr = tc::smem_u32(AB);
    const int q = warp & 3, h = warp >> 2;
    const bool issuer = warp == OZT / 32 - 1 && lane == 0;
    // A split unit: row ar, four K values 4 aq .. 4 aq + 3 of a 16-K stage
    const int ar = tid & 127, aq = tid >> 7;
    int G = 0, W = 0, last_commit = -1;
    for (;;) {
        // every warp arrives here after its tile loop (also when it left it
        // on an abort), so the abort flag read below is the same for all
        __syncthreads();  // the previous item's epilogue is done with s_cexp and s_J
        if (tid == 0) {
            const int it = atomicAdd(counter, 1);
            s_item = it;
            if (it < nitems) s_J = items[it];
        }
        __syncthreads();
        if (s_item >= nitems || *s_abort) break;
        const MapItem &J = s_J;
        if (tid < BN) s_cexp[tid] = tid < J.ncols ? J.cexp[J.col0 + tid] : 0;
        __syncthreads();
        // X digits once per item (zero outside the block's columns, below K
        // and below the diagonal); every MMA that read the previous item's
        // digits completed before its last fold
        const int kpad = (J.kend + MI_KC - 1) / MI_KC * MI_KC;
        for (int hu = tid; hu < BN * (kpad / 4); hu += OZT) {
            const int c = hu & (BN - 1), k0 = 4 * (hu >> 6);
            const int gc = J.col0 + c;
            unsigned long long v[4];
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int k = k0 + e;
                v[e] = (c < J.ncols && k < J.kend && k <= gc)
                           ? ((const unsigned long long *)J.X)[(size_t)k + (size_t)gc * J.ldx]
                           : 0ull;
            }
            uint32_t w01[NS], w23[NS];
            digits4(v, s_cexp[c], w01, w23);
            store_half(XB + (k0 >> 5) * MI_XCHUNK, B_SLICE, c, (k0 & 31) >> 3, (k0 & 7) >> 2, w01, w23);
        }
        tc::fence_proxy_async_smem();
        __syncthreads();
        const int ntiles = (J.m + BM - 1) / BM;
        const int nst = kpad / MI_KC;
        const unsigned long long *Ab = (const unsigned long long *)J.A;
        // the next stage's A values and row scale are loaded one stage ahead
        unsigned long long ra[4];
        int rx = 0;
        auto load = [&](int tile, int st) {
            const int grow = tile * BM + ar;
            const bool live = tile < ntiles && grow < J.m;
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int k = st * MI_KC + 4 * aq + e;
                ra[e] = (live && k < J.kend) ? Ab[(size_t)grow + (size_t)k * J.lda] : 0ull;
            }
            if (st == 0) rx = live ? J.rexp[grow] : 0;
        };
        load(0, 0);
        for (int tile = 0; tile < ntiles; tile++) {
            const int row0 = tile * BM;
            const int rr = 32 * q + lane, grow_e = row0 + rr;
            const int er = grow_e < J.m ? J.rexp[grow_e] : 0;  // in flight during the stages
            const int emax = rx;  // loaded with this tile's first stage
            long long acc_hi[16], acc_lo[16];
#pragma unroll
            for (int j = 0; j < 16; j++) {
                acc_hi[j] = 0;
                acc_lo[j] = 0;
            }
            for (int st = 0; st < nst; st++, G++) {
                const int buf = G & 1;
                if (G >= 2 &&
                    !tc::wait_abort_warp(&empty_b[buf], ((G - 2) >> 1) & 1, s_abort, status, ST_WAIT_TIMEOUT))
                    break;
                {
                    uint32_t w01[NS], w23[NS];
                    digits4(ra, emax, w01, w23);
                    uint8_t *dst = AB + (size_t)buf * MI_ABYTES + (ar >> 3) * MI_ASBO + (aq >> 1) * LBO + (ar & 7) * 16 +
                                   (aq & 1) * 8;
#pragma unroll
                    for (int sl = 0; sl < NS; sl++) *(uint2 *)(dst + sl * MI_ASLICE) = make_uint2(w01[sl], w23[sl]);
                }
                if (st + 1 < nst) {
                    load(tile, st + 1);
                } else {
                    load(tile + 1, 0);
                }
                tc::fence_proxy_async_smem();
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(&full_b[buf]);
                if (issuer) {
                    bool ok = tc::wait_abort(&full_b[buf], (G >> 1) & 1, s_abort, status, ST_WAIT_TIMEOUT);
                    if (ok && st == 0 && W > 0) ok = tc::wait_abort(&tfree, (W - 1) & 1, s_abort, status, ST_WAIT_TIMEOUT);
                    if (ok) {
                        tc::fence_after_sync();
                        const int k0 = st * MI_KC;
                        const uint64_t da = tc::desc_nosw(aaddr + buf * MI_ABYTES, LBO, MI_ASBO);
                        const uint64_t db =
                            tc::desc_nosw(xaddr + (k0 >> 5) * MI_XCHUNK + ((k0 & 31) >> 4) * 2 * LBO, LBO, SBO);
#pragma unroll
                        for (int sl = 0; sl < NS; sl++) {
                            const int ntot = 64 * (NS - sl);
                            const uint64_t ad = da + ((uint64_t)(sl * MI_ASLICE) >> 4);
                            const uint32_t acc = (st == 0 && sl == 0) ? 0u : 1u;
                            const int n1 = ntot < 256 ? ntot : 256;
                            tc::mma_bf16(tbase + 64 * sl, ad, db, tc::idesc_bf16_f32(128, n1), acc);
                            if (ntot > 256)
                                tc::mma_bf16(tbase + 64 * sl + 256, ad, db + ((uint64_t)(32 * SBO) >> 4),
                                             tc::idesc_bf16_f32(128, ntot - 256), acc);
                        }
                        tc::mma_commit(&empty_b[buf]);
                        last_commit = G;
                    }
                }
                if (__any_sync(0xffffffffu, *s_abort)) break;
                if (st + 1 == nst) {
                    // the tile's last commit covers all its MMAs
                    if (!tc::wait_abort_warp(&empty_b[buf], (G >> 1) & 1, s_abort, status, ST_WAIT_TIMEOUT)) break;
                    tc::fence_after_sync();
                    flush_acc(tbase, q, h, acc_hi, acc_lo);
                    tc::fence_before_sync();
                    __syncwarp();
                    if (lane == 0) tc::mbar_arrive(&tfree);
                }
            }
            if (__any_sync(0xffffffffu, *s_abort)) break;
            W++;
            // epilogue: TMEM lane rr = output row, columns 16 h + j of the block
            if (grow_e < J.m && er) {
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const int c = 16 * h + j;
                    if (c >= J.ncols) continue;
                    const int ec = s_cexp[c];
                    double v;
                    if (er == 0x7FF || ec == 0x7FF)
                        v = __longlong_as_double(0x7FF8000000000000ll);
                    else
                        v = ec ? oz::assemble_fast(acc_hi[j], acc_lo[j], (er - 1022) + (ec - 1022) - 63) : 0.0;
                    J.out[(size_t)grow_e + (size_t)(J.col0 + c) * J.ldo] = v;
                }
            } else if (grow_e < J.m) {
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const int c = 16 * h + j;
                    if (c < J.ncols) J.out[(size_t)grow_e + (size_t)(J.col0 + c) * J.ldo] = 0.0;
                }
            }
        }
    }
    // after an abort the issuer's last MMAs may still run: wait (bounded)
    if (last_commit >= 0) tc::mbar_wait(&empty_b[last_commit & 1], (last_commit >> 1) & 1);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, 512);
}

}  // namespace ozg

void map_items(const MapItem *d_items, int nitems, int *d_counter)
{
    if (nitems <= 0) return;
    cudaStream_t st = stream();
    cudaMemsetAsync(d_counter, 0, sizeof(int), st);
    cudaFuncSetAttribute(ozg::k_map_items, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ozg::MI_SMEM);
    const int grid = nitems < sm_count() ? nitems : sm_count();
    trace_begin();
    ozg::k_map_items<<<grid, ozg::OZT, ozg::MI_SMEM, st>>>(d_items, nitems, d_counter, status_ptr());
    note_launch("map_items");
}

}  // namespace lg
