// lg_ozaki.cu -- FP64-grade products of tall matrices on the BF16 tensor cores.
//
// Split-precision scheme (Ozaki-style, exponent scaled):
//   every FP64 value x of a scaling group (a column for the Gram, a row of the
//   left operand / a column of the right operand for the row map) is written
//   as x = 2^e * sum_{s<8} d_s 2^{-7(s+1)} with balanced base-128 integer
//   digits (|d_0| <= 128, |d_s| <= 64), 2^e > max|x| of the group.  Digits are
//   exact in BF16.  A product of two split values is
//   2^{e+f-14} sum_d 2^{-7d} P_d,  P_d = sum_{s+t=d} d_s d'_t,
//   and every P_d summed over K is an integer below 2^24 -- exact in the FP32
//   tensor-memory accumulators -- as long as K <= 256 rows (Gram) or K <= 64
//   (row map).  Terms with d <= 7 are kept (truncation ~2^-57 relative).
//   The digit orders d are packed side by side in TMEM (block d = 64 columns)
//   so one tcgen05.mma with N = 64*(8-s) accumulates digit s of the left
//   operand against all digits t <= 7-s of the right operand.
// All splitting and re-assembly is integer arithmetic on the IEEE bit
// patterns: GB300 runs FP64 (including FP64 conversions) at ~2 ops/clk/SM,
// so no FP64 instruction appears in the hot loops.
#include <math.h>

#include "lg_common.cuh"
#include "lg_tc.cuh"
#include "lg_ozdigits.cuh"
#include "../../include/lila_prim.h"

namespace lg {
namespace oz {

// ---------------------------------------------------------------------------
// column maximum exponents: grid (x, n), column blockIdx.y; each thread
// keeps four loads in flight (16-byte loads where the column is 16-byte
// aligned: A 16-byte aligned and lda even)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_colmax_exp(int m, int n, const double *A, int lda, int *colexp, int *status)
{
    const int c = blockIdx.y;
    const unsigned long long *col = (const unsigned long long *)(A + (size_t)c * lda);
    const size_t nth = (size_t)gridDim.x * blockDim.x, t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    int mx = 0;
    if (((uintptr_t)A & 15) == 0 && (lda & 1) == 0) {
        const ulonglong2 *c2 = (const ulonglong2 *)col;
        const size_t m2 = (size_t)m / 2;
        size_t r = t;
        for (; r + 3 * nth < m2; r += 4 * nth) {
            ulonglong2 x[4];
#pragma unroll
            for (int u = 0; u < 4; u++) x[u] = c2[r + u * nth];
#pragma unroll
            for (int u = 0; u < 4; u++) mx = max(mx, max(bexp(x[u].x), bexp(x[u].y)));
        }
        for (; r < m2; r += nth) {
            const ulonglong2 x = c2[r];
            mx = max(mx, max(bexp(x.x), bexp(x.y)));
        }
        if ((m & 1) && t == 0) mx = max(mx, bexp(col[m - 1]));
    } else {
        for (size_t r = t; r < (size_t)m; r += nth) mx = max(mx, bexp(col[r]));
    }
    mx = __reduce_max_sync(0xffffffffu, mx);
    __shared__ int red[32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x < 32) {
        mx = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0;
        mx = __reduce_max_sync(0xffffffffu, mx);
        if (threadIdx.x == 0) {
            if (mx == 0x7FF) atomicOr(status, ST_NONFINITE);
            atomicMax(&colexp[c], mx);
        }
    }
}

// ---------------------------------------------------------------------------
// Gram G = A^T A, A m x n (n <= 64), FP64-grade.
//   One persistent CTA per SM (256 threads), a contiguous row range each.
//   Stage = 64 rows x 64 columns x 8 digit slices in SMEM (64 KB), 3 stages.
//   SMEM operand index (M/N) = slice*64 + column, K = row in the stage.
//   Per 16-row K step, 6 MMAs (M = 128 covers slices s, s+1):
//     s in {0,2,4,6}: D[64 s : 512) += [slice s; slice s+1] x [slices 0..7-s].
//   TMEM lanes 0-63 accumulate digit order d in block d, lanes 64-127 order
//   d+1 in block d.  Every 256 rows the FP32 blocks (exact integers) are
//   folded into per-thread int64 accumulators hi = sum_{d<=3} P_d 2^{7(3-d)},
//   lo = sum_{4<=d<=7} P_d 2^{7(7-d)}.
// ---------------------------------------------------------------------------
constexpr int G_KC = 64;                    // rows per stage
constexpr int G_STAGES = 3;
constexpr uint32_t G_SBO = (G_KC / 8) * 128;  // 1024
constexpr uint32_t G_SLICE = 8 * G_SBO;       // 8192 bytes per slice
constexpr uint32_t G_STAGE_BYTES = NS * G_SLICE;  // 65536
constexpr int G_FLUSH_STAGES = 2;           // 128 rows between flushes (|P_d| < 2^22)
// per-warp transpose scratch: 8 columns x 32 rows, column stride 34 doubles
// (272 bytes: 16-byte aligned, and the 16-byte reads of a warp spread over
// the banks)
constexpr int G_TLD = 34;
constexpr uint32_t G_SCRATCH_BYTES = 16 * 8 * G_TLD * 8;  // 34,816

}  // namespace oz

// A uniform split of one matrix: CTA w takes rows [w rows_per, (w+1)
// rows_per) and partial slot w.
struct GramArgs {
    const double *A;
    int lda, m, n, rows_per;
    const int *colexp;
    long long *partial;
    const int *pred;  // the launch does nothing when *pred == 0 (null: always runs)
};

namespace oz {

// 512 threads (16 warps): the 512 load units of a stage (64 columns x 8
// groups of 8 rows) one per thread; TMEM lane L = 32 (warp % 4) + lane and
// Gram columns 16 (warp / 4) + [0, 16) per thread.  No block-wide barrier in
// the stage loop: each warp splits its units of stage st into buffer st % 3
// after that buffer's empty mbarrier shows the tensor core has read stage
// st - 3, then arrives on full; lane 0 of the last warp issues the stage's
// MMAs once all 16 warps have arrived and commits to empty.  After a flush
// window every warp arrives on tfree, which the issuer waits for before the
// next window's first (overwriting) MMA.
constexpr int GRAM_NT = 512;

__global__ void __launch_bounds__(GRAM_NT, 1) k_ozaki_gram(GramArgs g, int *status)
{
    if (g.pred && !*g.pred) return;
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t empty_b[G_STAGES], full_b[G_STAGES], tfree;
    __shared__ uint32_t tmem_base_s;
    __shared__ int s_abort_v;
    volatile int *s_abort = &s_abort_v;
    __shared__ int s_exp[64];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (tid == 0) {
        for (int b = 0; b < G_STAGES; b++) {
            tc::mbar_init(&empty_b[b], 1);
            tc::mbar_init(&full_b[b], GRAM_NT / 32);
        }
        tc::mbar_init(&tfree, GRAM_NT / 32);
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
    const uint32_t sbase = tc::smem_u32(smem);
    const int q = warp & 3, h = warp >> 2;
    const int L = 32 * q + lane;
    const bool top = L < 64;
    const double *A = g.A;
    const int lda = g.lda, n = g.n;
    const int r_beg = blockIdx.x * g.rows_per;
    const int r_end = min(g.m, r_beg + g.rows_per);
    long long *partial = g.partial + (size_t)blockIdx.x * 8192;
    const int nstage = r_end > r_beg ? (r_end - r_beg + G_KC - 1) / G_KC : 0;
    if (tid < 64) s_exp[tid] = tid < n ? g.colexp[tid] : 0;
    long long acc_hi[16], acc_lo[16];
#pragma unroll
    for (int j = 0; j < 16; j++) {
        acc_hi[j] = 0;
        acc_lo[j] = 0;
    }
    __syncthreads();
    // this thread's unit: column uc, 8-row group uk (8 consecutive threads take
    // 8 consecutive columns so their 16-byte stores fill one 128-byte line).
    // A warp's units are 8 columns x 32 rows; the warp loads them coalesced
    // (lane = row, one column per load: 256 contiguous bytes) and transposes
    // them through its own scratch; the values of stage st + 1 are loaded
    // while stage st is split and issued
    const int uc = ((tid >> 6) << 3) | (tid & 7), uk = (tid >> 3) & 7;
    const int wc0 = (tid >> 6) << 3, wr0 = 32 * ((tid >> 5) & 1);  // the warp's first column and row
    double *scr = (double *)(smem + G_STAGES * G_STAGE_BYTES) + (size_t)warp * 8 * G_TLD;
    unsigned long long rv[8];
    auto load_stage = [&](int st2) {
        const int row = r_beg + st2 * G_KC + wr0 + lane;
#pragma unroll
        for (int i = 0; i < 8; i++)
            rv[i] = (st2 < nstage && wc0 + i < n && row < r_end)
                        ? ((const unsigned long long *)A)[(size_t)row + (size_t)(wc0 + i) * lda]
                        : 0ull;
    };
    const bool issuer = warp == GRAM_NT / 32 - 1 && lane == 0;
    int last_commit = -1;
    load_stage(0);
    for (int st = 0; st < nstage; st++) {
        const int buf = st % G_STAGES;
        // buffer buf's previous stage (st - 3) has been read by the tensor core
        if (st >= G_STAGES &&
            !tc::wait_abort_warp(&empty_b[buf], ((st - G_STAGES) / G_STAGES) & 1, s_abort, status, ST_WAIT_TIMEOUT))
            break;
        uint8_t *stage = smem + (size_t)buf * G_STAGE_BYTES;
        {
            // transpose: lane = row of column wc0 + i -> unit (column uc, rows 8 uk' .. + 8)
            __syncwarp();
#pragma unroll
            for (int i = 0; i < 8; i++) scr[i * G_TLD + lane] = __longlong_as_double((long long)rv[i]);
            __syncwarp();
            unsigned long long uv[8];
            const double2 *src = (const double2 *)(scr + (uc & 7) * G_TLD + 8 * (uk & 3));
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const double2 d = src[k];
                uv[2 * k] = (unsigned long long)__double_as_longlong(d.x);
                uv[2 * k + 1] = (unsigned long long)__double_as_longlong(d.y);
            }
            const int emax = s_exp[uc];
#pragma unroll
            for (int hf = 0; hf < 2; hf++) {
                uint32_t w01[NS], w23[NS];
                digit_pair(fixed56(uv[4 * hf], emax), fixed56(uv[4 * hf + 1], emax), w01);
                digit_pair(fixed56(uv[4 * hf + 2], emax), fixed56(uv[4 * hf + 3], emax), w23);
#pragma unroll
                for (int s = 0; s < NS; s++)
                    *(uint2 *)(stage + s * G_SLICE + (uc >> 3) * G_SBO + uk * LBO + (uc & 7) * 16 + hf * 8) =
                        make_uint2(w01[s], w23[s]);
            }
        }
        load_stage(st + 1);  // in flight during the MMA issue and the next stage
        tc::fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&full_b[buf]);
        const bool window_start = (st % G_FLUSH_STAGES) == 0;
        if (issuer) {
            bool ok = tc::wait_abort(&full_b[buf], (st / G_STAGES) & 1, s_abort, status, ST_WAIT_TIMEOUT);
            if (ok && window_start && st > 0)
                ok = tc::wait_abort(&tfree, ((st / G_FLUSH_STAGES) - 1) & 1, s_abort, status, ST_WAIT_TIMEOUT);
            if (ok) {
                tc::fence_after_sync();
                const uint32_t sb = sbase + buf * G_STAGE_BYTES;
#pragma unroll
                for (int ks = 0; ks < G_KC / 16; ks++) {
                    const uint32_t koff = ks * 2 * LBO;
#pragma unroll
                    for (int s = 0; s < NS; s += 2) {
                        const int ntot = 64 * (NS - s);
                        const uint64_t ad = tc::desc_nosw(sb + s * G_SLICE + koff, LBO, G_SBO);
                        const uint32_t acc = (window_start && ks == 0 && s == 0) ? 0u : 1u;
                        const int n1 = ntot < 256 ? ntot : 256;
                        tc::mma_bf16(tbase + 64 * s, ad, tc::desc_nosw(sb + koff, LBO, G_SBO),
                                     tc::idesc_bf16_f32(128, n1), acc);
                        if (ntot > 256)
                            tc::mma_bf16(tbase + 64 * s + 256, ad, tc::desc_nosw(sb + 32 * G_SBO + koff, LBO, G_SBO),
                                         tc::idesc_bf16_f32(128, ntot - 256), acc);
                    }
                }
                tc::mma_commit(&empty_b[buf]);
                last_commit = st;
            }
        }
        if (__any_sync(0xffffffffu, *s_abort)) break;
        const bool flush = ((st + 1) % G_FLUSH_STAGES) == 0 || st == nstage - 1;
        if (flush) {
            // this stage's commit also covers every earlier MMA (in-order issue)
            if (!tc::wait_abort_warp(&empty_b[buf], (st / G_STAGES) & 1, s_abort, status, ST_WAIT_TIMEOUT)) break;
            tc::fence_after_sync();
            // top lanes hold order d in block d, bottom lanes order d in
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
                        const long long x = combine4(v[0][j], v[1][j], v[2][j], v[3][j]);
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
    // after an abort the issuer's last MMAs may still run: wait (bounded) for
    // its last commit before TMEM is released
    if (last_commit >= 0) tc::mbar_wait(&empty_b[last_commit % G_STAGES], (last_commit / G_STAGES) & 1);
    __syncthreads();
    if (!*s_abort) {
        // every MMA has completed (the last stage flushed); combine the two TMEM
        // halves through shared memory (bottom lanes hand over)
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        long long *xh = (long long *)smem;
        long long *xl = xh + 64 * 64;
        if (!top) {
#pragma unroll
            for (int j = 0; j < 16; j++) {
                const int i = L - 64, c = 16 * h + j;
                xh[i * 64 + c] = acc_hi[j];
                xl[i * 64 + c] = acc_lo[j];
            }
        }
        __syncthreads();
        if (top) {
            // integer partials: the parts of one matrix share its column
            // scales, so their sum is exact and G is rounded once
            long long *ph = partial;
            long long *pl = ph + 4096;
#pragma unroll
            for (int j = 0; j < 16; j++) {
                const int c = 16 * h + j;
                ph[L + 64 * c] = acc_hi[j] + xh[L * 64 + c];
                pl[L + 64 * c] = acc_lo[j] + xl[L * 64 + c];
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, 512);
}

// G(i, c) from the CTAs' integer partials: eight threads per entry split the
// parts and add their int64 sums by shuffles (exact in any order), so the
// reduction spreads over many SMs; G is rounded once.
__global__ void k_gram_reduce(int n, int nparts, const long long *partial, const int *colexp, double *G, int ldg,
                              const int *pred)
{
    if (pred && !*pred) return;
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;
    const int idx = gid >> 3, l = gid & 7;
    const bool ok = idx < n * n;
    const int i = ok ? idx % n : 0, c = ok ? idx / n : 0;
    long long hi = 0, lo = 0;
    if (ok)
        for (int p = l; p < nparts; p += 8) {
            hi += partial[(size_t)p * 8192 + i + 64 * c];
            lo += partial[(size_t)p * 8192 + 4096 + i + 64 * c];
        }
    for (int o = 1; o < 8; o <<= 1) {
        hi += __shfl_xor_sync(0xffffffffu, hi, o);
        lo += __shfl_xor_sync(0xffffffffu, lo, o);
    }
    if (ok && l == 0) {
        const int ei = colexp[i], ec = colexp[c];
        G[(size_t)i + (size_t)c * ldg] = (ei && ec) ? assemble(hi, lo, (ei - 1022) + (ec - 1022) - 63) : 0.0;
    }
}

// ---------------------------------------------------------------------------
// Row map out = A X, A m x n (n <= 64), X n x nout (nout <= 64), FP64-grade.
//   Tile = 128 rows.  A digits per row (row scale), X digits per output
//   column (column scale).  SMEM: A tile 8 slices x 128 x 64 BF16 (128 KB),
//   X digits 8 slices x 64 x 64 (64 KB, loaded once per CTA).
//   Per K step (K = 64 -> 4 steps): for s = 0..7,
//     D[64 s : 512) += A_s x [X_0 .. X_{7-s}]      (N = 64 (8 - s))
//   so TMEM block d holds P_d for all 64 output columns of the tile.
// ---------------------------------------------------------------------------
constexpr uint32_t M_SBO = 1024;              // (64 / 8) * 128
constexpr uint32_t M_ASLICE = 16 * M_SBO;     // 128 rows -> 16 KB per slice
constexpr uint32_t M_XSLICE = 8 * M_SBO;      // 64 columns -> 8 KB per slice
constexpr uint32_t M_A_BYTES = NS * M_ASLICE; // 131072
constexpr uint32_t M_X_BYTES = NS * M_XSLICE; // 65536

}  // namespace oz

// One problem whose 128-row tiles are spread over the CTAs.
struct MapArgs {
    MapJob one;
    int *colexp_out;  // column scales of out (64 ints, zeroed), or null
    const int *pred;  // the launch does nothing when *pred == 0 (null: always runs)
    const int *rexp_in;  // row scales of A (m ints: the largest biased exponent of each row), or null
    int *rexp_out;       // receives the row scales of out (m ints), or null
};

namespace oz {

// 512 threads (16 warps): thread -> row r = tid % 128 of a tile and column
// groups kg = tid / 128 + 4 p (p = 0, 1); in the epilogue warp w reads TMEM
// lanes 32 (w % 4) .. + 32 and output columns 16 (w / 4) .. + 16.
constexpr int MAP_NT = 512;

__global__ void __launch_bounds__(MAP_NT, 1) k_ozaki_map(MapArgs args, int *status)
{
    if (args.pred && !*args.pred) return;
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sA = smem;
    uint8_t *sX = smem + M_A_BYTES;
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base_s;
    __shared__ int s_xexp[64];
    __shared__ int s_rexp[4][128];
    __shared__ int s_abort;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (tid == 0) {
        tc::mbar_init(&mbar, 1);
        tc::fence_mbar_init();
        s_abort = 0;
    }
    if (warp == 0) {
        tc::tmem_alloc(&tmem_base_s, 512);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = tmem_base_s;
    const uint32_t aaddr = tc::smem_u32(sA), xaddr = tc::smem_u32(sX);
    const int q = warp & 3, h = warp >> 2;
    uint32_t parity = 0;
    const MapJob J = args.one;
    const int m = J.m, n = J.n, nout = J.nout, lda = J.lda, ldo = J.ldo;
    const double *A = J.A;
    double *out = J.out;
    // X column scales, then X digits (unit = (output column j, 8-row group kg of X))
    if (tid < 64) {
        int mx = 0;
        if (tid < nout)
            for (int k = 0; k < n; k++)
                mx = max(mx, bexp(((const unsigned long long *)J.X)[(size_t)k + (size_t)tid * J.ldx]));
        s_xexp[tid] = mx;
    }
    __syncthreads();
    {
        const int j = tid >> 3, kg = tid & 7;  // 512 units, one per thread
#pragma unroll
        for (int hf = 0; hf < 2; hf++) {
            long long Xv[4];
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int k = kg * 8 + 4 * hf + e;
                const unsigned long long b =
                    (j < nout && k < n) ? ((const unsigned long long *)J.X)[(size_t)k + (size_t)j * J.ldx] : 0ull;
                Xv[e] = fixed56(b, s_xexp[j]);
            }
            uint32_t w01[NS], w23[NS];
            digit_pair(Xv[0], Xv[1], w01);
            digit_pair(Xv[2], Xv[3], w23);
#pragma unroll
            for (int t = 0; t < NS; t++)
                *(uint2 *)(sX + t * M_XSLICE + (j >> 3) * M_SBO + kg * LBO + (j & 7) * 16 + hf * 8) =
                    make_uint2(w01[t], w23[t]);
        }
    }
    const int ntiles = (m + 127) / 128;
    // the rows of tile i + 1 are loaded into vb while tile i's MMAs and
    // epilogue run (the split of tile i has consumed vb by then)
    const int r = tid & 127, quarter = tid >> 7;
    unsigned long long vb[2][8];
    auto load_tile = [&](int tl) {
        const int grow = tl * 128 + r;
#pragma unroll
        for (int p = 0; p < 2; p++) {
            const int kg = quarter + 4 * p;
#pragma unroll
            for (int e = 0; e < 8; e++) {
                const int k = kg * 8 + e;
                vb[p][e] = (tl < ntiles && grow < m && k < n)
                               ? ((const unsigned long long *)A)[(size_t)grow + (size_t)k * lda]
                               : 0ull;
            }
        }
    };
    uint32_t cmax0[4] = {0, 0, 0, 0}, cmax1[4] = {0, 0, 0, 0};  // output column scales (packed pairs)
    load_tile(blockIdx.x);
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int row0 = tile * 128;
        int mx = 0;
#pragma unroll
        for (int p = 0; p < 2; p++)
#pragma unroll
            for (int e = 0; e < 8; e++) mx = max(mx, bexp(vb[p][e]));
        s_rexp[quarter][r] = mx;
        __syncthreads();
        const int emax = max(max(s_rexp[0][r], s_rexp[1][r]), max(s_rexp[2][r], s_rexp[3][r]));
        // K half p (column groups 4p .. 4p + 3, interleaved with the other half
        // in the core matrices) is split, then its MMAs are issued, so the
        // MMAs of half 0 run while half 1 is split
#pragma unroll
        for (int p = 0; p < 2; p++) {
            const int kg = quarter + 4 * p;
#pragma unroll
            for (int hf = 0; hf < 2; hf++) {
                uint32_t w01[NS], w23[NS];
                digit_pair(fixed56(vb[p][4 * hf], emax), fixed56(vb[p][4 * hf + 1], emax), w01);
                digit_pair(fixed56(vb[p][4 * hf + 2], emax), fixed56(vb[p][4 * hf + 3], emax), w23);
#pragma unroll
                for (int s = 0; s < NS; s++)
                    *(uint2 *)(sA + s * M_ASLICE + (r >> 3) * M_SBO + kg * LBO + (r & 7) * 16 + hf * 8) =
                        make_uint2(w01[s], w23[s]);
            }
            tc::fence_proxy_async_smem();
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
            if (p == 1) load_tile(tile + gridDim.x);  // in flight during the MMAs and the epilogue
            if (tid == 0) {
#pragma unroll
                for (int kk = 0; kk < 2; kk++) {
                    const int ks = 2 * p + kk;
                    const uint32_t koff = ks * 2 * LBO;
#pragma unroll
                    for (int s = 0; s < NS; s++) {
                        const int ntot = 64 * (NS - s);
                        const uint64_t ad = tc::desc_nosw(aaddr + s * M_ASLICE + koff, LBO, M_SBO);
                        const uint32_t acc = (ks == 0 && s == 0) ? 0u : 1u;
                        const int n1 = ntot < 256 ? ntot : 256;
                        tc::mma_bf16(tbase + 64 * s, ad, tc::desc_nosw(xaddr + koff, LBO, M_SBO),
                                     tc::idesc_bf16_f32(128, n1), acc);
                        if (ntot > 256)
                            tc::mma_bf16(tbase + 64 * s + 256, ad,
                                         tc::desc_nosw(xaddr + 32 * M_SBO + koff, LBO, M_SBO),
                                         tc::idesc_bf16_f32(128, ntot - 256), acc);
                    }
                }
                if (p == 1) tc::mma_commit(&mbar);
            }
        }
        if (!tc::mbar_wait(&mbar, parity)) {
            if (tid == 0) atomicOr(status, ST_WAIT_TIMEOUT);
            s_abort = 1;
        }
        parity ^= 1u;
        tc::fence_after_sync();
        if (!s_abort) {
            // epilogue: lane row 32q + lane, output columns 16h + [0, 16) in two
            // chunks of 8; orders 0..3 then 4..7 (four TMEM loads each)
            const int rr = 32 * q + lane;
            const int orow = row0 + rr;
            const int er = max(max(s_rexp[0][rr], s_rexp[1][rr]), max(s_rexp[2][rr], s_rexp[3][rr]));
#pragma unroll 1
            for (int ch = 0; ch < 2; ch++) {
                const uint32_t col = (uint32_t)(16 * h + 8 * ch);
                long long hi[8], lo[8];
                {
                    uint32_t v[4][8];
#pragma unroll
                    for (int d = 0; d < 4; d++)
                        tc::tmem_ld8(tbase + ((uint32_t)(32 * q) << 16) + (uint32_t)(64 * d) + col, v[d]);
                    tc::tmem_ld_wait();
#pragma unroll
                    for (int j = 0; j < 8; j++) hi[j] = combine4(v[0][j], v[1][j], v[2][j], v[3][j]);
                }
                {
                    uint32_t v[4][8];
#pragma unroll
                    for (int d = 0; d < 4; d++)
                        tc::tmem_ld8(tbase + ((uint32_t)(32 * q) << 16) + (uint32_t)(64 * (d + 4)) + col, v[d]);
                    tc::tmem_ld_wait();
#pragma unroll
                    for (int j = 0; j < 8; j++) lo[j] = combine4(v[0][j], v[1][j], v[2][j], v[3][j]);
                }
                if (orow < m) {
                    uint32_t ex[8];
#pragma unroll
                    for (int j = 0; j < 8; j++) {
                        const int c = (int)col + j;
                        ex[j] = 0;
                        if (c < nout) {
                            const int fx = s_xexp[c];
                            const double v =
                                (er && fx) ? assemble_fast(hi[j], lo[j], (er - 1022) + (fx - 1022) - 63) : 0.0;
                            out[(size_t)orow + (size_t)c * ldo] = v;
                            ex[j] = (uint32_t)bexp((unsigned long long)__double_as_longlong(v));
                        }
                    }
                    // running column maxima, two 16-bit exponents per word
#pragma unroll
                    for (int p = 0; p < 4; p++) {
                        const uint32_t pr = ex[2 * p] | (ex[2 * p + 1] << 16);
                        if (ch == 0)
                            cmax0[p] = __vmaxu2(cmax0[p], pr);
                        else
                            cmax1[p] = __vmaxu2(cmax1[p], pr);
                    }
                }
            }
        }
        tc::fence_before_sync();
        __syncthreads();
        if (s_abort) break;
    }
    if (args.colexp_out) {
        // this warp's 16 output columns: maxima over its lanes (rows), then
        // over the CTAs by atomicMax
#pragma unroll
        for (int ch = 0; ch < 2; ch++)
#pragma unroll
            for (int p = 0; p < 4; p++) {
                uint32_t v = ch == 0 ? cmax0[p] : cmax1[p];
                for (int o = 16; o > 0; o >>= 1) v = __vmaxu2(v, __shfl_xor_sync(0xffffffffu, v, o));
                if (lane == 0) {
#pragma unroll
                    for (int hw = 0; hw < 2; hw++) {
                        const int c = 16 * h + 8 * ch + 2 * p + hw;
                        const int e = (int)((v >> (16 * hw)) & 0xFFFFu);
                        if (c < nout && e) {
                            if (e == 0x7FF) atomicOr(status, ST_NONFINITE);
                            atomicMax(&args.colexp_out[c], e);
                        }
                    }
                }
            }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, 512);
}

// ---------------------------------------------------------------------------
// The row map with the row scales of A given (rexp_in: the scale pre-pass or
// the map that produced A wrote them), on the same tiles, digits and TMEM
// layout as k_ozaki_map.  With the scales known, a tile's first K half can be
// split before its second half is loaded, so the schedule runs one half
// ahead: the next tile's first half is split while the tensor core runs this
// tile's second half, and its second half while the tensor core runs its
// first half after this tile's epilogue; the rows of the tile after next are
// loaded half by half as the registers free up.  Two commits per tile
// (mbar0 after the first half's MMAs, mbar1 after the second's).  Writes the
// row scales of out when rexp_out is given (the next map's rexp_in).  The
// outputs are bit-identical to k_ozaki_map's.
// ---------------------------------------------------------------------------
// kScales: the launch tracks out's column scales (colexp_out) and row
// scales (rexp_out); the final maps of a leaf need neither.
template <bool kScales>
__global__ void __launch_bounds__(MAP_NT, 1) k_ozaki_map_pre(MapArgs args, int *status)
{
    if (args.pred && !*args.pred) return;
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sA = smem;
    uint8_t *sX = smem + M_A_BYTES;
    __shared__ __align__(8) uint64_t mbar0, mbar1, drain;
    __shared__ uint32_t tmem_base_s;
    __shared__ int s_xexp[64];
    __shared__ int s_er[2][128];     // row scales of the tiles in flight (tile parity)
    __shared__ int s_omax[4][128];   // the four column groups' output row maxima
    __shared__ int s_abort;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        tc::mbar_init(&mbar0, 1);
        tc::mbar_init(&mbar1, 1);
        tc::mbar_init(&drain, 1);
        tc::fence_mbar_init();
        s_abort = 0;
    }
    if (warp == 0) {
        tc::tmem_alloc(&tmem_base_s, 512);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = tmem_base_s;
    const uint32_t aaddr = tc::smem_u32(sA), xaddr = tc::smem_u32(sX);
    const int q = warp & 3, h = warp >> 2;
    const MapJob J = args.one;
    const int m = J.m, n = J.n, nout = J.nout, lda = J.lda, ldo = J.ldo;
    const double *A = J.A;
    double *out = J.out;
    const int *rexp_in = args.rexp_in;
    // X column scales, then X digits (as k_ozaki_map)
    if (tid < 64) {
        int mx = 0;
        if (tid < nout)
            for (int k = 0; k < n; k++)
                mx = max(mx, bexp(((const unsigned long long *)J.X)[(size_t)k + (size_t)tid * J.ldx]));
        s_xexp[tid] = mx;
    }
    __syncthreads();
    {
        const int j = tid >> 3, kg = tid & 7;
#pragma unroll
        for (int hf = 0; hf < 2; hf++) {
            long long Xv[4];
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int k = kg * 8 + 4 * hf + e;
                const unsigned long long b =
                    (j < nout && k < n) ? ((const unsigned long long *)J.X)[(size_t)k + (size_t)j * J.ldx] : 0ull;
                Xv[e] = fixed56(b, s_xexp[j]);
            }
            uint32_t w01[NS], w23[NS];
            digit_pair(Xv[0], Xv[1], w01);
            digit_pair(Xv[2], Xv[3], w23);
#pragma unroll
            for (int t = 0; t < NS; t++)
                *(uint2 *)(sX + t * M_XSLICE + (j >> 3) * M_SBO + kg * LBO + (j & 7) * 16 + hf * 8) =
                    make_uint2(w01[t], w23[t]);
        }
    }
    const int ntiles = (m + 127) / 128;
    const int r = tid & 127, quarter = tid >> 7;
    unsigned long long vb[2][8];
    auto load_half = [&](int tl, int p) {
        const int grow = tl * 128 + r;
        const int kg = quarter + 4 * p;
#pragma unroll
        for (int e = 0; e < 8; e++) {
            const int k = kg * 8 + e;
            vb[p][e] = (tl < ntiles && grow < m && k < n)
                           ? ((const unsigned long long *)A)[(size_t)grow + (size_t)k * lda]
                           : 0ull;
        }
    };
    auto row_scale = [&](int tl) { return (tl < ntiles && tl * 128 + r < m) ? rexp_in[(size_t)tl * 128 + r] : 0; };
    // K half p of this thread's row (column group quarter + 4 p) into the digit buffer
    auto split_half = [&](int p, int emax) {
        const int kg = quarter + 4 * p;
#pragma unroll
        for (int hf = 0; hf < 2; hf++) {
            uint32_t w01[NS], w23[NS];
            digit_pair(fixed56(vb[p][4 * hf], emax), fixed56(vb[p][4 * hf + 1], emax), w01);
            digit_pair(fixed56(vb[p][4 * hf + 2], emax), fixed56(vb[p][4 * hf + 3], emax), w23);
#pragma unroll
            for (int s = 0; s < NS; s++)
                *(uint2 *)(sA + s * M_ASLICE + (r >> 3) * M_SBO + kg * LBO + (r & 7) * 16 + hf * 8) =
                    make_uint2(w01[s], w23[s]);
        }
        tc::fence_proxy_async_smem();
    };
    auto issue_half = [&](int p) {
#pragma unroll
        for (int kk = 0; kk < 2; kk++) {
            const int ks = 2 * p + kk;
            const uint32_t koff = ks * 2 * LBO;
#pragma unroll
            for (int s = 0; s < NS; s++) {
                const int ntot = 64 * (NS - s);
                const uint64_t ad = tc::desc_nosw(aaddr + s * M_ASLICE + koff, LBO, M_SBO);
                const uint32_t acc = (ks == 0 && s == 0) ? 0u : 1u;
                const int n1 = ntot < 256 ? ntot : 256;
                tc::mma_bf16(tbase + 64 * s, ad, tc::desc_nosw(xaddr + koff, LBO, M_SBO), tc::idesc_bf16_f32(128, n1),
                             acc);
                if (ntot > 256)
                    tc::mma_bf16(tbase + 64 * s + 256, ad, tc::desc_nosw(xaddr + 32 * M_SBO + koff, LBO, M_SBO),
                                 tc::idesc_bf16_f32(128, ntot - 256), acc);
            }
        }
        tc::mma_commit(p == 0 ? &mbar0 : &mbar1);
    };
    auto sync_digits = [&]() {
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
    };
    uint32_t cmax0[4] = {0, 0, 0, 0}, cmax1[4] = {0, 0, 0, 0};  // output column scales (packed pairs)
    int tile = blockIdx.x;
    int en_pre = 0;  // the next tile's row scale, loaded one tile ahead with its first half
    if (tile < ntiles) {
        // prologue: the first tile's two halves, the next tile's rows loaded as they free up
        const int e0 = row_scale(tile);
        load_half(tile, 0);
        load_half(tile, 1);
        if (quarter == 0) s_er[0][r] = e0;
        split_half(0, e0);
        sync_digits();
        if (tid == 0) issue_half(0);
        load_half(tile + gridDim.x, 0);
        en_pre = row_scale(tile + gridDim.x);
        split_half(1, e0);
        sync_digits();
        if (tid == 0) issue_half(1);
        load_half(tile + gridDim.x, 1);
    }
    for (int it = 0; tile < ntiles; tile += gridDim.x, it++) {
        const int next = tile + gridDim.x;
        const bool has_next = next < ntiles;
        const int en = en_pre;
        if (has_next) {
            if (quarter == 0) s_er[(it + 1) & 1][r] = en;
            // the tensor core has read this tile's first half: the next tile's first half goes in
            if (!tc::mbar_wait(&mbar0, it & 1)) {
                if (tid == 0) atomicOr(status, ST_WAIT_TIMEOUT);
                s_abort = 1;
            }
            split_half(0, en);
            load_half(next + gridDim.x, 0);
            en_pre = row_scale(next + gridDim.x);
        }
        if (!tc::mbar_wait(&mbar1, it & 1)) {
            if (tid == 0) atomicOr(status, ST_WAIT_TIMEOUT);
            s_abort = 1;
        }
        tc::fence_after_sync();
        if (!s_abort) {
            // epilogue (as k_ozaki_map): lane row 32q + lane, output columns 16h + [0, 16)
            const int rr = 32 * q + lane;
            const int orow = tile * 128 + rr;
            const int er = s_er[it & 1][rr];
            int omax = 0;
#pragma unroll 1
            for (int ch = 0; ch < 2; ch++) {
                const uint32_t col = (uint32_t)(16 * h + 8 * ch);
                long long hi[8], lo[8];
                {
                    uint32_t v[4][8];
#pragma unroll
                    for (int d = 0; d < 4; d++)
                        tc::tmem_ld8(tbase + ((uint32_t)(32 * q) << 16) + (uint32_t)(64 * d) + col, v[d]);
                    tc::tmem_ld_wait();
#pragma unroll
                    for (int j = 0; j < 8; j++) hi[j] = combine4(v[0][j], v[1][j], v[2][j], v[3][j]);
                }
                {
                    uint32_t v[4][8];
#pragma unroll
                    for (int d = 0; d < 4; d++)
                        tc::tmem_ld8(tbase + ((uint32_t)(32 * q) << 16) + (uint32_t)(64 * (d + 4)) + col, v[d]);
                    tc::tmem_ld_wait();
#pragma unroll
                    for (int j = 0; j < 8; j++) lo[j] = combine4(v[0][j], v[1][j], v[2][j], v[3][j]);
                }
                if (orow < m) {
                    uint32_t ex[8];
#pragma unroll
                    for (int j = 0; j < 8; j++) {
                        const int c = (int)col + j;
                        ex[j] = 0;
                        if (c < nout) {
                            const int fx = s_xexp[c];
                            const double v =
                                (er && fx) ? assemble_fast(hi[j], lo[j], (er - 1022) + (fx - 1022) - 63) : 0.0;
                            out[(size_t)orow + (size_t)c * ldo] = v;
                            if (kScales) {
                                ex[j] = (uint32_t)bexp((unsigned long long)__double_as_longlong(v));
                                omax = max(omax, (int)ex[j]);
                            }
                        }
                    }
                    if (kScales) {
#pragma unroll
                        for (int p = 0; p < 4; p++) {
                            const uint32_t pr = ex[2 * p] | (ex[2 * p + 1] << 16);
                            if (ch == 0)
                                cmax0[p] = __vmaxu2(cmax0[p], pr);
                            else
                                cmax1[p] = __vmaxu2(cmax1[p], pr);
                        }
                    }
                }
            }
            if (kScales) s_omax[h][rr] = omax;
        }
        sync_digits();  // TMEM drained, the next tile's first-half digits and s_omax visible
        if (s_abort) break;
        if (kScales && args.rexp_out && warp < 4) {
            const int rr = 32 * q + lane, orow = tile * 128 + rr;
            if (orow < m)
                args.rexp_out[orow] = max(max(s_omax[0][rr], s_omax[1][rr]), max(s_omax[2][rr], s_omax[3][rr]));
        }
        if (has_next) {
            if (tid == 0) issue_half(0);
            split_half(1, en);
            sync_digits();
            if (tid == 0) issue_half(1);
            load_half(next + gridDim.x, 1);
        }
    }
    if (kScales && args.colexp_out) {
#pragma unroll
        for (int ch = 0; ch < 2; ch++)
#pragma unroll
            for (int p = 0; p < 4; p++) {
                uint32_t v = ch == 0 ? cmax0[p] : cmax1[p];
                for (int o = 16; o > 0; o >>= 1) v = __vmaxu2(v, __shfl_xor_sync(0xffffffffu, v, o));
                if (lane == 0) {
#pragma unroll
                    for (int hw = 0; hw < 2; hw++) {
                        const int c = 16 * h + 8 * ch + 2 * p + hw;
                        const int e = (int)((v >> (16 * hw)) & 0xFFFFu);
                        if (c < nout && e) {
                            if (e == 0x7FF) atomicOr(status, ST_NONFINITE);
                            atomicMax(&args.colexp_out[c], e);
                        }
                    }
                }
            }
    }
    // every MMA this CTA issued is complete before TMEM is freed
    if (tid == 0) {
        tc::mma_commit(&drain);
        tc::mbar_wait(&drain, 0);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, 512);
}

// Row and column scales of A (m x n, n <= 64) in one pass: rexp[r] (m ints,
// may be null) the largest biased exponent of row r, colexp (64 ints,
// zeroed) the largest of each column (atomicMax over the CTAs).  A CTA takes
// 2048 consecutive rows, warp w rows 256 w .. + 256 of them, lane l the row
// pairs 64 k + 2 l (k = 0..3), so that each load of a column is 512
// contiguous bytes per warp (16-byte loads where A's columns are 16-byte
// aligned); column maxima go through shared-memory atomics.
__global__ void __launch_bounds__(256) k_scales_rc(int m, int n, const double *A, int lda, int *colexp, int *rexp,
                                                   int *status)
{
    __shared__ int s_cmax[64];
    if (threadIdx.x < 64) s_cmax[threadIdx.x] = 0;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned long long *a = (const unsigned long long *)A;
    const bool vec = ((uintptr_t)A & 15) == 0 && (lda & 1) == 0;
    for (size_t r0 = (size_t)blockIdx.x * 2048; r0 < (size_t)m; r0 += (size_t)gridDim.x * 2048) {
        const size_t rw = r0 + 256 * (size_t)warp + 2 * lane;  // this lane's first row pair
        const bool full = rw + 192 + 2 <= (size_t)m;          // all four pairs inside A
        int rm[8];
#pragma unroll
        for (int e = 0; e < 8; e++) rm[e] = 0;
#pragma unroll 4
        for (int c = 0; c < n; c++) {
            const unsigned long long *col = a + (size_t)c * lda;
            unsigned long long v[8];
            if (vec && full) {
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const ulonglong2 x = *(const ulonglong2 *)(col + rw + 64 * k);
                    v[2 * k] = x.x;
                    v[2 * k + 1] = x.y;
                }
            } else {
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const size_t r = rw + 64 * k;
                    v[2 * k] = r < (size_t)m ? col[r] : 0ull;
                    v[2 * k + 1] = r + 1 < (size_t)m ? col[r + 1] : 0ull;
                }
            }
            int cm = 0;
#pragma unroll
            for (int e = 0; e < 8; e++) {
                const int x = bexp(v[e]);
                rm[e] = max(rm[e], x);
                cm = max(cm, x);
            }
            cm = __reduce_max_sync(0xffffffffu, cm);
            if (lane == 0 && cm) atomicMax(&s_cmax[c], cm);
        }
        if (rexp) {
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const size_t r = rw + 64 * k;
                if (r < (size_t)m) rexp[r] = rm[2 * k];
                if (r + 1 < (size_t)m) rexp[r + 1] = rm[2 * k + 1];
            }
        }
    }
    __syncthreads();
    if (threadIdx.x < n) {
        const int e = s_cmax[threadIdx.x];
        if (e) {
            if (e == 0x7FF) atomicOr(status, ST_NONFINITE);
            atomicMax(&colexp[threadIdx.x], e);
        }
    }
}

}  // namespace oz

static int g_sm_count = 0;
int sm_count()
{
    if (!g_sm_count) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_sm_count, cudaDevAttrMultiProcessorCount, dev);
        if (g_sm_count <= 0) g_sm_count = 152;
    }
    return g_sm_count;
}

// Workspace (doubles) of ozaki_gram for a grid of `parts` CTAs.
long long ozaki_gram_work(int parts) { return 64 + (long long)parts * 8192; }

bool ozaki_gram_tma(int m, int n, const double *A, int lda, int rows_per, const int *colexp, long long *partial,
                    int parts, const int *pred);
// Kernel choice of the tall split products (lila_prim_ozaki_map_path):
// 0 (default) the TMA-fed Gram where A allows TMA and the register-fed row
// map, in its one-half-ahead form where the caller passes the row scales
// (the fastest measured set; the transposed-tile map took 3.9 ms per
// 4,194,304 x 64 map against 2.0 ms); 1 both register-fed, the row map
// computing its own row scales; 2 and 3 the TMA-fed Gram and the TMA-fed
// transposed-tile row map with its outputs rounded through the FP64-pipe
// conversion (2) or integer instructions (3), the same bits.
static int g_map_path = 0;

// G = A^T A (n <= 64) to FP64 grade.  work: ozaki_gram_work(sm_count()) doubles.
int ozaki_gram(int m, int n, const double *A, int lda, double *G, int ldg, double *work, long long lwork,
               int rows_per_override, bool colexp_ready, const int *pred, int *rexp_out)
{
    if (n <= 0 || n > 64 || m < 0) return -1;
    const int parts = sm_count();
    if (lwork < ozaki_gram_work(parts)) return -2;
    int *colexp = (int *)work;
    long long *partial = (long long *)(work + 64);
    cudaStream_t st = stream();
    if (!colexp_ready) {
        cudaMemsetAsync(colexp, 0, 64 * sizeof(int), st);
        trace_break();
        trace_begin();
        if (rexp_out) {
            // the row scales too, for a following row map of A
            const int tiles = (m + 2047) / 2048, gx = tiles < sm_count() * 8 ? tiles : sm_count() * 8;
            oz::k_scales_rc<<<gx > 0 ? gx : 1, 256, 0, st>>>(m, n, A, lda, colexp, rexp_out, status_ptr());
        } else {
            const int gx = (sm_count() * 8 + n - 1) / n;  // ~8 CTAs per SM over all columns
            oz::k_colmax_exp<<<dim3(gx, n), 256, 0, st>>>(m, n, A, lda, colexp, status_ptr());
        }
        note_launch("ozaki_colmax");
    }
    const size_t smem = oz::G_STAGES * oz::G_STAGE_BYTES + oz::G_SCRATCH_BYTES;
    cudaFuncSetAttribute(oz::k_ozaki_gram, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int rows_per = (m + parts - 1) / parts;
    rows_per = (rows_per + oz::G_KC - 1) / oz::G_KC * oz::G_KC;
    if (rows_per == 0) rows_per = oz::G_KC;
    if (rows_per_override > 0) rows_per = (rows_per_override + oz::G_KC - 1) / oz::G_KC * oz::G_KC;
    if (g_map_path != 1 && ozaki_gram_tma(m, n, A, lda, rows_per, colexp, partial, parts, pred)) {
        trace_begin();
        oz::k_gram_reduce<<<(n * n * 8 + 255) / 256, 256, 0, st>>>(n, parts, partial, colexp, G, ldg, pred);
        note_launch("ozaki_gram_reduce");
        return 0;
    }
    trace_begin();
    GramArgs ga{};
    ga.A = A;
    ga.lda = lda;
    ga.m = m;
    ga.n = n;
    ga.rows_per = rows_per;
    ga.colexp = colexp;
    ga.partial = partial;
    ga.pred = pred;
    oz::k_ozaki_gram<<<parts, oz::GRAM_NT, smem, st>>>(ga, status_ptr());
    note_launch("ozaki_gram");
    trace_begin();
    oz::k_gram_reduce<<<(n * n * 8 + 255) / 256, 256, 0, st>>>(n, parts, partial, colexp, G, ldg, pred);
    note_launch("ozaki_gram_reduce");
    return 0;
}

bool ozaki_map_tma(int m, int n, const double *A, int lda, const double *X, int ldx, int nout, double *out, int ldo,
                   int *colexp_out, bool int_asm, const int *pred);

// out = A X (n, nout <= 64) to FP64 grade.  out may be A itself (each row is
// read before it is written, by the same CTA), but must not alias X.
int ozaki_map(int m, int n, const double *A, int lda, const double *X, int ldx, int nout, double *out, int ldo,
              int *colexp_out, const int *pred, const int *rexp_in, int *rexp_out)
{
    if (n <= 0 || n > 64 || nout <= 0 || nout > 64 || m < 0) return -1;
    if (colexp_out) {
        cudaMemsetAsync(colexp_out, 0, 64 * sizeof(int), stream());
        trace_break();
    }
    if (m == 0) return 0;
    if (g_map_path >= 2 && ozaki_map_tma(m, n, A, lda, X, ldx, nout, out, ldo, colexp_out, g_map_path == 3, pred))
        return 0;
    const size_t smem = oz::M_A_BYTES + oz::M_X_BYTES;
    cudaFuncSetAttribute(oz::k_ozaki_map, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int tiles = (m + 127) / 128;
    int grid = tiles < sm_count() ? tiles : sm_count();
    MapArgs ma{};
    ma.one = MapJob{A, lda, m, n, X, ldx, nout, out, ldo};
    ma.colexp_out = colexp_out;
    ma.pred = pred;
    ma.rexp_in = rexp_in;
    ma.rexp_out = rexp_out;
    trace_begin();
    if (rexp_in && g_map_path == 0) {
        static bool attr = false;
        if (!attr) {
            cudaFuncSetAttribute(oz::k_ozaki_map_pre<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            cudaFuncSetAttribute(oz::k_ozaki_map_pre<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            attr = true;
        }
        if (colexp_out || rexp_out)
            oz::k_ozaki_map_pre<true><<<grid, oz::MAP_NT, smem, stream()>>>(ma, status_ptr());
        else
            oz::k_ozaki_map_pre<false><<<grid, oz::MAP_NT, smem, stream()>>>(ma, status_ptr());
    } else {
        oz::k_ozaki_map<<<grid, oz::MAP_NT, smem, stream()>>>(ma, status_ptr());
    }
    note_launch("ozaki_map");
    return 0;
}

}  // namespace lg

using namespace lg;

extern "C" {
long long lila_prim_ozaki_gram_work(void) { return ozaki_gram_work(sm_count()); }
int lila_prim_ozaki_gram(int m, int n, const double *A, int lda, double *G, int ldg, double *work, long long lwork)
{
    return ozaki_gram(m, n, A, lda, G, ldg, work, lwork);
}
int lila_prim_ozaki_map(int m, int n, const double *A, int lda, const double *X, int ldx, int nout, double *out, int ldo)
{
    return ozaki_map(m, n, A, lda, X, ldx, nout, out, ldo);
}
// Kernel choice of the tall Gram and row map (see g_map_path); returns the
// previous setting.
int lila_prim_ozaki_map_path(int path)
{
    const int prev = g_map_path;
    if (path >= 0 && path <= 3) g_map_path = path;
    return prev;
}
// Diagnostic form: rows handled per CTA forced to rows_per (rounded up to 64).
int lila_prim_ozaki_gram_rows(int m, int n, const double *A, int lda, double *G, int ldg, double *work,
                              long long lwork, int rows_per)
{
    return ozaki_gram(m, n, A, lda, G, ldg, work, lwork, rows_per);
}
}
