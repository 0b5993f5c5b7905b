// lg_ozstream.cu -- TMA-fed, warp-specialised split-precision kernels of the
// tall-skinny leaf: the row map out = A X (A m x n, X n x nout, n, nout <= 64)
// and the Gram G = A^T A (further below), FP64-grade.
//
// The digit scheme is that of lg_ozaki.cu (eight balanced base-128 digits per
// value, row scales for A, column scales for X, digit orders d = s + t <= 7
// accumulated in separate FP32 TMEM blocks, exact).
//
// Row map, transposed tiles.  One tcgen05.mma computes D = Xop * Bop^T with
//   Xop (M = 128 rows, K = 16): digit slices t and t + 1 of X^T stacked,
//       rows 0..63 = X_t(:, j)^T, rows 64..127 = X_{t+1}(:, j)^T (j = output
//       column), for t = 0, 2, 4, 6 (four stacked pairs, resident in shared
//       memory for the whole launch);
//   Bop (N rows, K = 16): the digit slices s = 0 .. 7 - t of a tile of 32
//       rows of A, row s * 32 + r = digit s of row r.
// So TMEM lane j (< 64) column s * 32 + r holds order t + s of out(r, j) and
// lane 64 + j the order t + 1 + s; with the MMA's D placed t * 32 columns
// into the tile's TMEM block, block d (32 columns) of lane j accumulates the
// even-t part of order d, block d of lane 64 + j the odd-t part of order
// d + 1.  A tile takes 8 x 32 = 256 TMEM columns, so two tiles alternate in
// the 512 columns: the epilogue drains tile i while the tensor core works on
// tile i + 1.  Per 16-column K chunk of a tile: 4 MMAs, N = (8 - t) 32.
//
// Roles of one persistent CTA per SM (448 threads):
//   producer (warp 12, one lane): 2-D TMA loads of the raw FP64 tile
//       (32 rows x 64 columns, 16 KB) into a ring of three slots;
//   splitters (warps 8..11, lane = row): warp w reads columns 16 w .. + 16 of
//       the tile, the four warps agree on each row's scale (largest exponent),
//       warp w writes the digit chunk w (8 slices x 32 rows x K16, canonical
//       K-major layout) into a ring of six chunk slots;
//   MMA issuer (warp 13, one lane): 4 MMAs per chunk, one commit per chunk
//       that frees its slot, one per tile that hands the TMEM block to the
//       epilogue;
//   epilogue (warps 0..7, warp % 4 = TMEM lane quarter, warp / 4 = row half):
//       the odd-t warps fold their orders into two int64 words per output
//       and hand them over shared memory to the even-t warps, which add
//       their own, round to FP64 and write the tile into a staging buffer;
//       all eight then store it column by column (32 rows = 256 contiguous
//       bytes per warp store).
// Every hand-off is an mbarrier with a bounded wait; a wait that gives up
// sets ST_WAIT_TIMEOUT and an abort flag that ends every role, and the CTA
// waits for its own MMAs and TMA loads before it frees TMEM and exits.
// Each tile's rows are read (TMA) before they are written (epilogue) by the
// same CTA, so out may be A itself.
#include <cuda.h>
#include <math.h>

#include "lg_common.cuh"
#include "lg_tc.cuh"
#include "lg_ozdigits.cuh"

namespace lg {
namespace ozs {

using namespace oz;

constexpr int TR = 32;                                 // rows of A per tile
constexpr int TR_NRAW = 3;                             // raw tile slots
constexpr int TR_NDIG = 6;                             // digit chunk slots
constexpr uint32_t TR_RAW_BYTES = TR * 64 * 8;         // one TMA box: 32 rows x 64 columns, column-major
constexpr uint32_t TR_CH_SBO = 256;                    // 8-row groups of a chunk (2 core matrices along K)
constexpr uint32_t TR_CH_SLICE = (TR / 8) * TR_CH_SBO;  // one digit slice of a chunk: 32 rows x K16
constexpr uint32_t TR_CH_BYTES = NS * TR_CH_SLICE;     // 8 KB
constexpr uint32_t TR_X_SBO = 1024;                    // 8-row groups of a stacked pair (8 core matrices along K)
constexpr uint32_t TR_XP_BYTES = 16 * TR_X_SBO;        // one stacked pair: 128 rows x K64
constexpr uint32_t TR_OFF_RAW = 4 * TR_XP_BYTES;
constexpr uint32_t TR_OFF_DIG = TR_OFF_RAW + TR_NRAW * TR_RAW_BYTES;
constexpr uint32_t TR_OFF_XCH = TR_OFF_DIG + TR_NDIG * TR_CH_BYTES;
constexpr uint32_t TR_XCH_BYTES = 4 * 2 * 2 * 4 * 32 * 16;  // (warp pair, row group, side, row, lane) x (hi, lo)
constexpr uint32_t TR_OFF_STG = TR_OFF_XCH + TR_XCH_BYTES;
constexpr int TR_STG_LD = 34;                          // doubles per staged column (32 rows + pad)
constexpr uint32_t TR_STG_BYTES = 64 * TR_STG_LD * 8;
constexpr uint32_t TR_SMEM = TR_OFF_STG + TR_STG_BYTES;  // 214,016
constexpr int TR_EPI = 8;                              // warps 0..7
constexpr int TR_W_SPLIT = 8;                          // warps 8..11
constexpr int TR_W_PROD = 12;
constexpr int TR_W_MMA = 13;
constexpr int TR_THREADS = 14 * 32;

struct MapTmaArgs {
    int m, n;
    const double *X;
    int ldx, nout;
    double *out;
    int ldo;
    int *colexp_out;  // column scales of out (64 ints, zeroed), or null
    const int *pred;  // the launch does nothing when *pred == 0 (null: always runs)
};

__device__ __forceinline__ unsigned long long dbits(double v) { return (unsigned long long)__double_as_longlong(v); }

// kIntAsm: the epilogue's int64 -> double rounding by integer instructions
// (assemble_int) instead of the FP64-pipe conversion (assemble_fast); the
// two give identical bits.
template <bool kIntAsm>
__global__ void __launch_bounds__(TR_THREADS, 1)
    k_map_tma(const __grid_constant__ CUtensorMap tmA, const MapTmaArgs a, int *status)
{
    if (a.pred && !*a.pred) return;
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t raw_full[TR_NRAW], raw_empty[TR_NRAW], dig_full[TR_NDIG], dig_empty[TR_NDIG],
        tm_full[2], tm_empty[2], pm_full[2], rx_full[4], rx_empty[4], x_full[4][2][2], x_empty[4][2][2], stg_full,
        stg_empty, drain;
    __shared__ uint32_t tmem_base_s;
    __shared__ int s_abort_v;
    __shared__ int s_xexp[64];
    __shared__ int s_rexp[4][TR];      // row scales of the tiles in flight
    __shared__ int s_pmax[2][4][TR];   // the splitter warps' partial row maxima
    volatile int *s_abort = &s_abort_v;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m = a.m, n = a.n, nout = a.nout;
    const uint32_t sbase = tc::smem_u32(smem);
    if (sbase & 1023) {
        // the operand layouts assume a 1024-byte aligned base
        if (tid == 0) atomicOr(status, ST_LAUNCH_ERROR);
        return;
    }
    if (tid == 0) {
        for (int k = 0; k < TR_NRAW; k++) {
            tc::mbar_init(&raw_full[k], 1);
            tc::mbar_init(&raw_empty[k], 4);
        }
        for (int k = 0; k < TR_NDIG; k++) {
            tc::mbar_init(&dig_full[k], 1);
            tc::mbar_init(&dig_empty[k], 1);
        }
        for (int k = 0; k < 2; k++) {
            tc::mbar_init(&tm_full[k], 1);
            tc::mbar_init(&tm_empty[k], TR_EPI);
            tc::mbar_init(&pm_full[k], 4);
        }
        for (int k = 0; k < 4; k++) {
            tc::mbar_init(&rx_full[k], 1);
            tc::mbar_init(&rx_empty[k], TR_EPI);
            for (int g = 0; g < 2; g++)
                for (int d = 0; d < 2; d++) {
                    tc::mbar_init(&x_full[k][g][d], 1);
                    tc::mbar_init(&x_empty[k][g][d], 1);
                }
        }
        tc::mbar_init(&stg_full, TR_EPI);
        tc::mbar_init(&stg_empty, TR_EPI);
        tc::mbar_init(&drain, 1);
        tc::fence_mbar_init();
        s_abort_v = 0;
    }
    if (warp == TR_W_MMA) {
        tc::tmem_alloc(&tmem_base_s, 512);
        tc::tmem_relinquish();
    }
    if (warp == TR_W_PROD && lane == 0) tc::prefetch_tmap(&tmA);
    // X column scales, then the four stacked digit pairs (512 units: output
    // column j, 8-row group kg of X)
    if (tid < 64) {
        int mx = 0;
        if (tid < nout)
            for (int k = 0; k < n; k++) mx = max(mx, bexp(dbits(a.X[(size_t)k + (size_t)tid * a.ldx])));
        s_xexp[tid] = mx;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = tmem_base_s;
    for (int u = tid; u < 512; u += TR_THREADS) {
        const int j = u >> 3, kg = u & 7;
        long long Xv[8];
#pragma unroll
        for (int e = 0; e < 8; e++) {
            const int k = kg * 8 + e;
            const unsigned long long b = (j < nout && k < n) ? dbits(a.X[(size_t)k + (size_t)j * a.ldx]) : 0ull;
            Xv[e] = fixed56(b, s_xexp[j]);
        }
        uint32_t w0[NS], w1[NS], w2[NS], w3[NS];
        digit_pair(Xv[0], Xv[1], w0);
        digit_pair(Xv[2], Xv[3], w1);
        digit_pair(Xv[4], Xv[5], w2);
        digit_pair(Xv[6], Xv[7], w3);
#pragma unroll
        for (int t = 0; t < NS; t++) {
            const int mrow = 64 * (t & 1) + j;
            *(uint4 *)(smem + (t >> 1) * TR_XP_BYTES + (mrow >> 3) * TR_X_SBO + kg * LBO + (mrow & 7) * 16) =
                make_uint4(w0[t], w1[t], w2[t], w3[t]);
        }
    }
    tc::fence_proxy_async_smem();
    __syncthreads();

    const int ntiles = (m + TR - 1) / TR;
    if (warp == TR_W_PROD) {
        // ---- producer: raw tiles by TMA ------------------------------------
        if (lane == 0) {
            int it = 0;
            for (int t = blockIdx.x; t < ntiles; t += gridDim.x, it++) {
                const int slot = it % TR_NRAW;
                if (it >= TR_NRAW &&
                    !tc::wait_abort(&raw_empty[slot], ((it / TR_NRAW) - 1) & 1, s_abort, status, ST_WAIT_TIMEOUT))
                    break;
                tc::mbar_arrive_expect_tx(&raw_full[slot], TR_RAW_BYTES);
                tc::tma_load_2d(sbase + TR_OFF_RAW + slot * TR_RAW_BYTES, &tmA, t * TR, 0, &raw_full[slot]);
            }
            // the loads still in flight land before the CTA may exit
            for (int k = it > TR_NRAW ? it - TR_NRAW : 0; k < it; k++)
                tc::mbar_wait(&raw_full[k % TR_NRAW], (k / TR_NRAW) & 1);
        }
    } else if (warp == TR_W_MMA) {
        // ---- MMA issuer ------------------------------------------------------
        if (lane == 0) {
            bool ok = true;
            int it = 0;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, it++) {
                const int b = it & 1;
                if (it >= 2 && !tc::wait_abort(&tm_empty[b], ((it >> 1) - 1) & 1, s_abort, status, ST_WAIT_TIMEOUT))
                    break;
                tc::fence_after_sync();
                for (int c = 0; c < 4; c++) {
                    const int g = 4 * it + c, ds = g % TR_NDIG;
                    if (!tc::wait_abort(&dig_full[ds], (g / TR_NDIG) & 1, s_abort, status, ST_WAIT_TIMEOUT)) {
                        ok = false;
                        break;
                    }
                    tc::fence_after_sync();
                    const uint64_t bd = tc::desc_nosw(sbase + TR_OFF_DIG + ds * TR_CH_BYTES, LBO, TR_CH_SBO);
#pragma unroll
                    for (int p = 0; p < 4; p++) {
                        const uint64_t ad =
                            tc::desc_nosw(sbase + p * TR_XP_BYTES + c * 2 * LBO, LBO, TR_X_SBO);
                        tc::mma_bf16(tbase + b * 256 + 64 * p, ad, bd, tc::idesc_bf16_f32(128, (8 - 2 * p) * TR),
                                     (c > 0 || p > 0) ? 1u : 0u);
                    }
                    tc::mma_commit(&dig_empty[ds]);
                }
                if (ok) tc::mma_commit(&tm_full[b]);
            }
            // every MMA issued by this thread is complete before TMEM is freed
            tc::mma_commit(&drain);
            tc::mbar_wait(&drain, 0);
        }
    } else if (warp >= TR_W_SPLIT) {
        // ---- splitters: warp w = K chunk w, lane = row of the tile ----------
        const int w = warp - TR_W_SPLIT, r = lane;
        int it = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, it++) {
            const int slot = it % TR_NRAW;
            const int g = 4 * it + w, ds = g % TR_NDIG;
            if (g >= TR_NDIG &&
                !tc::wait_abort_warp(&dig_empty[ds], ((g / TR_NDIG) - 1) & 1, s_abort, status, ST_WAIT_TIMEOUT))
                break;
            if (!tc::wait_abort_warp(&raw_full[slot], (it / TR_NRAW) & 1, s_abort, status, ST_WAIT_TIMEOUT)) break;
            const double *raw = (const double *)(smem + TR_OFF_RAW + slot * TR_RAW_BYTES);
            unsigned long long v[16];
            int mx = 0;
#pragma unroll
            for (int e = 0; e < 16; e++) {
                v[e] = dbits(raw[(16 * w + e) * TR + r]);
                mx = max(mx, bexp(v[e]));
            }
            s_pmax[it & 1][w][r] = mx;
            __syncwarp();
            if (lane == 0) {
                tc::mbar_arrive(&raw_empty[slot]);
                tc::mbar_arrive(&pm_full[it & 1]);
            }
            if (!tc::wait_abort_warp(&pm_full[it & 1], (it >> 1) & 1, s_abort, status, ST_WAIT_TIMEOUT)) break;
            const int rmax =
                max(max(s_pmax[it & 1][0][r], s_pmax[it & 1][1][r]), max(s_pmax[it & 1][2][r], s_pmax[it & 1][3][r]));
            if (w == 0) {
                // the row scales of this tile, for the epilogue
                if (it >= 4 &&
                    !tc::wait_abort_warp(&rx_empty[it & 3], ((it >> 2) - 1) & 1, s_abort, status, ST_WAIT_TIMEOUT))
                    break;
                s_rexp[it & 3][r] = rmax;
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(&rx_full[it & 3]);
            }
            uint8_t *dst = smem + TR_OFF_DIG + ds * TR_CH_BYTES + (r >> 3) * TR_CH_SBO + (r & 7) * 16;
#pragma unroll
            for (int h = 0; h < 2; h++) {
                long long Xv[8];
#pragma unroll
                for (int e = 0; e < 8; e++) Xv[e] = fixed56(v[8 * h + e], rmax);
                uint32_t w0[NS], w1[NS], w2[NS], w3[NS];
                digit_pair(Xv[0], Xv[1], w0);
                digit_pair(Xv[2], Xv[3], w1);
                digit_pair(Xv[4], Xv[5], w2);
                digit_pair(Xv[6], Xv[7], w3);
#pragma unroll
                for (int s = 0; s < NS; s++)
                    *(uint4 *)(dst + s * TR_CH_SLICE + h * LBO) = make_uint4(w0[s], w1[s], w2[s], w3[s]);
            }
            tc::fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&dig_full[ds]);
        }
    } else {
        // ---- epilogue: warps 0..7 --------------------------------------------
        const int q = warp & 3, rh = warp >> 2;
        const bool top = q < 2;                  // even-t lanes (orders d in block d)
        const int j = 32 * (q & 1) + lane;       // output column of this lane
        const int pr = (q & 1) + 2 * rh;         // the even / odd warp pair
        const int fx = s_xexp[j];
        double *stg = (double *)(smem + TR_OFF_STG);
        int cmax[8];
#pragma unroll
        for (int c = 0; c < 8; c++) cmax[c] = 0;
        int it = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, it++) {
            const int b = it & 1;
            if (!tc::wait_abort_warp(&rx_full[it & 3], (it >> 2) & 1, s_abort, status, ST_WAIT_TIMEOUT)) break;
            if (!tc::wait_abort_warp(&tm_full[b], (it >> 1) & 1, s_abort, status, ST_WAIT_TIMEOUT)) break;
            tc::fence_after_sync();
            bool ok = true;
#pragma unroll 1
            for (int grp = 0; grp < 2 && ok; grp++) {
                const int r0 = 16 * rh + 8 * grp;
                long long hi[8], lo[8];
                {
                    uint32_t v[8][8];
#pragma unroll
                    for (int d = 0; d < 8; d++)
                        tc::tmem_ld8(tbase + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * 256 + d * TR + r0), v[d]);
                    tc::tmem_ld_wait();
                    if (grp == 1) {
                        // every TMEM read of this tile is done: its block may take tile it + 2
                        tc::fence_before_sync();
                        __syncwarp();
                        if (lane == 0) tc::mbar_arrive(&tm_empty[b]);
                    }
#pragma unroll
                    for (int i = 0; i < 8; i++) {
                        if (top) {
                            hi[i] = combine4(v[0][i], v[1][i], v[2][i], v[3][i]);
                            lo[i] = combine4(v[4][i], v[5][i], v[6][i], v[7][i]);
                        } else {
                            // block d holds order d + 1; block 7 (order 8) is not needed
                            hi[i] = combine4(0u, v[0][i], v[1][i], v[2][i]);
                            lo[i] = combine4(v[3][i], v[4][i], v[5][i], v[6][i]);
                        }
                    }
                }
                // each side hands the other the partial sums of half the rows
                // and rounds the other half: the even-t warp rows 0..3 of the
                // group, the odd-t warp rows 4..7
                const int side = top ? 0 : 1;
                longlong2 *xo = (longlong2 *)(smem + TR_OFF_XCH) + (size_t)(((pr * 2 + grp) * 2 + side) * 4) * 32 + lane;
                const longlong2 *xi =
                    (const longlong2 *)(smem + TR_OFF_XCH) + (size_t)(((pr * 2 + grp) * 2 + (1 - side)) * 4) * 32 + lane;
                if (it >= 1 &&
                    !tc::wait_abort_warp(&x_empty[pr][grp][side], (it - 1) & 1, s_abort, status, ST_WAIT_TIMEOUT)) {
                    ok = false;
                    break;
                }
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const int ro = top ? 4 + i : i;  // the rows the other side rounds
                    xo[i * 32] = make_longlong2(hi[ro], lo[ro]);
                }
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(&x_full[pr][grp][side]);
                if (!tc::wait_abort_warp(&x_full[pr][grp][1 - side], it & 1, s_abort, status, ST_WAIT_TIMEOUT)) {
                    ok = false;
                    break;
                }
                long long h4[4], l4[4];
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const int rm = top ? i : 4 + i;  // the rows this side rounds
                    const longlong2 o = xi[i * 32];
                    h4[i] = hi[rm] + o.x;
                    l4[i] = lo[rm] + o.y;
                }
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(&x_empty[pr][grp][1 - side]);
                if (grp == 0 && it >= 1 &&
                    !tc::wait_abort_warp(&stg_empty, (it - 1) & 1, s_abort, status, ST_WAIT_TIMEOUT)) {
                    ok = false;
                    break;
                }
                const int rb = r0 + (top ? 0 : 4);
                double val[4];
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const int e = s_rexp[it & 3][rb + i];
                    const int sc = (e - 1022) + (fx - 1022) - 63;
                    val[i] = (e && fx) ? (kIntAsm ? assemble_int(h4[i], l4[i], sc) : assemble_fast(h4[i], l4[i], sc))
                                       : 0.0;
                }
                double2 *sp = (double2 *)(stg + j * TR_STG_LD + rb);
                sp[0] = make_double2(val[0], val[1]);
                sp[1] = make_double2(val[2], val[3]);
            }
            if (!ok) break;
            // this tile's row scales have been read, its staged values written
            __syncwarp();
            if (lane == 0) {
                tc::mbar_arrive(&rx_empty[it & 3]);
                tc::mbar_arrive(&stg_full);
            }
            // store: warp e writes columns 8 e .. 8 e + 7, lane = row
            if (!tc::wait_abort_warp(&stg_full, it & 1, s_abort, status, ST_WAIT_TIMEOUT)) break;
            const int row = t * TR + lane;
#pragma unroll
            for (int c = 0; c < 8; c++) {
                const int jj = 8 * warp + c;
                const double v = stg[jj * TR_STG_LD + lane];
                if (row < m && jj < nout) {
                    a.out[(size_t)row + (size_t)jj * a.ldo] = v;
                    cmax[c] = max(cmax[c], bexp(dbits(v)));
                }
            }
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&stg_empty);
        }
        if (a.colexp_out) {
#pragma unroll
            for (int c = 0; c < 8; c++) {
                const int e = __reduce_max_sync(0xffffffffu, cmax[c]);
                const int jj = 8 * warp + c;
                if (lane == 0 && jj < nout && e) {
                    if (e == 0x7FF) atomicOr(status, ST_NONFINITE);
                    atomicMax(&a.colexp_out[jj], e);
                }
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == TR_W_MMA) tc::tmem_dealloc(tbase, 512);
}

// ---------------------------------------------------------------------------
// Gram G = A^T A (n <= 64) per CTA over a contiguous row range, TMA-fed.
//   The digit arithmetic, the MMA schedule (per 16-row K step 6 MMAs with
//   M = 128 covering digit slices s, s + 1), the flush of the FP32 order
//   blocks into int64 every 128 rows and the integer partials are those of
//   k_ozaki_gram (lg_ozaki.cu).  The raw rows come by TMA instead of
//   per-thread global loads: a producer lane keeps a ring of three 64-row
//   stages in flight (four 2-D boxes of 16 rows x 64 columns per stage,
//   128-byte swizzled so that the splitters' 16-byte reads of 8 rows of one
//   column are conflict-free), and the splitters read them from shared
//   memory without a transposition scratch.
// ---------------------------------------------------------------------------
constexpr int GT_KC = 64;                              // rows per stage
constexpr int GT_RAW = 3;                              // raw stage slots
constexpr int GT_DIG = 2;                              // digit stage slots
// stages per flush window: 128 rows.  A tensor-memory block sums per row at
// most 6 * 2^12 in magnitude (order 6 of the even slices: d_0 d_6 + d_2 d_4
// + d_4 d_2 + d_6 d_0, |d_0| <= 128, |d_s| <= 64), so 128 rows stay below
// 2^22 (3,145,728), the bound of the exact FP32 -> integer step of the fold
// (combine4); 192 rows could exceed it
constexpr int GT_FLUSH = 2;
constexpr uint32_t GT_BOX_BYTES = 16 * 64 * 8;         // one box: 16 rows x 64 columns
constexpr uint32_t GT_RAW_BYTES = 4 * GT_BOX_BYTES;    // 32768
constexpr uint32_t GT_SBO = (GT_KC / 8) * 128;         // 1024
constexpr uint32_t GT_SLICE = 8 * GT_SBO;              // 64 columns x 64 rows of one digit plane
constexpr uint32_t GT_DIG_BYTES = NS * GT_SLICE;       // 65536
constexpr uint32_t GT_OFF_RAW = GT_DIG * GT_DIG_BYTES;
constexpr uint32_t GT_SMEM = GT_OFF_RAW + GT_RAW * GT_RAW_BYTES;  // 229,376
constexpr int GT_NT = 512;
constexpr int GT_PRODUCER = 32 * 14;                   // lane 0 of warp 14 issues the TMA loads

struct GramTmaArgs {
    int m, n, rows_per;
    const int *colexp;
    long long *partial;
    const int *pred;  // the launch does nothing when *pred == 0 (null: always runs)
};

__global__ void __launch_bounds__(GT_NT, 1)
    k_gram_tma(const __grid_constant__ CUtensorMap tmA, const GramTmaArgs g, int *status)
{
    if (g.pred && !*g.pred) return;
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t empty_b[GT_DIG], full_b[GT_DIG], raw_full[GT_RAW], raw_empty[GT_RAW], tfree;
    __shared__ uint32_t tmem_base_s;
    __shared__ int s_abort_v;
    __shared__ int s_exp[64];
    volatile int *s_abort = &s_abort_v;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t sbase = tc::smem_u32(smem);
    if (sbase & 1023) {
        // the swizzled TMA boxes need a 1024-byte aligned base
        if (tid == 0) atomicOr(status, ST_LAUNCH_ERROR);
        return;
    }
    if (tid == 0) {
        for (int b = 0; b < GT_DIG; b++) {
            tc::mbar_init(&empty_b[b], 1);
            tc::mbar_init(&full_b[b], GT_NT / 32);
        }
        for (int b = 0; b < GT_RAW; b++) {
            tc::mbar_init(&raw_full[b], 1);
            tc::mbar_init(&raw_empty[b], GT_NT / 32);
        }
        tc::mbar_init(&tfree, GT_NT / 32);
        tc::fence_mbar_init();
        s_abort_v = 0;
    }
    if (warp == 0) {
        tc::tmem_alloc(&tmem_base_s, 512);
        tc::tmem_relinquish();
    }
    if (tid == GT_PRODUCER) tc::prefetch_tmap(&tmA);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = tmem_base_s;
    const int q = warp & 3, h = warp >> 2;
    const int L = 32 * q + lane;
    const bool top = L < 64;
    const int n = g.n;
    const int r_beg = blockIdx.x * g.rows_per;
    const int r_end = min(g.m, r_beg + g.rows_per);
    long long *partial = g.partial + (size_t)blockIdx.x * 8192;
    const int nstage = r_end > r_beg ? (r_end - r_beg + GT_KC - 1) / GT_KC : 0;
    if (tid < 64) s_exp[tid] = tid < n ? g.colexp[tid] : 0;
    long long acc_hi[16], acc_lo[16];
#pragma unroll
    for (int j = 0; j < 16; j++) {
        acc_hi[j] = 0;
        acc_lo[j] = 0;
    }
    __syncthreads();
    // this thread's unit: column uc, 8-row group uk; a warp takes 8
    // consecutive columns x 4 row groups (its 16-byte digit stores fill whole
    // 128-byte lines, and its swizzled raw reads hit distinct banks)
    const int uc = ((tid >> 6) << 3) | (tid & 7), uk = (tid >> 3) & 7;
    const int emax = s_exp[uc];
    const bool producer = tid == GT_PRODUCER;
    const bool issuer = warp == GT_NT / 32 - 1 && lane == 0;
    int issued = 0;
    auto issue_raw = [&](int st2) {
        const uint32_t slot = st2 % GT_RAW;
        tc::mbar_arrive_expect_tx(&raw_full[slot], GT_RAW_BYTES);
#pragma unroll
        for (int b = 0; b < 4; b++)
            tc::tma_load_2d(sbase + GT_OFF_RAW + slot * GT_RAW_BYTES + b * GT_BOX_BYTES, &tmA,
                            r_beg + st2 * GT_KC + 16 * b, 0, &raw_full[slot]);
        issued = st2 + 1;
    };
    if (producer)
        for (int s2 = 0; s2 < GT_RAW && s2 < nstage; s2++) issue_raw(s2);
    int last_commit = -1;
    // Stage s: its raw rows (TMA slot s % 3) split into digit buffer s % 2.
    // Split-ahead schedule: stage st + 1 is split while the tensor core runs
    // stage st, then the window ending with stage st is folded (which waits
    // for stage st's MMAs) and stage st + 1 is issued.
    auto split_stage = [&](int s2) -> bool {
        const int buf = s2 % GT_DIG;
        const uint32_t rs = s2 % GT_RAW;
        // digit buffer buf's previous stage (s2 - 2) has been read by the tensor core
        if (s2 >= GT_DIG &&
            !tc::wait_abort_warp(&empty_b[buf], ((s2 - GT_DIG) / GT_DIG) & 1, s_abort, status, ST_WAIT_TIMEOUT))
            return false;
        if (!tc::wait_abort_warp(&raw_full[rs], (s2 / GT_RAW) & 1, s_abort, status, ST_WAIT_TIMEOUT)) return false;
        unsigned long long uv[8];
        {
            const uint8_t *col = smem + GT_OFF_RAW + rs * GT_RAW_BYTES + (uk >> 1) * GT_BOX_BYTES + uc * 128;
            const int row0 = r_beg + s2 * GT_KC + 8 * uk;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int chunk = 4 * (uk & 1) + i;  // two rows per 16-byte chunk, 128-byte swizzle
                const uint4 d = *(const uint4 *)(col + ((chunk ^ (uc & 7)) << 4));
                uv[2 * i] = row0 + 2 * i < r_end ? ((unsigned long long)d.y << 32 | d.x) : 0ull;
                uv[2 * i + 1] = row0 + 2 * i + 1 < r_end ? ((unsigned long long)d.w << 32 | d.z) : 0ull;
            }
        }
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&raw_empty[rs]);
        uint8_t *stage = smem + (size_t)buf * GT_DIG_BYTES;
#pragma unroll
        for (int hf = 0; hf < 2; hf++) {
            uint32_t w01[NS], w23[NS];
            digit_pair(fixed56(uv[4 * hf], emax), fixed56(uv[4 * hf + 1], emax), w01);
            digit_pair(fixed56(uv[4 * hf + 2], emax), fixed56(uv[4 * hf + 3], emax), w23);
#pragma unroll
            for (int s = 0; s < NS; s++)
                *(uint2 *)(stage + s * GT_SLICE + (uc >> 3) * GT_SBO + uk * LBO + (uc & 7) * 16 + hf * 8) =
                    make_uint2(w01[s], w23[s]);
        }
        tc::fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&full_b[buf]);
        return true;
    };
    // the issuer's MMAs of stage s2 (a window's first stage waits for the
    // previous window's fold)
    auto issue_stage = [&](int s2) {
        const int buf = s2 % GT_DIG;
        const bool window_start = (s2 % GT_FLUSH) == 0;
        bool ok = tc::wait_abort(&full_b[buf], (s2 / GT_DIG) & 1, s_abort, status, ST_WAIT_TIMEOUT);
        if (ok && window_start && s2 > 0)
            ok = tc::wait_abort(&tfree, ((s2 / GT_FLUSH) - 1) & 1, s_abort, status, ST_WAIT_TIMEOUT);
        if (!ok) return;
        tc::fence_after_sync();
        const uint32_t sb = sbase + buf * GT_DIG_BYTES;
#pragma unroll
        for (int ks = 0; ks < GT_KC / 16; ks++) {
            const uint32_t koff = ks * 2 * LBO;
#pragma unroll
            for (int s = 0; s < NS; s += 2) {
                const int ntot = 64 * (NS - s);
                const uint64_t ad = tc::desc_nosw(sb + s * GT_SLICE + koff, LBO, GT_SBO);
                const uint32_t acc = (window_start && ks == 0 && s == 0) ? 0u : 1u;
                const int n1 = ntot < 256 ? ntot : 256;
                tc::mma_bf16(tbase + 64 * s, ad, tc::desc_nosw(sb + koff, LBO, GT_SBO), tc::idesc_bf16_f32(128, n1),
                             acc);
                if (ntot > 256)
                    tc::mma_bf16(tbase + 64 * s + 256, ad, tc::desc_nosw(sb + 4 * GT_SLICE + koff, LBO, GT_SBO),
                                 tc::idesc_bf16_f32(128, ntot - 256), acc);
            }
        }
        tc::mma_commit(&empty_b[buf]);
        last_commit = s2;
    };
    if (nstage > 0 && split_stage(0) && issuer) issue_stage(0);
    for (int st = 0; st < nstage; st++) {
        // stage st's raw slot is refilled with stage st + 3 once every warp has read it
        if (producer && st + GT_RAW < nstage) {
            if (tc::wait_abort(&raw_empty[st % GT_RAW], (st / GT_RAW) & 1, s_abort, status, ST_WAIT_TIMEOUT))
                issue_raw(st + GT_RAW);
        }
        if (__any_sync(0xffffffffu, *s_abort)) break;
        if (st + 1 < nstage && !split_stage(st + 1)) break;
        const bool flush = ((st + 1) % GT_FLUSH) == 0 || st == nstage - 1;
        if (flush) {
            // stage st's commit also covers every earlier MMA (in-order issue)
            const int buf = st % GT_DIG;
            if (!tc::wait_abort_warp(&empty_b[buf], (st / GT_DIG) & 1, s_abort, status, ST_WAIT_TIMEOUT)) break;
            tc::fence_after_sync();
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
        if (issuer && st + 1 < nstage) issue_stage(st + 1);
    }
    // after an abort the issuer's last MMAs may still run, and the producer's
    // last loads may still land: wait (bounded) for both before TMEM and the
    // shared memory are released
    if (last_commit >= 0) tc::mbar_wait(&empty_b[last_commit % GT_DIG], (last_commit / GT_DIG) & 1);
    if (producer)
        for (int k = issued > GT_RAW ? issued - GT_RAW : 0; k < issued; k++)
            tc::mbar_wait(&raw_full[k % GT_RAW], (k / GT_RAW) & 1);
    __syncthreads();
    if (!*s_abort) {
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

}  // namespace ozs

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn()
{
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
        else
            cudaGetLastError();
    }
    return fn;
}

// A 2-D tensor map of the column-major m x n FP64 matrix A (lda) with boxes of
// `box_rows` rows x `box_cols` columns (128-byte swizzled when swz128);
// false when A's address or lda does not meet TMA's 16-byte rules.
bool tma_map_2d(CUtensorMap *tm, const double *A, int lda, int m, int n, int box_rows, int box_cols,
                bool swz128 = false)
{
    if (((uintptr_t)A & 15) || (lda & 1) || m < 1 || n < 1) return false;
    EncodeTiledFn enc = encode_fn();
    if (!enc) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)m, (cuuint64_t)n};
    const cuuint64_t strides[1] = {(cuuint64_t)lda * 8};
    const cuuint32_t box[2] = {(cuuint32_t)box_rows, (cuuint32_t)box_cols};
    const cuuint32_t es[2] = {1, 1};
    return enc(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, (void *)A, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               swz128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// out = A X by the TMA-fed kernel; false (nothing enqueued) when A does not
// meet TMA's alignment rules, so the caller takes the register-fed kernel.
bool ozaki_map_tma(int m, int n, const double *A, int lda, const double *X, int ldx, int nout, double *out, int ldo,
                   int *colexp_out, bool int_asm, const int *pred)
{
    CUtensorMap tm;
    if (!tma_map_2d(&tm, A, lda, m, n, ozs::TR, 64)) return false;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(ozs::k_map_tma<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ozs::TR_SMEM);
        cudaFuncSetAttribute(ozs::k_map_tma<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ozs::TR_SMEM);
        attr = true;
    }
    const int tiles = (m + ozs::TR - 1) / ozs::TR;
    const int grid = tiles < sm_count() ? tiles : sm_count();
    ozs::MapTmaArgs args{m, n, X, ldx, nout, out, ldo, colexp_out, pred};
    trace_begin();
    if (int_asm)
        ozs::k_map_tma<true><<<grid, ozs::TR_THREADS, ozs::TR_SMEM, stream()>>>(tm, args, status_ptr());
    else
        ozs::k_map_tma<false><<<grid, ozs::TR_THREADS, ozs::TR_SMEM, stream()>>>(tm, args, status_ptr());
    note_launch("ozaki_map");
    return true;
}

// The CTA grid's integer Gram partials of A (rows_per rows per CTA, a
// multiple of 64) by the TMA-fed kernel; false (nothing enqueued) when A does
// not meet TMA's alignment rules.
bool ozaki_gram_tma(int m, int n, const double *A, int lda, int rows_per, const int *colexp, long long *partial,
                    int parts, const int *pred)
{
    CUtensorMap tm;
    if (!tma_map_2d(&tm, A, lda, m, n, 16, 64, true)) return false;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(ozs::k_gram_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ozs::GT_SMEM);
        attr = true;
    }
    ozs::GramTmaArgs args{m, n, rows_per, colexp, partial, pred};
    trace_begin();
    ozs::k_gram_tma<<<parts, ozs::GT_NT, ozs::GT_SMEM, stream()>>>(tm, args, status_ptr());
    note_launch("ozaki_gram");
    return true;
}

}  // namespace lg
