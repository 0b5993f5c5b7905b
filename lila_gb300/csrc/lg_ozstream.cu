// lg_ozstream.cu -- the tall-skinny split-precision row map out = A X
// (A m x n, X n x nout, n, nout <= 64, FP64-grade) as a warp-specialised,
// TMA-fed persistent kernel.
//
// The digit scheme is that of lg_ozaki.cu (eight balanced base-128 digits per
// value, row scales for A, column scales for X, digit orders d = s + t <= 7
// accumulated in separate TMEM blocks).  What differs is the schedule: one
// CTA per SM walks its 128-row tiles with four roles running at once,
//
//   producer (1 thread):   2-D TMA loads (cp.async.bulk.tensor) of the raw
//                          FP64 tile, two half tiles of 128 rows x 32
//                          columns, into a ring of three shared-memory slots;
//   splitters (8 warps):   row scales of the tile, then per K chunk of 16
//                          columns the BF16 digit planes into a ring of two
//                          chunk slots (canonical K-major layout);
//   MMA issuer (1 thread): 12 tcgen05.mma per chunk into the 8 order blocks
//                          of TMEM (512 columns), one commit per chunk that
//                          frees its slot, one per tile that hands TMEM to
//                          the epilogue;
//   epilogue (8 warps):    TMEM -> FP64 assembly -> coalesced stores, while
//                          the splitters already work on the next tile.
//
// The hand-offs are mbarriers: raw_full (TMA bytes), raw_empty (splitters),
// dig_full (splitters), dig_empty (MMA commit), tm_full (MMA commit),
// tm_empty (epilogue).  Every wait is bounded; one that gives up sets
// ST_WAIT_TIMEOUT and an abort flag that ends every role, and the CTA waits
// for its own MMAs and TMA loads before it frees TMEM and exits.
//
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

constexpr int RAW_SLOTS = 3;
constexpr int DIG_SLOTS = 2;
constexpr uint32_t RAW_BYTES = 128 * 32 * 8;   // half tile: 128 rows x 32 columns of FP64
constexpr uint32_t DIG_SBO = 256;              // 8-row groups of a K16 chunk (2 core matrices along K)
constexpr uint32_t DIG_SLICE = 16 * DIG_SBO;   // one digit plane of a chunk: 128 rows x 16 K BF16
constexpr uint32_t DIG_BYTES = NS * DIG_SLICE;
constexpr uint32_t X_SBO = 1024;               // 8-column groups of X's digits (8 core matrices along K)
constexpr uint32_t X_SLICE = 8 * X_SBO;        // one digit plane of X: 64 columns x 64 K
constexpr uint32_t X_BYTES = NS * X_SLICE;
constexpr uint32_t OFF_DIG = X_BYTES;
constexpr uint32_t OFF_RAW = OFF_DIG + DIG_SLOTS * DIG_BYTES;
constexpr uint32_t SMEM_BYTES = OFF_RAW + RAW_SLOTS * RAW_BYTES;  // 229,376

constexpr int N_EPI = 8;      // warps 0..7
constexpr int N_SPLIT = 8;    // warps 8..15
constexpr int W_PROD = 16;
constexpr int W_MMA = 17;
constexpr int THREADS = 18 * 32;

struct MapTmaArgs {
    int m, n;
    const double *X;
    int ldx, nout;
    double *out;
    int ldo;
    int *colexp_out;  // column scales of out (64 ints, zeroed), or null
};

__device__ __forceinline__ unsigned long long dbits(double v) { return (unsigned long long)__double_as_longlong(v); }

// kIntAsm: the epilogue's int64 -> double rounding by integer instructions
// (assemble_int) instead of the FP64-pipe conversion (assemble_fast); the
// two give identical bits.
template <bool kIntAsm>
__global__ void __launch_bounds__(THREADS, 1)
    k_map_tma(const __grid_constant__ CUtensorMap tmA, const MapTmaArgs a, int *status)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t raw_full[RAW_SLOTS], raw_empty[RAW_SLOTS], dig_full[DIG_SLOTS],
        dig_empty[DIG_SLOTS], tm_full, tm_empty, drain;
    __shared__ uint32_t tmem_base_s;
    __shared__ int s_abort_v;
    __shared__ int s_xexp[64];
    __shared__ int s_rexp[2][128];
    volatile int *s_abort = &s_abort_v;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m = a.m, n = a.n, nout = a.nout;
    if (tc::smem_u32(smem) & 1023) {
        // the TMA destinations and operand layouts assume a 1024-byte aligned base
        if (tid == 0) atomicOr(status, ST_LAUNCH_ERROR);
        return;
    }

    if (tid == 0) {
        for (int k = 0; k < RAW_SLOTS; k++) {
            tc::mbar_init(&raw_full[k], 1);
            tc::mbar_init(&raw_empty[k], N_SPLIT);
        }
        for (int k = 0; k < DIG_SLOTS; k++) {
            tc::mbar_init(&dig_full[k], N_SPLIT);
            tc::mbar_init(&dig_empty[k], 1);
        }
        tc::mbar_init(&tm_full, 1);
        tc::mbar_init(&tm_empty, N_EPI);
        tc::mbar_init(&drain, 1);
        tc::fence_mbar_init();
        s_abort_v = 0;
    }
    if (warp == W_MMA) {
        tc::tmem_alloc(&tmem_base_s, 512);
        tc::tmem_relinquish();
    }
    if (warp == W_PROD && lane == 0) tc::prefetch_tmap(&tmA);
    // X column scales, then X's digits (512 units: output column j, 8-row group kg)
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
    const uint32_t sbase = tc::smem_u32(smem);
    if (tid < 512) {
        const int j = tid >> 3, kg = tid & 7;
#pragma unroll
        for (int hf = 0; hf < 2; hf++) {
            long long Xv[4];
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int k = kg * 8 + 4 * hf + e;
                const unsigned long long b = (j < nout && k < n) ? dbits(a.X[(size_t)k + (size_t)j * a.ldx]) : 0ull;
                Xv[e] = fixed56(b, s_xexp[j]);
            }
            uint32_t w01[NS], w23[NS];
            digit_pair(Xv[0], Xv[1], w01);
            digit_pair(Xv[2], Xv[3], w23);
#pragma unroll
            for (int t = 0; t < NS; t++)
                *(uint2 *)(smem + t * X_SLICE + (j >> 3) * X_SBO + kg * LBO + (j & 7) * 16 + hf * 8) =
                    make_uint2(w01[t], w23[t]);
        }
    }
    tc::fence_proxy_async_smem();
    __syncthreads();

    const int ntiles = (m + 127) / 128;
    if (warp == W_PROD) {
        // ---- producer: raw half tiles by TMA ------------------------------
        if (lane == 0) {
            uint32_t cnt = 0;
            for (int t = blockIdx.x; t < ntiles && !*s_abort; t += gridDim.x) {
                for (int hh = 0; hh < 2; hh++, cnt++) {
                    const uint32_t slot = cnt % RAW_SLOTS;
                    if (cnt >= RAW_SLOTS &&
                        !tc::wait_abort(&raw_empty[slot], ((cnt / RAW_SLOTS) - 1) & 1, s_abort, status, ST_WAIT_TIMEOUT))
                        break;
                    tc::mbar_arrive_expect_tx(&raw_full[slot], RAW_BYTES);
                    tc::tma_load_2d(sbase + OFF_RAW + slot * RAW_BYTES, &tmA, t * 128, 32 * hh, &raw_full[slot]);
                }
            }
            // the loads still in flight land before the CTA may exit
            for (uint32_t k = cnt > RAW_SLOTS ? cnt - RAW_SLOTS : 0; k < cnt; k++)
                tc::mbar_wait(&raw_full[k % RAW_SLOTS], (k / RAW_SLOTS) & 1);
        }
    } else if (warp == W_MMA) {
        // ---- MMA issuer ------------------------------------------------------
        if (lane == 0) {
            uint32_t g = 0;
            int it = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, it++) {
                if (it > 0 && !tc::wait_abort(&tm_empty, (it - 1) & 1, s_abort, status, ST_WAIT_TIMEOUT)) break;
                tc::fence_after_sync();
                for (int c = 0; c < 4; c++, g++) {
                    const uint32_t ds = g % DIG_SLOTS;
                    if (!tc::wait_abort(&dig_full[ds], (g / DIG_SLOTS) & 1, s_abort, status, ST_WAIT_TIMEOUT)) {
                        ok = false;
                        break;
                    }
                    tc::fence_after_sync();
                    const uint32_t abase = sbase + OFF_DIG + ds * DIG_BYTES;
                    const uint32_t bbase = sbase + (uint32_t)c * 2 * LBO;  // chunk c's K range of X's digits
#pragma unroll
                    for (int s = 0; s < NS; s++) {
                        const int ntot = 64 * (NS - s);
                        const uint64_t ad = tc::desc_nosw(abase + s * DIG_SLICE, LBO, DIG_SBO);
                        const uint32_t acc = (c == 0 && s == 0) ? 0u : 1u;
                        const int n1 = ntot < 256 ? ntot : 256;
                        tc::mma_bf16(tbase + 64 * s, ad, tc::desc_nosw(bbase, LBO, X_SBO), tc::idesc_bf16_f32(128, n1),
                                     acc);
                        if (ntot > 256)
                            tc::mma_bf16(tbase + 64 * s + 256, ad, tc::desc_nosw(bbase + 4 * X_SLICE, LBO, X_SBO),
                                         tc::idesc_bf16_f32(128, ntot - 256), acc);
                    }
                    tc::mma_commit(&dig_empty[ds]);
                }
                if (ok) tc::mma_commit(&tm_full);
            }
            // every MMA issued by this thread is complete before TMEM is freed
            tc::mma_commit(&drain);
            tc::mbar_wait(&drain, 0);
        }
    } else if (warp >= N_EPI) {
        // ---- splitters: warps 8..15, thread = (row r, column half hh) -------
        const int st = tid - 32 * N_EPI;
        const int r = st >> 1, hh = st & 1;
        uint32_t rc = 0, g = 0;
        int it = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, it++, rc += 2) {
            const uint32_t sa = rc % RAW_SLOTS, sb = (rc + 1) % RAW_SLOTS;
            if (!tc::wait_abort_warp(&raw_full[sa], (rc / RAW_SLOTS) & 1, s_abort, status, ST_WAIT_TIMEOUT)) break;
            if (!tc::wait_abort_warp(&raw_full[sb], ((rc + 1) / RAW_SLOTS) & 1, s_abort, status, ST_WAIT_TIMEOUT))
                break;
            const double *ra = (const double *)(smem + OFF_RAW + sa * RAW_BYTES);
            const double *rb = (const double *)(smem + OFF_RAW + sb * RAW_BYTES);
            // the row's largest exponent: this thread's 32 values, then its partner's
            int mx = 0;
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const double *src = (c < 2 ? ra : rb) + (size_t)(16 * (c & 1) + 8 * hh) * 128 + r;
#pragma unroll
                for (int e = 0; e < 8; e++) mx = max(mx, bexp(dbits(src[e * 128])));
            }
            mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, 1));
            if (hh == 0) s_rexp[it & 1][r] = mx;
            bool ok = true;
#pragma unroll 1
            for (int c = 0; c < 4; c++, g++) {
                const uint32_t ds = g % DIG_SLOTS;
                if (g >= DIG_SLOTS &&
                    !tc::wait_abort_warp(&dig_empty[ds], ((g / DIG_SLOTS) - 1) & 1, s_abort, status, ST_WAIT_TIMEOUT)) {
                    ok = false;
                    break;
                }
                const double *src = (c < 2 ? ra : rb) + (size_t)(16 * (c & 1) + 8 * hh) * 128 + r;
                long long Xv[8];
#pragma unroll
                for (int e = 0; e < 8; e++) Xv[e] = fixed56(dbits(src[e * 128]), mx);
                uint32_t w0[NS], w1[NS], w2[NS], w3[NS];
                digit_pair(Xv[0], Xv[1], w0);
                digit_pair(Xv[2], Xv[3], w1);
                digit_pair(Xv[4], Xv[5], w2);
                digit_pair(Xv[6], Xv[7], w3);
                uint8_t *dst = smem + OFF_DIG + ds * DIG_BYTES + (r >> 3) * DIG_SBO + hh * LBO + (r & 7) * 16;
#pragma unroll
                for (int s = 0; s < NS; s++) *(uint4 *)(dst + s * DIG_SLICE) = make_uint4(w0[s], w1[s], w2[s], w3[s]);
                tc::fence_proxy_async_smem();
                __syncwarp();
                if (lane == 0) {
                    tc::mbar_arrive(&dig_full[ds]);
                    if (c == 1) tc::mbar_arrive(&raw_empty[sa]);  // chunks 0, 1 were the first half tile
                    if (c == 3) tc::mbar_arrive(&raw_empty[sb]);
                }
            }
            if (!ok) break;
        }
    } else {
        // ---- epilogue: warps 0..7, TMEM lane quarter q, output columns 32 h .. + 32
        const int q = warp & 3, h = warp >> 2;
        const int rr = 32 * q + lane;
        uint32_t cmax[4][4];
#pragma unroll
        for (int c = 0; c < 4; c++)
#pragma unroll
            for (int p = 0; p < 4; p++) cmax[c][p] = 0u;
        int it = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, it++) {
            if (!tc::wait_abort_warp(&tm_full, it & 1, s_abort, status, ST_WAIT_TIMEOUT)) break;
            tc::fence_after_sync();
            const int er = s_rexp[it & 1][rr];
            const int orow = t * 128 + rr;
#pragma unroll
            for (int ch = 0; ch < 4; ch++) {
                const uint32_t col = (uint32_t)(32 * h + 8 * ch);
                const uint32_t ta = tbase + ((uint32_t)(32 * q) << 16) + col;
                long long hi[8], lo[8];
                {
                    uint32_t v[4][8];
#pragma unroll
                    for (int d = 0; d < 4; d++) tc::tmem_ld8(ta + (uint32_t)(64 * d), v[d]);
                    tc::tmem_ld_wait();
#pragma unroll
                    for (int j = 0; j < 8; j++) hi[j] = combine4(v[0][j], v[1][j], v[2][j], v[3][j]);
                }
                {
                    uint32_t v[4][8];
#pragma unroll
                    for (int d = 0; d < 4; d++) tc::tmem_ld8(ta + (uint32_t)(64 * (d + 4)), v[d]);
                    tc::tmem_ld_wait();
#pragma unroll
                    for (int j = 0; j < 8; j++) lo[j] = combine4(v[0][j], v[1][j], v[2][j], v[3][j]);
                }
                if (ch == 3) {
                    // every TMEM read of this tile is done: the next tile's MMAs may start
                    tc::fence_before_sync();
                    __syncwarp();
                    if (lane == 0) tc::mbar_arrive(&tm_empty);
                }
                if (orow < m) {
                    uint32_t ex[8];
#pragma unroll
                    for (int j = 0; j < 8; j++) {
                        const int c = (int)col + j;
                        ex[j] = 0;
                        if (c < nout) {
                            const int fx = s_xexp[c];
                            const int sc = (er - 1022) + (fx - 1022) - 63;
                            const double v = (er && fx) ? (kIntAsm ? assemble_int(hi[j], lo[j], sc)
                                                                   : assemble_fast(hi[j], lo[j], sc))
                                                        : 0.0;
                            a.out[(size_t)orow + (size_t)c * a.ldo] = v;
                            ex[j] = (uint32_t)bexp(dbits(v));
                        }
                    }
#pragma unroll
                    for (int p = 0; p < 4; p++) cmax[ch][p] = __vmaxu2(cmax[ch][p], ex[2 * p] | (ex[2 * p + 1] << 16));
                }
            }
        }
        if (a.colexp_out) {
#pragma unroll
            for (int ch = 0; ch < 4; ch++)
#pragma unroll
                for (int p = 0; p < 4; p++) {
                    uint32_t v = cmax[ch][p];
                    for (int o = 16; o > 0; o >>= 1) v = __vmaxu2(v, __shfl_xor_sync(0xffffffffu, v, o));
                    if (lane == 0) {
#pragma unroll
                        for (int hw = 0; hw < 2; hw++) {
                            const int c = 32 * h + 8 * ch + 2 * p + hw;
                            const int e = (int)((v >> (16 * hw)) & 0xFFFFu);
                            if (c < nout && e) {
                                if (e == 0x7FF) atomicOr(status, ST_NONFINITE);
                                atomicMax(&a.colexp_out[c], e);
                            }
                        }
                    }
                }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == W_MMA) tc::tmem_dealloc(tbase, 512);
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
constexpr int GT_FLUSH = 2;                            // stages per flush window (128 rows: |P_d| < 2^22)
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
};

__global__ void __launch_bounds__(GT_NT, 1)
    k_gram_tma(const __grid_constant__ CUtensorMap tmA, const GramTmaArgs g, int *status)
{
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
    for (int st = 0; st < nstage; st++) {
        const int buf = st % GT_DIG;
        const uint32_t rs = st % GT_RAW;
        // the slot that stage st - 1 used is refilled with stage st - 1 + GT_RAW
        // once every warp has read it
        if (producer && st >= 1 && st - 1 + GT_RAW < nstage) {
            if (!tc::wait_abort(&raw_empty[(st - 1) % GT_RAW], ((st - 1) / GT_RAW) & 1, s_abort, status,
                                ST_WAIT_TIMEOUT))
                ;  // abort: the flag ends every warp's loop below
            else
                issue_raw(st - 1 + GT_RAW);
        }
        // digit buffer buf's previous stage (st - 2) has been read by the tensor core
        if (st >= GT_DIG &&
            !tc::wait_abort_warp(&empty_b[buf], ((st - GT_DIG) / GT_DIG) & 1, s_abort, status, ST_WAIT_TIMEOUT))
            break;
        if (!tc::wait_abort_warp(&raw_full[rs], (st / GT_RAW) & 1, s_abort, status, ST_WAIT_TIMEOUT)) break;
        unsigned long long uv[8];
        {
            const uint8_t *col = smem + GT_OFF_RAW + rs * GT_RAW_BYTES + (uk >> 1) * GT_BOX_BYTES + uc * 128;
            const int row0 = r_beg + st * GT_KC + 8 * uk;
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
        const bool window_start = (st % GT_FLUSH) == 0;
        if (issuer) {
            bool ok = tc::wait_abort(&full_b[buf], (st / GT_DIG) & 1, s_abort, status, ST_WAIT_TIMEOUT);
            if (ok && window_start && st > 0)
                ok = tc::wait_abort(&tfree, ((st / GT_FLUSH) - 1) & 1, s_abort, status, ST_WAIT_TIMEOUT);
            if (ok) {
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
                        tc::mma_bf16(tbase + 64 * s, ad, tc::desc_nosw(sb + koff, LBO, GT_SBO),
                                     tc::idesc_bf16_f32(128, n1), acc);
                        if (ntot > 256)
                            tc::mma_bf16(tbase + 64 * s + 256, ad, tc::desc_nosw(sb + 4 * GT_SLICE + koff, LBO, GT_SBO),
                                         tc::idesc_bf16_f32(128, ntot - 256), acc);
                    }
                }
                tc::mma_commit(&empty_b[buf]);
                last_commit = st;
            }
        }
        if (__any_sync(0xffffffffu, *s_abort)) break;
        const bool flush = ((st + 1) % GT_FLUSH) == 0 || st == nstage - 1;
        if (flush) {
            // this stage's commit also covers every earlier MMA (in-order issue)
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
                   int *colexp_out, bool int_asm)
{
    CUtensorMap tm;
    if (!tma_map_2d(&tm, A, lda, m, n, 128, 32)) return false;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(ozs::k_map_tma<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ozs::SMEM_BYTES);
        cudaFuncSetAttribute(ozs::k_map_tma<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ozs::SMEM_BYTES);
        attr = true;
    }
    const int tiles = (m + 127) / 128;
    const int grid = tiles < sm_count() ? tiles : sm_count();
    ozs::MapTmaArgs args{m, n, X, ldx, nout, out, ldo, colexp_out};
    trace_begin();
    if (int_asm)
        ozs::k_map_tma<true><<<grid, ozs::THREADS, ozs::SMEM_BYTES, stream()>>>(tm, args, status_ptr());
    else
        ozs::k_map_tma<false><<<grid, ozs::THREADS, ozs::SMEM_BYTES, stream()>>>(tm, args, status_ptr());
    note_launch("ozaki_map");
    return true;
}

// The CTA grid's integer Gram partials of A (rows_per rows per CTA, a
// multiple of 64) by the TMA-fed kernel; false (nothing enqueued) when A does
// not meet TMA's alignment rules.
bool ozaki_gram_tma(int m, int n, const double *A, int lda, int rows_per, const int *colexp, long long *partial,
                    int parts)
{
    CUtensorMap tm;
    if (!tma_map_2d(&tm, A, lda, m, n, 16, 64, true)) return false;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(ozs::k_gram_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ozs::GT_SMEM);
        attr = true;
    }
    ozs::GramTmaArgs args{m, n, rows_per, colexp, partial};
    trace_begin();
    ozs::k_gram_tma<<<parts, ozs::GT_NT, ozs::GT_SMEM, stream()>>>(tm, args, status_ptr());
    note_launch("ozaki_gram");
    return true;
}

}  // namespace lg
