// lg_tsmixed.cu -- tall-skinny QR leaf with FP64-grade split-precision
// products: Cholesky QR 2 (shifted Cholesky QR 3 when the matrix is too
// ill-conditioned for the plain Gram) followed by Householder reconstruction,
// returning the same V, R, T and Q as lila_dgeqrf_w03_mt_hr
// (lila-c/lila_dgeqrf_w03_mt_hr.c:3-33, lila_ormhr2_w03_hr.c:3-84).
//
// Data flow for the leaf block A(i:m, i:i+n), ml = m - i, n <= 64:
//   G1 = A^T A                 (split-precision Gram, tensor cores)
//   R1 = chol(G1 [+ sigma I])  (FP64, one CTA; sigma only for the shifted form)
//   Q  = A R1^-1               (split-precision row map into the Q buffer)
//   repeat 1 or 2 times: G = Q^T Q, Rk = chol(G), R = Rk R, and, except for
//   the last pass, Q = Q Rk^-1 (in place)
//   with Xl = Rk^-1 of the last pass the final orthonormal factor is Q Xl; the
//   sign-choice LU of its top n x n block and the tile coupling of the
//   reconstruction are done on n x n FP64 matrices, yielding two n x n maps:
//   M_V (rows below the leaf's top block -> V) and M_Q = Xl S (-> Q S).
//   V(i+n:m) = Q M_V and Q = Q M_Q are two more split-precision row maps.
#include <math.h>
#include <string.h>

#include <algorithm>

#include "lg_common.cuh"
#include "../../include/lila.h"
#include "../../include/lila_gpu.h"

namespace lg {

static inline int imin2(int a, int b) { return a < b ? a : b; }
static inline int tile_end2(int a, int end, int mt)
{
    int b = (a / mt + 1) * mt;
    return b < end ? b : end;
}

__global__ void k_status_or(int *status, int bits) { atomicOr(status, bits); }

// The pass control block (see k_factor_pass below).
constexpr int kMaxPasses = 5;

// sigma / ||Q||_F^2 of the shifted passes for an ml x n leaf (see the pass
// control below); the chunked out-of-core Gram is a double-double sum of
// such Grams and takes the same bound.
static double leaf_shift_factor(int ml, int n)
{
    const double u = 0x1p-53;
    return 11.0 * ((double)n * (n + 1) * u + 0x1p-49 * sqrt((double)ml));
}

struct PassCtl {
    int active;          // 1 while passes remain: the next Gram, factor and map run
    int plain_run;       // unshifted passes in a row
    int passes;          // passes factored
    int shifted_passes;
    int ran;             // the last factor launch did its pass (R = Rk R follows)
};

// Rows of A kept for the residual check: every stride-th row of the leaf,
// at most kSampleRows of them.
constexpr int kSampleRows = 8192;

struct MixedWs {
    double *G, *R, *Rk, *X, *Tmp, *Qt, *Atop, *MV, *MQ, *W, *S;
    PassCtl *ctl;  // the device-side pass control
    double *chk;  // [0] sum of squared residuals, [1] sum of squares of the sampled rows, [2] res, [3] orth,
                  // [4] failed, [5] unshifted passes in a row at the end (see k_check_decide)
    double *As;   // the sampled rows of A (kSampleRows x 64, ld kSampleRows)
    double *oz;
    long long ozlen;
};

static long long mixed_ws_len(int n)
{
    // 10 n x n blocks (64 x 64), S, pass control, check scalars, sampled rows, Gram workspace
    return 10LL * 64 * 64 + 64 + 64 + 64 + (long long)kSampleRows * 64 + ozaki_gram_work(sm_count());
}

static MixedWs carve(double *w, long long len)
{
    MixedWs s;
    const long long B = 64 * 64;
    s.G = w;
    s.R = w + B;
    s.Rk = w + 2 * B;
    s.X = w + 3 * B;
    s.Tmp = w + 4 * B;
    s.Qt = w + 5 * B;
    s.Atop = w + 6 * B;
    s.MV = w + 7 * B;
    s.MQ = w + 8 * B;
    s.W = w + 9 * B;
    s.S = w + 10 * B;
    s.ctl = (PassCtl *)(w + 10 * B + 64 + 8);
    s.chk = w + 10 * B + 128;
    s.As = w + 10 * B + 192;
    s.oz = s.As + (long long)kSampleRows * 64;
    s.ozlen = len - (s.oz - w);
    return s;
}

// ---------------------------------------------------------------------------
// On-device accuracy check of the leaf's result, the measures of
// lila_test_qq_orth_1 (||I - Q^T Q||_F) and lila_test_qr_repres_1
// (||A - Q R||_F / ||A||_F) (lila-c-lila_param/lila/src/lila_test_qq_orth_1.c:3-19,
// lila_test_qr_repres_1.c:3-27):
//   orth: level 1 takes it from the last pass's Gram G = C^T C of the
//         candidate C that the final row map turns into Q = C M_Q:
//         Q^T Q = M_Q^T G M_Q up to the rounding of that FP64-grade map (an
//         n x n computation); level 2 forms Q^T Q of the output by one more
//         split-precision Gram pass over Q.
//   res:  over every stride-th row of the leaf (at most kSampleRows rows,
//         gathered before the final map overwrites A with V), the ratio of
//         the residual rows ||a_r - q_r R|| to ||a_r||, in FP64.
// Both are compared with 50 n 2^-53.
// ---------------------------------------------------------------------------
static int sample_stride(int ml) { return ml <= kSampleRows ? 1 : (ml + kSampleRows - 1) / kSampleRows; }
static int sample_count(int ml, int stride) { return (ml + stride - 1) / stride; }

__global__ void k_gather_rows(int ns, int n, int stride, const double *A, int lda, double *As)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= ns) return;
    const size_t r = (size_t)s * stride;
    for (int c = 0; c < n; c++) As[s + (size_t)c * kSampleRows] = A[r + (size_t)c * lda];
}

// acc[0] += sum_s ||a_s - q_s triu(R)||^2, acc[1] += sum_s ||a_s||^2 over the
// sampled rows s (row s * stride of Q).  A CTA takes 32 sampled rows; warp w
// forms columns 16 w .. 16 w + 15 of q_s triu(R) (16 independent sums per
// thread, k running only to the warp's last column).
__global__ void __launch_bounds__(128) k_res_sample(int ns, int n, int stride, const double *As, const double *Q,
                                                    int ldq, const double *R, int ldr, double *acc)
{
    __shared__ double Rs[64 * 64];
    __shared__ double red[2][4];
    for (int k = threadIdx.x; k < 64 * 64; k += blockDim.x) {
        const int r = k & 63, c = k >> 6;
        Rs[k] = (r <= c && c < n) ? R[r + (size_t)c * ldr] : 0.0;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int s = blockIdx.x * 32 + lane;
    double e2 = 0.0, a2 = 0.0;
    if (s < ns) {
        const size_t row = (size_t)s * stride;
        double v[16];
#pragma unroll
        for (int c = 0; c < 16; c++) v[c] = 0.0;
        const int kend = min(n, 16 * w + 16);
#pragma unroll 4
        for (int k = 0; k < kend; k++) {
            const double q = Q[row + (size_t)k * ldq];
            const double *rk = Rs + k + 64 * 16 * w;
#pragma unroll
            for (int c = 0; c < 16; c++) v[c] = fma(q, rk[64 * c], v[c]);
        }
#pragma unroll
        for (int c = 0; c < 16; c++) {
            const int col = 16 * w + c;
            if (col < n) {
                const double a = As[s + (size_t)col * kSampleRows];
                e2 += (a - v[c]) * (a - v[c]);
                a2 += a * a;
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        e2 += __shfl_xor_sync(0xffffffffu, e2, o);
        a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    if (lane == 0) {
        red[0][w] = e2;
        red[1][w] = a2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        atomicAdd(&acc[0], red[0][0] + red[0][1] + red[0][2] + red[0][3]);
        atomicAdd(&acc[1], red[1][0] + red[1][1] + red[1][2] + red[1][3]);
    }
}

// orth = ||E - I||_F (E n x n), res = sqrt(acc[0] / acc[1]); acc[2] = res,
// acc[3] = orth; acc[4] = 1 when either exceeds tol (or is not finite),
// else 0; acc[5] = the unshifted passes in a row that ended the pass control
// ctl (2 without one).  fail_bits are ORed into the status word on a failure.
__global__ void k_check_decide(int n, const double *E, int lde, double *acc, double tol, const PassCtl *ctl,
                               int *status, int fail_bits)
{
    __shared__ double red[8];
    double v = 0.0;
    for (int k = threadIdx.x; k < n * n; k += blockDim.x) {
        const int r = k % n, c = k / n;
        const double d = E[r + (size_t)c * lde] - (r == c ? 1.0 : 0.0);
        v += d * d;
    }
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
        const double orth = sqrt(t);
        const double res = acc[1] > 0.0 ? sqrt(acc[0] / acc[1]) : sqrt(acc[0]);
        acc[2] = res;
        acc[3] = orth;
        const bool bad = !(res <= tol) || !(orth <= tol);
        acc[4] = bad ? 1.0 : 0.0;
        acc[5] = ctl ? (double)ctl->plain_run : 2.0;
        if (bad && fail_bits) atomicOr(status, fail_bits);
    }
}

static GemmEpi ep(double a, double b)
{
    GemmEpi e;
    e.alpha = a;
    e.beta = b;
    return e;
}

// The reconstruction on n x n data (lila-c/lila_ormhr2_w03_hr.c:23-80 per tile,
// with the tall rows deferred to the row maps): inputs Qt = top n rows of the
// final orthonormal factor, R (upper, final), Xl; outputs Atop (leaf top block
// of A: S R above the diagonal, L and V rows below), T tiles, S, MQ, MV.
static void reconstruct_small(int n, int i0, int mt, MixedWs &w, double *T, int ldt)
{
    // Atop = upper(R), strictly lower zero
    set2d(n, n, 0.0, 0.0, w.Atop, n, 0);
    GemmEpi e = ep(1, 0);
    copy2d(n, n, w.R, n, w.Tmp, n);
    set2d(n, n, 0.0, 0.0, w.Tmp, n, 2);
    copy2d(n, n, w.Tmp, n, w.Atop, n);
    for (int j = i0; j < i0 + n;) {
        const int nt = imin2(tile_end2(j, i0 + n, mt) - j, n);
        const int lj = j - i0;
        double *Tj = T + (j % mt) + (size_t)j * ldt;
        if (lj > 0) {
            flip_rows(lj, nt, w.S, w.Atop + (size_t)lj * n, n, 0);
            // W = L_prev^-1 Qt(0:lj, tile)
            copy2d(lj, nt, w.Qt + (size_t)lj * n, n, w.W, lj);
            trsm_left_lower_unit(lj, nt, w.Atop, n, w.W, lj);
            // Qt(lj:n, tile) -= Atop(lj:n, 0:lj) W
            gemm(n - lj, nt, lj, opnd(w.Atop + lj, n), opnd(w.W, lj), w.Qt + lj + (size_t)lj * n, n, ep(-1, 1));
            // MV(:, tile) = Xl(:, tile) - MV(:, 0:lj) W
            copy2d(n, nt, w.X + (size_t)lj * n, n, w.MV + (size_t)lj * n, n);
            gemm(n, nt, lj, opnd(w.MV, n), opnd(w.W, lj), w.MV + (size_t)lj * n, n, ep(-1, 1));
        } else {
            copy2d(n, nt, w.X, n, w.MV, n);
        }
        copy2d(nt, nt, w.Qt + lj + (size_t)lj * n, n, Tj, ldt);
        lu_sign(nt, Tj, ldt, w.S + lj);
        flip_rows(nt, nt, w.S + lj, w.Atop + lj + (size_t)lj * n, n, 1);
        move_strict_lower_dev(nt, Tj, ldt, w.Atop + lj + (size_t)lj * n, n);
        const int below = n - lj - nt;
        if (below > 0) {
            copy2d(below, nt, w.Qt + lj + nt + (size_t)lj * n, n, w.Atop + lj + nt + (size_t)lj * n, n);
            trsm_right_upper(below, nt, 1.0, Tj, ldt, w.Atop + lj + nt + (size_t)lj * n, n, w.S + lj, "hr_small");
        }
        trsm_right_upper(n, nt, 1.0, Tj, ldt, w.MV + (size_t)lj * n, n, w.S + lj, "hr_small");
        trsm_right_lower_unit_trans(nt, nt, -1.0, w.Atop + lj + (size_t)lj * n, n, Tj, ldt);
        j += nt;
    }
    (void)e;
    copy2d(n, n, w.X, n, w.MQ, n);
    flip_cols(n, n, w.S, w.MQ, n);
}

// ---------------------------------------------------------------------------
// Pass control on the device.  Each pass factors the Gram of the current
// orthonormal candidate (A for the first pass).  A pass whose trial Cholesky
// breaks down or whose factor has a 1-norm condition estimate above 1e7 is
// redone with a shift sigma = shift_factor ||Q||_F^2 (shifted Cholesky QR);
// the leaf stops after two consecutive unshifted passes (Cholesky QR 2), so
// a matrix of condition number kappa takes about
// log(kappa / 1e7) / log(1 / sqrt(shift_factor)) shifted passes before the
// final two.
//
// The shift has to exceed the error of the computed Gram plus the backward
// error of its Cholesky factorization.  The shifted Cholesky QR of the
// literature uses 11 (m n + n (n + 1)) u: the m n u term bounds a Gram summed
// in FP64 (gamma_m of dsyrk).  The split-precision Gram here is an exact
// integer sum rounded once, whose error per entry is below
// 2^-50 (max|a_i| sum|a_j| + sum|a_i| max|a_j|) <= 2^-49 sqrt(m) ||a_i|| ||a_j||
// (the bound the product tests check), so shift_factor =
// 11 (n (n + 1) u + 2^-49 sqrt(m)): for 4,194,304 x 64, 4.5e-11 instead of
// 3.3e-7, and one shifted pass divides the condition number by about 1.5e5
// instead of 1.7e3 (kappa 1e10 takes one shifted pass, 1e14 two).
// The decisions are taken by k_factor_pass and kept in a PassCtl block in
// the workspace: the host enqueues kMaxPasses passes and the Gram, factor
// and row-map kernels of the passes after the last one do nothing (their
// launches read `active` first), so the leaf never waits for the host
// between passes.
// ---------------------------------------------------------------------------
__global__ void k_pass_init(PassCtl *c)
{
    c->active = 1;
    c->plain_run = 0;
    c->passes = 0;
    c->shifted_passes = 0;
    c->ran = 0;
}

constexpr int FP_LD = 65;  // padded leading dimension of the 64 x 64 blocks in shared memory
constexpr int FP_NT = 512;
constexpr int FP_YLD = 33;  // leading dimension of the inverse's 32 x 32 product blocks
constexpr size_t FP_SMEM = (3 * 64 * FP_LD + 32 * FP_YLD) * sizeof(double);

// Upper Cholesky factor of the n x n block K (in place, ld FP_LD, upper
// triangle used), right-looking with the pivot one step ahead: in step j
// warp 0 applies row j of R to row j + 1, takes that row's pivot (rsqrt_nr)
// and scales the row, while the warps of the other three SM sub-partitions
// (warp % 4 != 0) apply row j to rows j + 2 .. n - 1, so a step ends with one
// block barrier and warp 0's FP64 chain shares its sub-partition with no
// update work.  Returns 0, 1 at a pivot that is not positive and finite (the
// block is then partly factored) or, with ratio_limit > 0, 2 as soon as the
// largest diagonal entry of R exceeds ratio_limit times the smallest (a
// lower bound of the 1-norm condition number of R).  s_flag is a pair of
// shared words the caller has zeroed behind a barrier: pivot j reports in
// s_flag[j & 1], read by every thread after the barrier that ends its step,
// and next written two steps later, after the following barrier.
__device__ int sm_potrf(int n, double *K, double ratio_limit, int *s_flag)
{
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    double dmax = 0.0, dmin = INFINITY;  // warp 0: the diagonal of R so far
    // warp 0: row j of K (already updated by rows 0 .. j - 1) factored and scaled
    auto pivot_row = [&](int j, double v0, double v1) {
        const int c0 = j + lane, c1 = c0 + 32;
        const double d = __shfl_sync(0xffffffffu, v0, 0);
        if (!(d > 0.0) || !isfinite(d)) {
            if (lane == 0) s_flag[j & 1] = 1;
            return;
        }
        const double y = rsqrt_nr(d), r = d * y;
        dmax = fmax(dmax, r);
        dmin = fmin(dmin, r);
        if (c0 < n) K[c0 * FP_LD + j] = lane == 0 ? r : v0 * y;
        if (c1 < n) K[c1 * FP_LD + j] = v1 * y;
        if (lane == 0 && ratio_limit > 0.0 && !(dmax <= ratio_limit * dmin)) s_flag[j & 1] = 2;
    };
    if (warp == 0) {
        const double v0 = lane < n ? K[lane * FP_LD] : 0.0;
        const double v1 = lane + 32 < n ? K[(lane + 32) * FP_LD] : 0.0;
        pivot_row(0, v0, v1);
    }
    __syncthreads();
    for (int j = 0; j + 1 < n; j++) {
        if (s_flag[j & 1]) return s_flag[j & 1];
        if (warp == 0) {
            // row j + 1 -= R(j, j + 1) R(j, :)
            const int c0 = j + 1 + lane, c1 = c0 + 32;
            const double a = K[(j + 1) * FP_LD + j];
            const double v0 = c0 < n ? fma(-a, K[c0 * FP_LD + j], K[c0 * FP_LD + j + 1]) : 0.0;
            const double v1 = c1 < n ? fma(-a, K[c1 * FP_LD + j], K[c1 * FP_LD + j + 1]) : 0.0;
            pivot_row(j + 1, v0, v1);
        } else if (warp & 3) {
            // rows p = j + 2 .. n - 1: element e = c (c + 1) / 2 + q of the
            // trailing upper triangle (columns c = 0 .. w - 1, rows q <= c, offset j + 2)
            const int wid = warp - (warp >> 2) - 1;  // 0 .. 11
            const int w = n - j - 2, tot = w * (w + 1) / 2;
            for (int e = wid * 32 + lane; e < tot; e += 384) {
                int c = (int)((sqrtf(8.0f * e + 1.0f) - 1.0f) * 0.5f);
                if (c * (c + 1) / 2 > e) c--;
                if ((c + 1) * (c + 2) / 2 <= e) c++;
                const int p = j + 2 + e - c * (c + 1) / 2;
                c += j + 2;
                K[c * FP_LD + p] = fma(-K[p * FP_LD + j], K[c * FP_LD + j], K[c * FP_LD + p]);
            }
        }
        __syncthreads();
    }
    return s_flag[(n - 1) & 1];
}

// X = K^-1 for the upper 64 x 64 K (both ld FP_LD; entries outside the
// leading n x n block of K hold the identity), blocked: the eight 8 x 8
// diagonal blocks are inverted by one thread per column, then blocks are
// joined pairwise, 8 -> 16 -> 32 -> 64, by X12 = -(X11 K12) X22, Y = X11 K12
// staged in Y (32 x FP_YLD).  In each product the threads of a warp share
// one row (X11 K12) or one column (Y X22) and so the same loop length.
__device__ void sm_trinv(const double *K, double *X, double *Y, double *s_rd)
{
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int k = tid; k < 64 * FP_LD; k += FP_NT) X[k] = 0.0;
    if (tid < 64) s_rd[tid] = 1.0 / K[tid * FP_LD + tid];
    __syncthreads();
    if (tid < 64) {
        // column kk = 8 b + k of diagonal block b
        const int b = tid >> 3, k = tid & 7, s = 8 * b, kk = s + k;
        const double dk = s_rd[kk];
        double x[8];
#pragma unroll
        for (int i = 0; i < 8; i++) x[i] = i == k ? dk : 0.0;
#pragma unroll
        for (int i = 6; i >= 0; i--) {
            if (i < k) {
                double sum = 0.0;
#pragma unroll
                for (int p = i + 1; p < 8; p++)
                    if (p <= k) sum = fma(K[(s + p) * FP_LD + s + i], x[p], sum);
                x[i] = -sum * s_rd[s + i];
            }
        }
#pragma unroll
        for (int i = 0; i < 8; i++)
            if (i <= k) X[kk * FP_LD + s + i] = x[i];
    }
    __syncthreads();
    for (int bs = 8; bs < 64; bs *= 2) {
        // lane = (pair q, index t): pair q joins the blocks at s = 2 bs q and s + bs
        const int q = lane / bs, t = lane % bs, s = 2 * bs * q, h = s + bs;
        double *Yq = Y + q * bs * (bs + 1);  // Y(i, k) at Yq[k (bs + 1) + i]
        // Y = X11 K12: warp row i, lane column t
        for (int i = warp; i < bs; i += FP_NT / 32) {
            double sum = 0.0;
            for (int p = i; p < bs; p++) sum = fma(X[(s + p) * FP_LD + s + i], K[(h + t) * FP_LD + s + p], sum);
            Yq[t * (bs + 1) + i] = sum;
        }
        __syncthreads();
        // X12 = -Y X22: warp column k, lane row t
        for (int k = warp; k < bs; k += FP_NT / 32) {
            double sum = 0.0;
            for (int p = 0; p <= k; p++) sum = fma(Yq[p * (bs + 1) + t], X[(h + k) * FP_LD + h + p], sum);
            X[(h + k) * FP_LD + s + t] = -sum;
        }
        __syncthreads();
    }
}

// max over columns c < n of sum_{r <= c} |B(r, c)| for the upper n x n blocks
// K and X (ld FP_LD): eight threads per column, then warp 0 over the columns.
__device__ void sm_norm1_pair(int n, const double *K, const double *X, double *s_nk, double *s_nx, double *out)
{
    const int tid = threadIdx.x, c = tid >> 3, l = tid & 7;
    double a = 0.0, b = 0.0;
    if (c < n)
        for (int r = l; r <= c; r += 8) {
            a += fabs(K[c * FP_LD + r]);
            b += fabs(X[c * FP_LD + r]);
        }
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if (l == 0) {
        s_nk[c] = a;
        s_nx[c] = b;
    }
    __syncthreads();
    if (tid < 32) {
        a = fmax(s_nk[tid], s_nk[tid + 32]);
        b = fmax(s_nx[tid], s_nx[tid + 32]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a = fmax(a, __shfl_xor_sync(0xffffffffu, a, o));
            b = fmax(b, __shfl_xor_sync(0xffffffffu, b, o));
        }
        if (tid == 0) {
            out[0] = a;
            out[1] = b;
        }
    }
    __syncthreads();
}

// One pass's factor from its Gram G (n x n, ld ldg), in one CTA of 512
// threads with the 64 x 64 blocks in shared memory: the trial Cholesky
// factor Rk of G (variant 0; its breakdown is not recorded in the status
// word), X = Rk^-1 and the 1-norm condition estimate ||Rk||_1 ||X||_1 (the
// trial stops as soon as the diagonal ratio max r_kk / min r_kk, a lower
// bound of it, exceeds the limit); when the trial fails (or for the first
// pass of variant 2) the shifted factor of G + sigma I, sigma = shift_factor
// trace(G); then Rk and X in global memory (k_rk_r forms R = Rk R) and the
// pass control updated.  Does nothing but clear ctl->ran once ctl->active
// is 0.
__global__ void __launch_bounds__(FP_NT, 1)
    k_factor_pass(int n, const double *G, int ldg, double *Rk, int ldk, double *X, int ldx, PassCtl *ctl,
                  int variant, double shift_factor, double cond_limit, int *status)
{
    if (!ctl->active) {
        if (threadIdx.x == 0) ctl->ran = 0;
        return;
    }
    extern __shared__ double fsm[];
    double *sG = fsm;                   // the Gram
    double *sK = fsm + 64 * FP_LD;      // Rk
    double *sX = fsm + 2 * 64 * FP_LD;  // Rk^-1
    double *sY = fsm + 3 * 64 * FP_LD;  // products of the blocked inverse
    __shared__ double s_rd[64], s_nk[64], s_nx[64], s_norms[2];
    __shared__ double s_sigma;
    __shared__ int s_flag[2], s_shift;
    const int tid = threadIdx.x;
    const int passes = ctl->passes;
    for (int k = tid; k < n * n; k += FP_NT) {
        const int r = k % n, c = k / n;
        sG[c * FP_LD + r] = G[r + (size_t)c * ldg];
    }
    if (tid == 0) s_shift = (variant == 2 && passes == 0) ? 1 : 0;
    __syncthreads();
    // K = upper(G) + add I on the leading n x n block, the identity outside it
    auto load_k = [&](double add) {
        for (int k = tid; k < 64 * 64; k += FP_NT) {
            const int r = k & 63, c = k >> 6;
            double v = r == c ? 1.0 : 0.0;
            if (r < n && c < n) v = r <= c ? sG[c * FP_LD + r] + (r == c ? add : 0.0) : 0.0;
            sK[c * FP_LD + r] = v;
        }
        if (tid < 2) s_flag[tid] = 0;
        __syncthreads();
    };
    if (!s_shift) {
        load_k(0.0);
        const int rc = sm_potrf(n, sK, variant != 1 ? cond_limit : 0.0, s_flag);
        if (variant != 1) {
            // trial: its breakdown, its diagonal ratio or a large condition estimate selects the shift
            bool good = rc == 0;
            if (good) {
                sm_trinv(sK, sX, sY, s_rd);
                sm_norm1_pair(n, sK, sX, s_nk, s_nx, s_norms);
                const double a = s_norms[0], b = s_norms[1];
                good = isfinite(a) && isfinite(b) && a * b <= cond_limit;
            }
            if (!good && tid == 0) s_shift = 1;
            __syncthreads();
        } else {
            if (rc && tid == 0) atomicOr(status, ST_CHOL_BREAKDOWN);
            sm_trinv(sK, sX, sY, s_rd);
        }
    }
    if (s_shift) {
        if (tid < 32) {
            double t = (tid < n ? sG[tid * FP_LD + tid] : 0.0) + (tid + 32 < n ? sG[(tid + 32) * FP_LD + tid + 32] : 0.0);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
            if (tid == 0) s_sigma = shift_factor * t;
        }
        __syncthreads();
        load_k(s_sigma);
        if (sm_potrf(n, sK, 0.0, s_flag) && tid == 0) atomicOr(status, ST_CHOL_BREAKDOWN);
        sm_trinv(sK, sX, sY, s_rd);
    }
    for (int k = tid; k < n * n; k += FP_NT) {
        const int r = k % n, c = k / n;
        Rk[r + (size_t)c * ldk] = sK[c * FP_LD + r];
        X[r + (size_t)c * ldx] = sX[c * FP_LD + r];
    }
    if (tid == 0) {
        PassCtl c = *ctl;
        c.ran = 1;
        if (s_shift) {
            c.shifted_passes++;
            c.plain_run = 0;
        } else {
            c.plain_run++;
        }
        c.passes++;
        c.active = (c.plain_run < 2 && c.passes < kMaxPasses) ? 1 : 0;
        *ctl = c;
    }
}

// R = Rk R (both upper triangular, n x n, ld n) after a factor pass that
// ran: CTA j forms column j (thread i: sum_{q = i}^{j} Rk(i, q) R(q, j)).
__global__ void k_rk_r(int n, const double *Rk, double *R, const PassCtl *ctl)
{
    if (!ctl->ran) return;
    __shared__ double col[64];
    const int j = blockIdx.x, i = threadIdx.x;
    if (i < n) col[i] = R[i + (size_t)j * n];
    __syncthreads();
    if (i < n) {
        double v = 0.0;
        for (int q = i; q <= j; q++) v = fma(Rk[i + (size_t)q * n], col[q], v);
        R[i + (size_t)j * n] = v;
    }
}

static void factor_pass_attr()
{
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_factor_pass, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FP_SMEM);
        attr = true;
    }
}

static void factor_pass_dev(int n, MixedWs &w, PassCtl *ctl, int variant, double shift_factor)
{
    factor_pass_attr();
    trace_begin();
    k_factor_pass<<<1, FP_NT, FP_SMEM, stream()>>>(n, w.G, n, w.Rk, n, w.X, n, ctl, variant, shift_factor, 1e7,
                                                   status_ptr());
    note_launch("factor_pass");
    trace_begin();
    k_rk_r<<<n, 64, 0, stream()>>>(n, w.Rk, w.R, ctl);
    note_launch("factor_rk_r");
}

// rsqrt_nr elementwise (tests of the pivot step): 0 where d is not positive and finite.
__global__ void k_rsqrt_nr(int n, const double *d, double *out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const double x = d[i];
        out[i] = (x > 0.0 && isfinite(x)) ? rsqrt_nr(x) : 0.0;
    }
}

// The pass control of lila_prim_factor_pass.
__device__ PassCtl d_prim_ctl;

// The pass control of the last leaf, kept for lila_gpu_last_variant /
// lila_gpu_last_passes (copied on the device when the leaf ends).
__device__ PassCtl d_last_ctl;
__global__ void k_keep_ctl(const PassCtl *c) { d_last_ctl = *c; }

// Read on the library stream (stream-ordered, so that it waits for nothing
// but this thread's own work, not for copies on other streams).
static PassCtl last_ctl()
{
    PassCtl c{};
    if (cudaMemcpyFromSymbolAsync(&c, d_last_ctl, sizeof c, 0, cudaMemcpyDeviceToHost, stream()) != cudaSuccess ||
        cudaStreamSynchronize(stream()) != cudaSuccess)
        cudaGetLastError();
    return c;
}

static int g_check_level = 1;
static int g_last_fallback = 0;
static double g_last_check[2] = {-1.0, -1.0};  // res, orth of the last checked leaf

// Workspace of the FP64 fallback (the TSQR leaf on the leaf's ml rows) that
// follows the leaf's own workspace.
static long long fallback_ws_len(int ml, int n)
{
    if (ml < 1 || n < 1) return 0;
    return lila_query_dgeqrf_w03_tsqr(0, 0, ml, n, 0, 1) + (long long)n;
}

// The leaf's row scales (ml ints) after its own workspace and the
// fallback's; without room for both, after its own when the fallback has no
// room anyway; else none (the maps then find the row scales themselves).
static long long row_scales_len(int ml) { return ((long long)ml + 1) / 2 + 32; }
static int *row_scales_ws(int ml, int n, double *work, long long lwork)
{
    const long long own = mixed_ws_len(n), full = own + fallback_ws_len(ml, n);
    if (lwork >= full + row_scales_len(ml)) return (int *)(work + full);
    if (lwork < full && lwork >= own + row_scales_len(ml)) return (int *)(work + own);
    return nullptr;
}

// Runs the check on the current outputs (Q S in Qii, S R in the top block of
// Aii, ld lda) against the sampled rows in w.As; E is the n x n matrix whose
// distance to I is the orthogonality measure.  Returns the flag (1 failed).
static int check_result(int ml, int n, const double *Qii, int ldq, const double *Rtop, int ldr, const double *E,
                        MixedWs &w, int fail_bits, const PassCtl *ctl, int *plain_run)
{
    const double tol = 50.0 * n * 0x1p-53;
    const int stride = sample_stride(ml), ns = sample_count(ml, stride);
    cudaStream_t st = stream();
    cudaMemsetAsync(w.chk, 0, 2 * sizeof(double), st);
    trace_break();
    trace_begin();
    k_res_sample<<<(ns + 31) / 32, 128, 0, st>>>(ns, n, stride, w.As, Qii, ldq, Rtop, ldr, w.chk);
    note_launch("check_residual");
    trace_begin();
    k_check_decide<<<1, 256, 0, st>>>(n, E, n, w.chk, tol, ctl, status_ptr(), fail_bits);
    note_launch("check_decide");
    // one read of res, orth, the verdict and the pass control's end state, into
    // page-locked memory of this host thread
    static thread_local double *h = nullptr;
    if (!h && cudaMallocHost((void **)&h, 8 * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        h = nullptr;
    }
    double v[4] = {-1.0, -1.0, 1.0, 0.0};
    double *dst = h ? h : v;
    if (cudaMemcpyAsync(dst, w.chk + 2, 4 * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return 1;
    if (h) memcpy(v, h, sizeof v);
    g_last_check[0] = v[0];
    g_last_check[1] = v[1];
    if (plain_run) *plain_run = (int)v[3];
    return v[2] != 0.0 ? 1 : 0;
}

static int mixed_leaf(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt, double *Q, int ldq,
                      double *work, long long lwork, int variant)
{
    const int ml = m - i;
    double *Aii = A + i + (size_t)i * lda;
    double *Qii = Q + i + (size_t)i * ldq;
    MixedWs w = carve(work, lwork);
    const double shift_factor = leaf_shift_factor(ml, n);
    // R = I
    set2d(n, n, 0.0, 1.0, w.R, n, 0);
    trace_begin();
    k_pass_init<<<1, 1, 0, stream()>>>(w.ctl);
    note_launch("pass_init");
    // kMaxPasses passes are enqueued; those after the last one the device
    // decides on do nothing.  The candidate is A for the first pass and the
    // Q buffer (mapped in place) afterwards; every map leaves the column
    // scales of its output for the next Gram.
    // With room in the workspace, the scale pre-pass also writes A's row
    // scales and every map those of its output, so that each map knows its
    // input's row scales before it loads the rows (the maps run one K half
    // ahead; see ozaki_map).
    int *rexp = row_scales_ws(ml, n, work, lwork);
    const double *cur = Aii;
    int cur_ld = lda;
    const int *act = &w.ctl->active;
    for (int p = 0; p < kMaxPasses; p++) {
        ozaki_gram(ml, n, cur, cur_ld, w.G, n, w.oz, w.ozlen, 0, p > 0, act, rexp);
        factor_pass_dev(n, w, w.ctl, variant, shift_factor);
        if (p + 1 < kMaxPasses) {
            ozaki_map(ml, n, cur, cur_ld, w.X, n, n, Qii, ldq, (int *)w.oz, act, rexp, rexp);
            cur = Qii;
            cur_ld = ldq;
        }
    }
    trace_begin();
    k_keep_ctl<<<1, 1, 0, stream()>>>(w.ctl);
    note_launch("pass_keep");
    g_last_fallback = 0;
    g_last_check[0] = g_last_check[1] = -1.0;
    // the final orthonormal factor is Q X (the first pass's map always runs:
    // the leaf takes at least two passes)
    // top n rows of the final orthonormal factor, FP64 on n x n data
    gemm(n, n, n, opnd(Qii, ldq), opnd(w.X, n, NT, M_UPPER), w.Qt, n, ep(1, 0));
    reconstruct_small(n, i, mt, w, T, ldt);
    const int level = g_check_level;
    const int stride = sample_stride(ml), ns = sample_count(ml, stride);
    if (level > 0) {
        // A is intact until the V map below writes over it
        trace_begin();
        k_gather_rows<<<(ns + 127) / 128, 128, 0, stream()>>>(ns, n, stride, Aii, lda, w.As);
        note_launch("check_gather");
    }
    if (ml > n) ozaki_map(ml - n, n, Qii + n, ldq, w.MV, n, n, Aii + n, lda, nullptr, nullptr, rexp ? rexp + n : nullptr);
    ozaki_map(ml, n, Qii, ldq, w.MQ, n, n, Qii, ldq, level > 1 ? (int *)w.oz : nullptr, nullptr, rexp);
    copy2d(n, n, w.Atop, n, Aii, lda);
    if (level == 0) return 0;
    const long long base = mixed_ws_len(n);
    const bool can_fall_back = lwork >= base + fallback_ws_len(ml, n);
    if (level > 1) {
        ozaki_gram(ml, n, Qii, ldq, w.W, n, w.oz, w.ozlen, 0, true);
    } else {
        // Q^T Q = M_Q^T G M_Q from the last pass's Gram
        gemm(n, n, n, opnd(w.G, n), opnd(w.MQ, n), w.Tmp, n, ep(1, 0));
        gemm(n, n, n, opnd(w.MQ, n, TR), opnd(w.Tmp, n), w.W, n, ep(1, 0));
    }
    int plain_run = 0;
    int bad = check_result(ml, n, Qii, ldq, Aii, lda, w.W, w, 0, w.ctl, &plain_run);
    // passes that never reached two unshifted ones in a row leave a factor
    // the theory of Cholesky QR 2 does not cover: re-solved like a failure
    if (plain_run < 2) bad = 1;
    if (!bad) return 0;
    int st = 0;
    cudaMemcpyAsync(&st, status_ptr(), sizeof(int), cudaMemcpyDeviceToHost, stream());
    cudaStreamSynchronize(stream());
    if ((st & ST_NONFINITE) || !can_fall_back) {
        // non-finite input, or no workspace for the fallback: reported, not re-solved
        k_status_or<<<1, 1, 0, stream()>>>(status_ptr(), ST_CHECK_FAILED);
        note_launch("status_or");
        return 1;
    }
    // FP64 fallback.  The computed factors satisfy A = (Q S)(S R) to the
    // residual check, so a Householder QR of Q S (the TSQR leaf, stable at
    // any condition number and rank) Q S = Q' R' gives A = Q' (R' S R): the
    // leaf's outputs are the TSQR leaf's V, T and Q', with R' S R in place
    // of R'.  No copy of A is needed.
    g_last_fallback = 1;
    copy2d(ml, n, Qii, ldq, Aii, lda);
    const long long lw_ts = lwork - base;
    lila_dgeqrf_w03_tsqr(0, 0, m, n, i, mt, A, lda, T, ldt, Q, ldq, work + base,
                         lw_ts > 0x7fffffffLL ? 0x7fffffff : (int)lw_ts);
    // R' S R: upper-triangular product into the top block, its strictly lower part (L) kept
    copy2d(n, n, Aii, lda, w.Tmp, n);
    GemmEpi eu = ep(1, 0);
    eu.upper_only = 1;
    gemm(n, n, n, opnd(Aii, lda, NT, M_UPPER), opnd(w.Atop, n, NT, M_UPPER), w.Tmp, n, eu);
    copy2d(n, n, w.Tmp, n, Aii, lda);
    // the fallback's result is checked with the full measure
    ozaki_gram(ml, n, Qii, ldq, w.W, n, w.oz, w.ozlen, 0, false);
    bad = check_result(ml, n, Qii, ldq, Aii, lda, w.W, w, ST_CHECK_FAILED, nullptr, nullptr);
    return bad ? 1 : 0;
}

long long need_mixed_leaf(int n) { return mixed_ws_len(n); }
long long need_mixed_leaf_full(int ml, int n)
{
    return mixed_ws_len(n) + fallback_ws_len(ml, n) + row_scales_len(ml);
}

// ---------------------------------------------------------------------------
// Out-of-core form: the leaf above for an m x n matrix that stays in host
// memory.  The rows stream through the device in chunks of C rows on two
// copy streams (in, out) with two buffer slots, so the copies of chunk c + 1
// (and the write-back of chunk c - 1) overlap the work on chunk c.  Every
// pass reads A once: the factor candidate of pass p is A X_0 .. X_{p-1},
// recomputed per chunk by the same row maps the in-core leaf applies to the
// whole matrix (a row's map depends only on that row), instead of being
// stored.  The chunk Grams are summed in double-double (TwoSum), so the sum
// adds no rounding beyond the chunks' own.  The final pass writes V (rows
// n..m) into A and Q, as the in-core leaf does.
// ---------------------------------------------------------------------------

// hi + lo += g elementwise, exactly up to the final rounding of lo (TwoSum).
__global__ void k_twosum_acc(int len, const double *g, double *hi, double *lo)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < len; k += gridDim.x * blockDim.x) {
        const double a = hi[k], b = g[k];
        const double s = a + b;
        const double bb = s - a;
        const double e = (a - (s - bb)) + (b - bb);
        hi[k] = s;
        lo[k] += e;
    }
}

__global__ void k_twosum_fin(int len, const double *hi, const double *lo, double *out)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < len; k += gridDim.x * blockDim.x) out[k] = hi[k] + lo[k];
}

struct OocBufs {
    double *Xs;                     // the chain's factors inverses X_0 .. (8 blocks of 64 x 64)
    double *Ghi, *Glo, *Gc;         // the pass's Gram sum (double-double) and one chunk's Gram
    double *in[2], *mid[2], *vout[2];  // per slot: the chunk, the chain's other buffer, V rows
};

static int ooc_rows(int m, int n, int rows_per_chunk)
{
    long long c = rows_per_chunk > 0 ? rows_per_chunk : 1048576;
    c = c < n ? n : c;
    const long long mr = ((long long)m + 127) / 128 * 128;
    if (c > mr) c = mr;
    c = (c + 127) / 128 * 128;
    return (int)c;
}

// Doubles of the out-of-core workspace; carves it into w and b when base is set.
static long long ooc_layout(int n, int C, double *base, OocBufs *b)
{
    auto al = [](long long v) { return (v + 31) / 32 * 32; };
    const long long B = 64 * 64, CB = al((long long)C * n);
    long long off = al(mixed_ws_len(n));
    double **slots[3] = {b ? b->in : nullptr, b ? b->mid : nullptr, b ? b->vout : nullptr};
    if (b) {
        b->Xs = base + off;
        b->Ghi = base + off + 8 * B;
        b->Glo = base + off + 9 * B;
        b->Gc = base + off + 10 * B;
    }
    off += 11 * B;
    for (int k = 0; k < 3; k++)
        for (int s = 0; s < 2; s++) {
            if (b) slots[k][s] = base + off;
            off += CB;
        }
    return off;
}

static int ooc_leaf(int m, int n, int mt, double *Ah, int lda, double *T, int ldt, double *Qh, int ldq,
                    int rows_per_chunk, double *work, long long lwork)
{
    const int C = ooc_rows(m, n, rows_per_chunk);
    OocBufs b;
    ooc_layout(n, C, work, &b);
    MixedWs w = carve(work, mixed_ws_len(n));
    const long long B = 64 * 64;
    const int nch = (int)(((long long)m + C - 1) / C);
    const double shift_factor = leaf_shift_factor(m, n);
    cudaStream_t st = stream(), s_in = nullptr, s_out = nullptr;
    cudaEvent_t ev_in[2], ev_free[2], ev_done[2], ev_small;
    if (cudaStreamCreateWithFlags(&s_in, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s_out, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        if (s_in) cudaStreamDestroy(s_in);
        return -100;
    }
    for (int k = 0; k < 2; k++) {
        cudaEventCreateWithFlags(&ev_in[k], cudaEventDisableTiming);
        cudaEventCreateWithFlags(&ev_free[k], cudaEventDisableTiming);
        cudaEventCreateWithFlags(&ev_done[k], cudaEventDisableTiming);
        cudaEventRecord(ev_free[k], st);
    }
    cudaEventCreateWithFlags(&ev_small, cudaEventDisableTiming);
    auto rows_of = [&](int c) { return (int)std::min<long long>(C, (long long)m - (long long)c * C); };
    // a copy the runtime refuses (e.g. a host pointer it cannot reach) fails the call
    cudaError_t copy_err = cudaSuccess;
    auto chk = [&](cudaError_t e) {
        if (e != cudaSuccess && copy_err == cudaSuccess) copy_err = e;
    };
    // chunk c into slot s once the slot's previous chunk is done with
    auto load = [&](int c, int s) {
        cudaStreamWaitEvent(s_in, ev_free[s], 0);
        chk(cudaMemcpy2DAsync(b.in[s], (size_t)C * 8, Ah + (size_t)c * C, (size_t)lda * 8, (size_t)rows_of(c) * 8,
                              n, cudaMemcpyDefault, s_in));
        cudaEventRecord(ev_in[s], s_in);
    };
    // the candidate A X_0 .. X_{nx-1} of the chunk in slot s
    auto chain = [&](int s, int rows, int nx) {
        double *cur = b.in[s], *oth = b.mid[s];
        for (int p = 0; p < nx; p++) {
            ozaki_map(rows, n, cur, C, b.Xs + p * B, n, n, oth, C);
            std::swap(cur, oth);
        }
        return cur;
    };
    set2d(n, n, 0.0, 1.0, w.R, n, 0);
    trace_begin();
    k_pass_init<<<1, 1, 0, st>>>(w.ctl);
    note_launch("pass_init");
    // here the host drives the passes (each pass streams A through the
    // device once), reading the device's decision after every pass
    PassCtl ps{};
    ps.active = 1;
    int nx = 0;
    while (ps.active) {
        set2d(n, n, 0.0, 0.0, b.Ghi, n, 0);
        set2d(n, n, 0.0, 0.0, b.Glo, n, 0);
        load(0, 0);
        for (int c = 0; c < nch; c++) {
            const int s = c & 1;
            if (c + 1 < nch) load(c + 1, s ^ 1);
            cudaStreamWaitEvent(st, ev_in[s], 0);
            double *cur = chain(s, rows_of(c), nx);
            ozaki_gram(rows_of(c), n, cur, C, b.Gc, n, w.oz, w.ozlen, 0, false);
            k_twosum_acc<<<(n * n + 255) / 256, 256, 0, st>>>(n * n, b.Gc, b.Ghi, b.Glo);
            note_launch("twosum_acc");
            cudaEventRecord(ev_free[s], st);
        }
        k_twosum_fin<<<(n * n + 255) / 256, 256, 0, st>>>(n * n, b.Ghi, b.Glo, w.G);
        note_launch("twosum_fin");
        factor_pass_dev(n, w, w.ctl, 0, shift_factor);
        cudaMemcpyAsync(&ps, w.ctl, sizeof ps, cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) break;
        if (ps.active) copy2d(n, n, w.X, n, b.Xs + nx++ * B, n);
    }
    trace_begin();
    k_keep_ctl<<<1, 1, 0, st>>>(w.ctl);
    note_launch("pass_keep");
    // top n rows of the final factor (chunk 0 holds them: C >= n), then the
    // reconstruction on n x n data
    load(0, 0);
    cudaStreamWaitEvent(st, ev_in[0], 0);
    double *cur0 = chain(0, rows_of(0), nx);
    gemm(n, n, n, opnd(cur0, C), opnd(w.X, n, NT, M_UPPER), w.Qt, n, ep(1, 0));
    cudaEventRecord(ev_free[0], st);
    reconstruct_small(n, 0, mt, w, T, ldt);
    // V rows into A (below the top n rows) and Q, chunk by chunk
    load(0, 0);
    for (int c = 0; c < nch; c++) {
        const int s = c & 1, rows = rows_of(c), skip = c == 0 ? n : 0;
        if (c + 1 < nch) load(c + 1, s ^ 1);
        cudaStreamWaitEvent(st, ev_in[s], 0);
        double *cur = chain(s, rows, nx);
        double *qout = cur == b.in[s] ? b.mid[s] : b.in[s];
        if (rows > skip) ozaki_map(rows - skip, n, cur + skip, C, w.MV, n, n, b.vout[s], C);
        ozaki_map(rows, n, cur, C, w.MQ, n, n, qout, C);
        cudaEventRecord(ev_done[s], st);
        cudaStreamWaitEvent(s_out, ev_done[s], 0);
        const size_t r0 = (size_t)c * C;
        if (rows > skip)
            chk(cudaMemcpy2DAsync(Ah + r0 + skip, (size_t)lda * 8, b.vout[s], (size_t)C * 8,
                                  (size_t)(rows - skip) * 8, n, cudaMemcpyDefault, s_out));
        chk(cudaMemcpy2DAsync(Qh + r0, (size_t)ldq * 8, qout, (size_t)C * 8, (size_t)rows * 8, n,
                              cudaMemcpyDefault, s_out));
        cudaEventRecord(ev_free[s], s_out);
    }
    // the top block of A (S R above the diagonal, L below)
    cudaEventRecord(ev_small, st);
    cudaStreamWaitEvent(s_out, ev_small, 0);
    chk(cudaMemcpy2DAsync(Ah, (size_t)lda * 8, w.Atop, (size_t)n * 8, (size_t)n * 8, n, cudaMemcpyDefault, s_out));
    cudaEventRecord(ev_small, s_out);
    cudaStreamWaitEvent(st, ev_small, 0);
    const cudaError_t e = cudaStreamSynchronize(st);
    for (int k = 0; k < 2; k++) {
        cudaEventDestroy(ev_in[k]);
        cudaEventDestroy(ev_free[k]);
        cudaEventDestroy(ev_done[k]);
    }
    cudaEventDestroy(ev_small);
    cudaStreamDestroy(s_in);
    cudaStreamDestroy(s_out);
    return (e == cudaSuccess && copy_err == cudaSuccess) ? 0 : -100;
}

int mixed_leaf_entry(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt, double *Q, int ldq,
                     double *work, long long lwork, int variant)
{
    return mixed_leaf(m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork, variant);
}

}  // namespace lg

using namespace lg;

extern "C" {

int lila_query_dgeqrf_w03_mt_hr_mixed(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                                      double *Q, int ldq, double *work, int lwork)
{
    long long v = need_mixed_leaf_full(m - i, n);
    return v > 0x7fffffffLL ? 0x7fffffff : (int)v;
}

int lila_dgeqrf_w03_mt_hr_mixed_v(int variant, int m, int n, int i, int mt, double *A, int lda, double *T,
                                  int ldt, double *Q, int ldq, double *work, int lwork)
{
    if (variant < 0 || variant > 2) return -1;
    if (m < 0) return -2;
    if (n < 0 || n > 64 || i + n > m) return -3;
    if (i < 0) return -4;
    if (mt <= 0) return -5;
    if (lda < (m > 1 ? m : 1)) return -7;
    if (ldt < mt) return -9;
    if (ldq < (m > 1 ? m : 1)) return -11;
    if (lwork < need_mixed_leaf(n)) return -13;
    if (n == 0) return 0;
    return graph_call("mt_hr_mixed",
                      {(long long)variant, (long long)m, (long long)n, (long long)i, (long long)mt,
                       (long long)(uintptr_t)A, (long long)lda, (long long)(uintptr_t)T, (long long)ldt,
                       (long long)(uintptr_t)Q, (long long)ldq, (long long)(uintptr_t)work, (long long)lwork},
                      [&] { return mixed_leaf(m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork, variant); });
}

int lila_dgeqrf_w03_mt_hr_mixed(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt, double *Q,
                                int ldq, double *work, int lwork)
{
    int e = lila_dgeqrf_w03_mt_hr_mixed_v(0, m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork);
    return e < 0 ? e + 1 : e;
}

long long lila_gpu_query_dgeqrf_tall_host(int m, int n, int rows_per_chunk)
{
    if (m < 1 || n < 1 || n > 64 || m < n) return 0;
    return ooc_layout(n, ooc_rows(m, n, rows_per_chunk), nullptr, nullptr);
}

int lila_gpu_dgeqrf_tall_host(int m, int n, int mt, double *A, int lda, double *T, int ldt, double *Q, int ldq,
                              int rows_per_chunk, double *work, long long lwork)
{
    if (m < 0) return -1;
    if (n < 0 || n > 64 || n > m) return -2;
    if (mt <= 0) return -3;
    if (!A && m) return -4;
    if (lda < (m > 1 ? m : 1)) return -5;
    if (!T && n) return -6;
    if (ldt < mt) return -7;
    if (!Q && m) return -8;
    if (ldq < (m > 1 ? m : 1)) return -9;
    if (rows_per_chunk < 0) return -10;
    if (n == 0) return 0;
    if (!work || lwork < lila_gpu_query_dgeqrf_tall_host(m, n, rows_per_chunk)) return -12;
    return ooc_leaf(m, n, mt, A, lda, T, ldt, Q, ldq, rows_per_chunk, work, lwork);
}

int lila_prim_rsqrt(int n, const double *d, double *out)
{
    if (n < 0) return -1;
    if (n == 0) return 0;
    if (!d) return -2;
    if (!out) return -3;
    trace_begin();
    k_rsqrt_nr<<<(n + 255) / 256, 256, 0, stream()>>>(n, d, out);
    note_launch("rsqrt_nr");
    return cudaGetLastError() == cudaSuccess ? 0 : -100;
}

int lila_prim_factor_pass(int n, const double *G, int ldg, double *Rk, int ldk, double *X, int ldx, int variant,
                          double shift_factor, double cond_limit)
{
    if (n < 1 || n > 64) return -1;
    if (!G) return -2;
    if (ldg < n) return -3;
    if (!Rk) return -4;
    if (ldk < n) return -5;
    if (!X) return -6;
    if (ldx < n) return -7;
    if (variant < 0 || variant > 2) return -8;
    PassCtl *c = nullptr;
    if (cudaGetSymbolAddress((void **)&c, d_prim_ctl) != cudaSuccess) return -100;
    factor_pass_attr();
    trace_begin();
    k_pass_init<<<1, 1, 0, stream()>>>(c);
    note_launch("pass_init");
    trace_begin();
    k_factor_pass<<<1, FP_NT, FP_SMEM, stream()>>>(n, G, ldg, Rk, ldk, X, ldx, c, variant, shift_factor, cond_limit,
                                                   status_ptr());
    note_launch("factor_pass");
    PassCtl h{};
    if (cudaMemcpyFromSymbolAsync(&h, d_prim_ctl, sizeof h, 0, cudaMemcpyDeviceToHost, stream()) != cudaSuccess ||
        cudaStreamSynchronize(stream()) != cudaSuccess)
        return -100;
    return h.shifted_passes ? 1 : 0;
}

int lila_gpu_last_variant(void) { return last_ctl().shifted_passes ? 2 : 1; }
int lila_gpu_last_passes(void) { return last_ctl().passes; }
int lila_gpu_last_fallback(void) { return g_last_fallback; }

int lila_gpu_set_check(int level)
{
    const int prev = g_check_level;
    if (level >= 0 && level <= 2) g_check_level = level;
    return prev;
}

int lila_gpu_last_check(double *res, double *orth)
{
    if (res) *res = g_last_check[0];
    if (orth) *orth = g_last_check[1];
    return g_last_check[0] < 0.0 ? -1 : 0;
}

}  // extern "C"
