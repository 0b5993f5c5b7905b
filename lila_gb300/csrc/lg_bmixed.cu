// lg_bmixed.cu -- batched least squares with split-precision Cholesky QR
// variants, per-instance routing and a checked fallback to FP64 Householder.
//
// Variants (chosen per instance by the caller, e.g. the learned selector):
//   0  Cholesky QR 2 with FP64-grade tensor-core products
//   1  shifted Cholesky QR 3 (a shifted first pass, then Cholesky QR 2)
//   2  FP64 Householder (the persistent batched solver of lg_batched.cu)
// Variants 0/1 need n <= 128, n + nrhs <= 136 and m >= 2n (other instances
// go to variant 2 whatever their route).  Every pass is one grouped
// split-precision GEMM launch over all routed instances (lg_ozgemm.cu) plus
// one small FP64 kernel per instance for the n x n work.  The variants only
// read A and B until the final step: the formed factors live in scratch
// blocks [Q | b] (m x (n + nrhs)), whose Gram gives Q^T Q and Q^T b together.
// The last Cholesky pass is implicit (least squares needs Q^T b, not Q), and
// its factor's orthogonality ||I - X^T G X||_F (G the FP64-grade Gram, X the
// inverse of its Cholesky factor) is measured on the device, its two n x n
// products as grouped split-precision GEMMs.  The solution x = X1 [X2] X y
// (each pass's inverse kept) is written to B(0:n, :) only when no Cholesky
// broke down and the orthogonality is at most 50 n 2^-53; other instances are
// re-solved by variant 2 from their untouched A and B (or, with
// LILA_GELS_NO_FALLBACK, left as they are).
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "lg_common.cuh"
#include "../../include/lila_gpu.h"

namespace lg {

constexpr int BM_LD = 136;  // leading dimension of the per-instance (n + nrhs)^2 blocks
constexpr int BM_NMAX = 128;  // largest n of the mixed variants

struct BMInst {
    int m, n, lda, ldb;
    double *A, *B;
    double *Q1, *Q2;    // scratch m x (n + nrhs) each, ld m
    double *G, *X1, *X2;  // BM_LD x BM_LD: Gram, inverses of the factors of passes 1 and 2
    int *colexp;        // BM_LD column scales of the current Gram
    int *xcexp;         // BM_LD column scales of X
    int *rexp;          // m row scales of the current map's left operand
};

// Per-instance flags of a solve (any nonzero flag sends the instance to the
// FP64 fallback).
enum BMFlag : int {
    FL_BREAKDOWN = 1,        // a Cholesky of an explicit pass broke down
    FL_CHECK = 2,            // the orthogonality check failed
    FL_FINAL_BREAKDOWN = 4,  // the Cholesky of the last (implicit) pass broke down
};

namespace bm {

constexpr int NT = 256;

// Packed upper storage of an n x n triangle in shared memory: column c holds
// rows 0..c contiguously, so a column is one contiguous run and a 128 x 128
// triangle takes 66 KB (three CTAs per SM instead of one for the full square).
__device__ __forceinline__ int pk(int r, int c) { return ((c * (c + 1)) >> 1) + r; }
static inline size_t packed_bytes(int n) { return (size_t)n * (n + 1) / 2 * sizeof(double); }

__device__ __forceinline__ double warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Upper Cholesky of the packed n x n S in place, right-looking with the
// pivot one step ahead (as the tall leaf's factor pass): in step j warp 0
// applies row j of R to row j + 1, takes that row's pivot (its 1 / sqrt by
// rsqrt_nr) and scales the row, while the warps of the other three SM
// sub-partitions (warp % 4 != 0) apply row j to rows j + 2 .. n - 1, one
// element of the trailing triangle per thread and step; a step ends with one
// block barrier.  False on a non-positive pivot (the pivot is then replaced
// by 1 so that the factor stays finite).
__device__ bool chol_packed(int n, double *S)
{
    __shared__ int bad;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    // warp 0: row j of S, already updated by rows 0 .. j - 1, in v (columns
    // j + lane + 32 q), factored and scaled
    auto pivot_row = [&](int j, const double (&v)[4]) {
        double d = __shfl_sync(0xffffffffu, v[0], 0);
        if (!(d > 0.0) || !isfinite(d)) {
            if (lane == 0) bad = 1;
            d = 1.0;
        }
        const double y = rsqrt_nr(d);
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int c = j + lane + 32 * q;
            if (c < n) S[pk(j, c)] = c == j ? d * y : v[q] * y;
        }
    };
    if (warp == 0) {
        double v[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int c = lane + 32 * q;
            v[q] = c < n ? S[pk(0, c)] : 0.0;
        }
        pivot_row(0, v);
    }
    __syncthreads();
    for (int j = 0; j + 1 < n; j++) {
        if (warp == 0) {
            // row j + 1 -= R(j, j + 1) R(j, :)
            const double a = S[pk(j, j + 1)];
            double v[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int c = j + 1 + lane + 32 * q;
                v[q] = c < n ? fma(-a, S[pk(j, c)], S[pk(j + 1, c)]) : 0.0;
            }
            pivot_row(j + 1, v);
        } else if (warp & 3) {
            // rows p = j + 2 .. n - 1: element e = cc (cc + 1) / 2 + q of the
            // trailing upper triangle (columns cc = 0 .. w - 1, rows q <= cc, offset j + 2)
            const int wid = warp - (warp >> 2) - 1;  // 0 .. 5
            const int w = n - j - 2, tot = w * (w + 1) / 2;
            for (int e = wid * 32 + lane; e < tot; e += 192) {
                int cc = (int)((sqrtf(8.0f * e + 1.0f) - 1.0f) * 0.5f);
                if (cc * (cc + 1) / 2 > e) cc--;
                if ((cc + 1) * (cc + 2) / 2 <= e) cc++;
                const int p = j + 2 + e - cc * (cc + 1) / 2;
                const int c = cc + j + 2;
                S[pk(p, c)] = fma(-S[pk(j, p)], S[pk(j, c)], S[pk(p, c)]);
            }
        }
        __syncthreads();
    }
    return bad == 0;
}

// S := S^-1 in place for the packed upper n x n S (n <= 128; column j from
// the already inverted leading block, as LAPACK's dtrti2:
// X(r, j) = -(sum_{p=r}^{j-1} X(r, p) R(p, j)) / R(j, j)).  The reciprocals
// of the diagonal are formed once into the shared rd (BM_LD doubles) and
// written over the diagonal first; two lanes share each row's dot product
// (even and odd p, two accumulators each); the next column of R is copied
// aside while the current one is formed, so a column costs one barrier.
__device__ void tri_inv_packed(int n, double *S, double *rd)
{
    __shared__ double colb[2][BM_LD];
    for (int r = threadIdx.x; r < n; r += NT) rd[r] = 1.0 / S[pk(r, r)];
    if (threadIdx.x == 0 && n > 1) colb[1][0] = S[pk(0, 1)];
    __syncthreads();
    for (int r = threadIdx.x; r < n; r += NT) S[pk(r, r)] = rd[r];
    __syncthreads();
    const int r = threadIdx.x >> 1, hb = threadIdx.x & 1;
    for (int j = 1; j < n; j++) {
        const double *cj = colb[j & 1];
        double v0 = 0.0, v1 = 0.0;
        if (r < j) {
            int p = r + hb;
            for (; p + 2 < j; p += 4) {
                v0 = fma(S[pk(r, p)], cj[p], v0);
                v1 = fma(S[pk(r, p + 2)], cj[p + 2], v1);
            }
            if (p < j) v0 = fma(S[pk(r, p)], cj[p], v0);
        }
        double v = v0 + v1;
        v += __shfl_xor_sync(0xffffffffu, v, 1);
        if (r < j && hb == 0) S[pk(r, j)] = -rd[j] * v;
        if (j + 1 < n)
            for (int q = threadIdx.x; q <= j; q += NT) colb[(j + 1) & 1][q] = S[pk(q, j + 1)];
        __syncthreads();
    }
}

// Packed upper S <- I (a broken-down instance continues on finite values;
// its flag already sends it to the fallback).
__device__ void identity_packed(int n, double *S)
{
    for (int c = threadIdx.x >> 5; c < n; c += NT / 32)
        for (int r = threadIdx.x & 31; r <= c; r += 32) S[pk(r, c)] = r == c ? 1.0 : 0.0;
    __syncthreads();
}

// The largest column 1-norm of the packed upper n x n S, in every thread
// (infinite when a column sum is not finite).
__device__ double max_col_abs_sum(int n, const double *S)
{
    __shared__ double red[NT / 32];
    double mx = 0.0;
    for (int c = threadIdx.x >> 5; c < n; c += NT / 32) {
        double v = 0.0;
        for (int r = threadIdx.x & 31; r <= c; r += 32) v += fabs(S[pk(r, c)]);
        v = warp_sum(v);
        mx = (v <= 1.7976931348623157e308) ? fmax(mx, v) : INFINITY;
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    double r = 0.0;
    for (int w = 0; w < NT / 32; w++) r = fmax(r, red[w]);
    __syncthreads();
    return r;
}

// Packed upper S <- the upper triangle of the n x n block at G (ld BM_LD).
__device__ void load_packed(int n, const double *G, double *S)
{
    for (int c = threadIdx.x >> 5; c < n; c += NT / 32)
        for (int r = threadIdx.x & 31; r <= c; r += 32) S[pk(r, c)] = G[r + BM_LD * c];
}

// Upper triangle of the packed S -> D (ld BM_LD); the strict lower part of
// D(0:n, 0:n) is zeroed when `zero_lower`.
__device__ void store_packed(int n, const double *S, double *D, int ldd, bool zero_lower)
{
    for (int c = threadIdx.x >> 5; c < n; c += NT / 32)
        for (int r = threadIdx.x & 31; r < n; r += 32) {
            if (r <= c)
                D[r + (size_t)ldd * c] = S[pk(r, c)];
            else if (zero_lower)
                D[r + (size_t)ldd * c] = 0.0;
        }
}

// y := R^-T y (forward substitution) for the packed upper R, one right-hand
// side (ld BM_LD in y) per warp; rd holds 1 / R(r, r).
__device__ void solve_rt(int n, const double *S, const double *rd, double *y, int nrhs)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int j = warp; j < nrhs; j += NT / 32) {
        double *yj = y + BM_LD * j;
        for (int r = 0; r < n; r++) {
            const double *sr = S + pk(0, r);
            double s = 0.0;
            for (int p = lane; p < r; p += 32) s += sr[p] * yj[p];
            s = warp_sum(s);
            if (lane == 0) yj[r] = (yj[r] - s) * rd[r];
            __syncwarp();
        }
    }
}

// One factor pass: Rk = chol(G [+ shift]), X = Rk^-1 into X1 (first pass) or
// X2 (second) and the largest biased exponent of each column of X (the
// scales of the row map's right operand).  shift: 0 none, 1 the shifted
// Cholesky QR 3 shift, 2 a trial: the unshifted factor is kept when it
// exists and its 1-norm condition number ||Rk||_1 ||Rk^-1||_1 is at most
// trial_limit, else the shifted one is formed and shifted[t] set (the
// instance then needs the extra pass of shifted Cholesky QR 3).
__global__ void __launch_bounds__(NT, 3) k_factor(const BMInst *inst, const int *list, int shift, int first, int *flag,
                                                  int *shifted, double trial_limit)
{
    extern __shared__ double S[];
    __shared__ double rd[BM_LD];
    const int t = list[blockIdx.x];
    const BMInst I = inst[t];
    const int n = I.n;
    bool done = false;
    if (shift == 2) {
        load_packed(n, I.G, S);
        __syncthreads();
        if (chol_packed(n, S)) {
            const double a = max_col_abs_sum(n, S);
            tri_inv_packed(n, S, rd);
            const double b = max_col_abs_sum(n, S);
            done = a * b <= trial_limit;
        }
        __syncthreads();
        if (!done && threadIdx.x == 0) shifted[t] = 1;
    }
    if (!done) {
        load_packed(n, I.G, S);
        __syncthreads();
        if (shift && threadIdx.x == 0) {
            double tr = 0.0;
            for (int k = 0; k < n; k++) tr += S[pk(k, k)];
            // the Gram is an exact integer sum rounded once (error per entry
            // below 2^-49 sqrt(m) ||a_i|| ||a_j||), so the shift needs no
            // m n u term (the tall leaf's reasoning, lg_tsmixed.cu)
            const double sig = 11.0 * ((double)n * (n + 1) * 0x1p-53 + 0x1p-49 * sqrt((double)I.m)) * tr;
            for (int k = 0; k < n; k++) S[pk(k, k)] += sig;
        }
        __syncthreads();
        const bool ok = chol_packed(n, S);
        if (!ok && threadIdx.x == 0) flag[t] |= FL_BREAKDOWN;
        if (!ok) identity_packed(n, S);
        tri_inv_packed(n, S, rd);
    }
    double *X = first ? I.X1 : I.X2;
    for (int c = threadIdx.x >> 5; c < n; c += NT / 32) {
        int mx = 0;
        for (int r = threadIdx.x & 31; r < n; r += 32) {
            const double v = r <= c ? S[pk(r, c)] : 0.0;
            X[r + BM_LD * c] = v;
            mx = max(mx, (int)((__double_as_longlong(v) >> 52) & 0x7FF));
        }
        for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if ((threadIdx.x & 31) == 0) I.xcexp[c] = mx;
    }
}

// b -> Qf(:, n : n + nrhs), Qf = Q1 (which = 0) or Q2 (which = 1).
__global__ void k_copy_b(const BMInst *inst, const int *list, const int *which, int nrhs)
{
    const int t = list[blockIdx.x];
    const BMInst I = inst[t];
    double *Q = which[blockIdx.x] ? I.Q2 : I.Q1;
    for (int j = 0; j < nrhs; j++)
        for (int r = threadIdx.x; r < I.m; r += blockDim.x)
            Q[(size_t)r + (size_t)(I.n + j) * I.m] = I.B[(size_t)r + (size_t)j * I.ldb];
}

// The check scratch of the last pass: the unused one of Q1 / Q2 (at least
// 2n (n + nrhs) doubles since m >= 2n) holds X (n x n, ld n) then T = G X.
__host__ __device__ __forceinline__ double *check_scratch(const BMInst &I, int which) { return which ? I.Q1 : I.Q2; }

// Last pass, first half.  G = [Q b]^T [Q b] (Q = Q_k, the last formed
// factor).  Rk = chol(G(0:n, 0:n)); y = Rk^-T (Q_k^T b) over
// G(0:n, n : n + nrhs); X = Rk^-1 -> the check scratch.  The implicit Q_{k+1} = Q_k Rk^-1 has
// Q_{k+1}^T Q_{k+1} = X^T G X, which the two grouped products that follow
// form at FP64 grade: T = G X, then I - X^T T over G(0:n, 0:n).
__global__ void __launch_bounds__(NT, 3) k_final_a(const BMInst *inst, const int *list, const int *which, int nrhs,
                                                int *flag)
{
    extern __shared__ double S[];
    __shared__ double y[BM_LD * 8];
    const int t = list[blockIdx.x];
    const BMInst I = inst[t];
    const int n = I.n;
    load_packed(n, I.G, S);
    for (int idx = threadIdx.x; idx < n * nrhs; idx += NT) {
        const int r = idx % n, j = idx / n;
        y[r + BM_LD * j] = I.G[r + BM_LD * (n + j)];
    }
    __syncthreads();
    const bool ok = chol_packed(n, S);
    if (!ok && threadIdx.x == 0) flag[t] |= FL_FINAL_BREAKDOWN;
    __shared__ double rd[BM_LD];
    for (int r = threadIdx.x; r < n; r += NT) rd[r] = 1.0 / S[pk(r, r)];
    __syncthreads();
    solve_rt(n, S, rd, y, nrhs);
    __syncthreads();
    for (int idx = threadIdx.x; idx < n * nrhs; idx += NT) {
        const int r = idx % n, j = idx / n;
        I.G[r + BM_LD * (n + j)] = y[r + BM_LD * j];
    }
    if (!ok) identity_packed(n, S);
    tri_inv_packed(n, S, rd);
    store_packed(n, S, check_scratch(I, which[blockIdx.x]), n, true);
}

// y := X y for the upper n x n X (ld ldx, global) and the right-hand sides
// y (ld BM_LD, shared), every (row, right-hand side) in parallel: no
// sequential dependence, unlike a substitution.
__device__ void upper_mv(int n, const double *X, int ldx, double *y, int nrhs)
{
    double o[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
        const int idx = threadIdx.x + u * NT;
        o[u] = 0.0;
        if (idx < n * nrhs) {
            const int r = idx % n, j = idx / n;
            const double *yj = y + BM_LD * j;
            double s0 = 0.0, s1 = 0.0;
            int p = r;
            for (; p + 1 < n; p += 2) {
                s0 += X[r + (size_t)ldx * p] * yj[p];
                s1 += X[r + (size_t)ldx * (p + 1)] * yj[p + 1];
            }
            if (p < n) s0 += X[r + (size_t)ldx * p] * yj[p];
            o[u] = s0 + s1;
        }
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 4; u++) {
        const int idx = threadIdx.x + u * NT;
        if (idx < n * nrhs) y[idx % n + BM_LD * (idx / n)] = o[u];
    }
    __syncthreads();
}

// Last pass, second half.  ||E||_F with E = I - X^T G X (in G(0:n, 0:n))
// is the orthogonality of the implicit factor; it is compared with
// climit * n * 2^-53.  On success x = R^-1 y = X1 [X2] X y (R = Rk [Rk2]
// Rk1, each pass's inverse kept) is written to B(0:n, :).
__global__ void __launch_bounds__(NT, 3) k_final_b(const BMInst *inst, const int *list, const int *which, int nrhs,
                                                double climit, int *flag, double *orth)
{
    __shared__ double y[BM_LD * 8];
    __shared__ double red[NT / 32];
    __shared__ int fail;
    const int t = list[blockIdx.x];
    const BMInst I = inst[t];
    const int n = I.n;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double part = 0.0;
    for (int c = warp; c < n; c += NT / 32)
        for (int r = lane; r < n; r += 32) {
            const double e = I.G[r + BM_LD * c];
            part += e * e;
        }
    part = warp_sum(part);
    if (lane == 0) red[warp] = part;
    __syncthreads();
    if (threadIdx.x == 0) {
        double sum = 0.0;
        for (int w = 0; w < NT / 32; w++) sum += red[w];
        const double e = sqrt(sum);
        const int f0 = flag[t];
        orth[t] = (f0 & FL_FINAL_BREAKDOWN) ? -1.0 : e;
        fail = f0 ? f0 : (!(e <= climit * n * 1.1102230246251565e-16) ? FL_CHECK : 0);
        if (fail) flag[t] = fail;
    }
    __syncthreads();
    if (fail) return;
    for (int idx = threadIdx.x; idx < n * nrhs; idx += NT) {
        const int r = idx % n, j = idx / n;
        y[r + BM_LD * j] = I.G[r + BM_LD * (n + j)];
    }
    __syncthreads();
    upper_mv(n, check_scratch(I, which[blockIdx.x]), n, y, nrhs);
    if (which[blockIdx.x]) upper_mv(n, I.X2, BM_LD, y, nrhs);
    upper_mv(n, I.X1, BM_LD, y, nrhs);
    for (int idx = threadIdx.x; idx < n * nrhs; idx += NT) {
        const int r = idx % n, j = idx / n;
        I.B[(size_t)r + (size_t)j * I.ldb] = y[r + BM_LD * j];
    }
}

}  // namespace bm

// ---------------------------------------------------------------------------
// Selector features, FP32 outputs, n <= 128 (one CTA per instance at a time):
//   f0 log2(m) / 12, f1 log2(n) / 7,
//   f2 log10(max / min column norm) / 4 (clipped to 4),
//   f3 log10 of the 1-norm condition number of the FP64 Householder R of an
//      s x n sparse sign sketch C A, s = min(2n, 176) (C: row r of A goes to
//      bucket h(r) mod s with sign s(r), so C A costs m n additions),
//      divided by 10 and clipped to 2 (2 also for an exactly singular R),
//   f4 log10(max / min pivot) / 3 of the FP32 Cholesky of A^T A
//      (2 when the FP32 factorization breaks down).
// A dense Gaussian sketch would cost 2 m n^2 FP64 flops, as much as the FP64
// solve itself; the sparse sketch keeps the estimate in FP64 (it must resolve
// condition numbers up to 1e16) at the cost of one pass over A.
// ---------------------------------------------------------------------------
namespace feat {

constexpr int NT = 256, LDC = 132, CH2 = 16, LD2 = 130, SMAX = 176, NB = 8;

// Shared memory of one size class (n <= nmax): the sketch (ld sld, odd so
// that threads reading consecutive columns hit distinct banks; later the
// FP32 Gram, ld nmax), a CH2-row FP64 chunk of A (later the block
// reflector's W, 2 NB x nmax) and the same chunk in FP32 (ld LDC).
__host__ __device__ inline int sketch_ld(int nmax) { return (min(2 * nmax, SMAX)) | 1; }
__host__ __device__ inline size_t smem_bytes(int nmax)
{
    return (size_t)sketch_ld(nmax) * nmax * 8 + (size_t)CH2 * LD2 * 8 + (size_t)CH2 * LDC * 4;
}

__device__ __forceinline__ uint32_t mix32(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7FEB352Du;
    x ^= x >> 15;
    x *= 0x846CA68Bu;
    x ^= x >> 16;
    return x;
}

__device__ __forceinline__ void tile_of(int blk, int &bi, int &bj)
{
    bj = (int)((sqrtf(8.0f * blk + 1.0f) - 1.0f) * 0.5f);
    while (bj * (bj + 1) / 2 > blk) bj--;
    while ((bj + 1) * (bj + 2) / 2 <= blk) bj++;
    bi = blk - bj * (bj + 1) / 2;
}

__device__ __forceinline__ double wsum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Householder QR (LAPACK dgeqrf conventions, tau = 0 for a zero column below
// the diagonal) of the ns x nn matrix S (ld sld) in shared memory, in panels
// of NB columns: each panel is factored column by column, then its block
// reflector I - V T V^T (T from V^T V by the dlarft recurrence) is applied
// to the trailing columns: W = V^T C (two threads per column, row halves),
// W = T^T W, C -= V W (one thread per element).  R is left in the upper
// triangle.  Wp needs 2 NB nn doubles.
__device__ void house_qr(int ns, int nn, double *S, int sld, double *Wp)
{
    __shared__ double s_tau[NB], s_T[NB * NB], s_G[NB * NB];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int j0 = 0; j0 < nn; j0 += NB) {
        const int jb = min(NB, nn - j0);
        for (int k = j0; k < j0 + jb; k++) {
            double *ck = S + (size_t)sld * k;
            if (warp == 0) {
                double ss = 0.0;
                for (int r = k + 1 + lane; r < ns; r += 32) ss += ck[r] * ck[r];
                ss = wsum(ss);
                const double alpha = ck[k];
                double tau = 0.0, sc = 0.0, beta = alpha;
                if (ss > 0.0) {
                    beta = -copysign(sqrt(alpha * alpha + ss), alpha);
                    tau = (beta - alpha) / beta;
                    sc = 1.0 / (alpha - beta);
                }
                if (tau != 0.0)
                    for (int r = k + 1 + lane; r < ns; r += 32) ck[r] *= sc;
                __syncwarp();
                if (lane == 0) {
                    ck[k] = beta;
                    s_tau[k - j0] = tau;
                }
            }
            __syncthreads();
            const double tau = s_tau[k - j0];
            const int c = k + 1 + warp;
            if (tau != 0.0 && c < j0 + jb) {
                double *cc = S + (size_t)sld * c;
                double d = 0.0;
                for (int r = k + 1 + lane; r < ns; r += 32) d += ck[r] * cc[r];
                const double w = tau * (cc[k] + wsum(d));
                for (int r = k + 1 + lane; r < ns; r += 32) cc[r] -= w * ck[r];
                __syncwarp();
                if (lane == 0) cc[k] -= w;
            }
            __syncthreads();
        }
        const int c0 = j0 + jb, nc = nn - c0;
        if (nc <= 0) break;
        // G(a, b) = v_a^T v_b, a < b (v_a: 1 at row j0 + a, S below, 0 above)
        for (int q = warp; q < jb * jb; q += NT / 32) {
            const int a = q % jb, b = q / jb;
            if (a >= b) continue;
            const double *va = S + (size_t)sld * (j0 + a), *vb = S + (size_t)sld * (j0 + b);
            double d = 0.0;
            for (int r = j0 + b + 1 + lane; r < ns; r += 32) d += va[r] * vb[r];
            d = wsum(d);
            if (lane == 0) s_G[a + NB * b] = d + va[j0 + b];
        }
        __syncthreads();
        if (tid == 0) {
            for (int i = 0; i < jb; i++) {
                const double ti = s_tau[i];
                for (int r = 0; r < i; r++) {
                    double x = 0.0;
                    for (int p = r; p < i; p++) x += s_T[r + NB * p] * s_G[p + NB * i];
                    s_T[r + NB * i] = -ti * x;
                }
                s_T[i + NB * i] = ti;
            }
        }
        // W = V^T C: thread (c, half) sums rows of its half
        const int rows = ns - j0, hrows = (rows + 1) >> 1;
        if (tid < 2 * nc) {
            const int cl = tid % nc, hf = tid / nc;
            const double *cc = S + (size_t)sld * (c0 + cl);
            double acc[NB];
#pragma unroll
            for (int i = 0; i < NB; i++) acc[i] = 0.0;
            const int r1 = min(ns, j0 + (hf + 1) * hrows);
            for (int r = j0 + hf * hrows; r < r1; r++) {
                const double x = cc[r];
#pragma unroll
                for (int i = 0; i < NB; i++) {
                    if (i < jb) {
                        const int d = j0 + i;
                        const double v = r > d ? S[r + (size_t)sld * d] : (r == d ? 1.0 : 0.0);
                        acc[i] += v * x;
                    }
                }
            }
#pragma unroll
            for (int i = 0; i < NB; i++) Wp[(hf * NB + i) * nn + cl] = acc[i];
        }
        __syncthreads();
        // W := T^T W (both halves summed)
        if (tid < nc) {
            double w[NB];
#pragma unroll
            for (int i = 0; i < NB; i++) w[i] = Wp[i * nn + tid] + Wp[(NB + i) * nn + tid];
#pragma unroll
            for (int i = NB - 1; i >= 0; i--) {
                double x = 0.0;
#pragma unroll
                for (int p = 0; p <= i; p++) x += s_T[p + NB * i] * w[p];
                if (i < jb) Wp[i * nn + tid] = x;
            }
        }
        __syncthreads();
        // C -= V W, four elements per thread at a time (independent chains)
        const int tot = rows * nc;
        for (int base = tid; base < tot; base += 4 * NT) {
            int rr[4], cl[4];
            double x[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int idx = min(base + u * NT, tot - 1);
                rr[u] = j0 + idx % rows;
                cl[u] = idx / rows;
                x[u] = 0.0;
            }
#pragma unroll
            for (int i = 0; i < NB; i++) {
                if (i < jb) {
                    const int d = j0 + i;
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        const double v = rr[u] > d ? S[rr[u] + (size_t)sld * d] : (rr[u] == d ? 1.0 : 0.0);
                        x[u] += v * Wp[i * nn + cl[u]];
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < 4; u++)
                if (base + u * NT < tot) S[rr[u] + (size_t)sld * (c0 + cl[u])] -= x[u];
        }
        __syncthreads();
    }
}

// The instances list[0 .. cnt), all with n <= nmax, one CTA per instance at a
// time.  One pass over A in CH2-row chunks (the next chunk is loaded into
// registers while the current one is used) feeds both the FP32 Gram (4 x 4
// register tiles) and the FP64 sketch.  The FP32 Gram is parked in the
// instance's Gram block (as floats, ld nmax) while the sketch is factored,
// then read back for the FP32 Cholesky.
__global__ void __launch_bounds__(NT, 2) k_features(const BMInst *inst, const int *list, int cnt, int nmax, float *F)
{
    extern __shared__ __align__(16) uint8_t fsm[];
    __shared__ double red[NT], red2[NT];
    __shared__ int bad;
    const int sld = sketch_ld(nmax);
    const int tid = threadIdx.x;
    double *SA = (double *)fsm;
    double *c64 = SA + (size_t)sld * nmax;
    float *c32 = (float *)(c64 + CH2 * LD2);
    for (int li = blockIdx.x; li < cnt; li += gridDim.x) {
        const int t = list[li];
        const BMInst I = inst[t];
        const int mm = I.m, nn = I.n, ns = min(2 * nn, SMAX);
        const int nb = (nn + 3) >> 2, nblk = nb * (nb + 1) / 2;
        const int chunk = CH2 * nn;
        float acc[3][16];
#pragma unroll
        for (int q = 0; q < 3; q++)
#pragma unroll
            for (int e = 0; e < 16; e++) acc[q][e] = 0.0f;
        for (int idx = tid; idx < sld * nn; idx += NT) SA[idx] = 0.0;
        for (int idx = tid; idx < CH2 * LDC; idx += NT) c32[idx] = 0.0f;  // columns >= nn stay zero
        double pf[8];
        auto load = [&](int r0) {
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const int idx = tid + k * NT;
                const int r = idx % CH2, c = idx / CH2;
                pf[k] = (idx < chunk && r0 + r < mm) ? I.A[(size_t)(r0 + r) + (size_t)c * I.lda] : 0.0;
            }
        };
        load(0);
        for (int r0 = 0; r0 < mm; r0 += CH2) {
            __syncthreads();
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const int idx = tid + k * NT;
                if (idx < chunk) {
                    const int r = idx % CH2, c = idx / CH2;
                    c64[r * LD2 + c] = pf[k];
                    c32[r * LDC + c] = (float)pf[k];
                }
            }
            __syncthreads();
            if (r0 + CH2 < mm) load(r0 + CH2);
#pragma unroll
            for (int q = 0; q < 3; q++) {
                const int blk = tid + q * NT;
                if (blk < nblk) {
                    int bi, bj;
                    tile_of(blk, bi, bj);
#pragma unroll 4
                    for (int r = 0; r < CH2; r++) {
                        const float4 x = *(const float4 *)(c32 + r * LDC + 4 * bi);
                        const float4 y = *(const float4 *)(c32 + r * LDC + 4 * bj);
                        const float xs[4] = {x.x, x.y, x.z, x.w}, ys[4] = {y.x, y.y, y.z, y.w};
#pragma unroll
                        for (int a = 0; a < 4; a++)
#pragma unroll
                            for (int b = 0; b < 4; b++) acc[q][4 * a + b] = fmaf(xs[a], ys[b], acc[q][4 * a + b]);
                    }
                }
            }
            if (tid < nn) {
                const int c = tid;
                for (int r = 0; r < CH2 && r0 + r < mm; r++) {
                    const uint32_t h = mix32((uint32_t)(r0 + r) * 0x9E3779B9u + 0x3C6EF372u);
                    const int b = (int)((h >> 1) % (uint32_t)ns);
                    const double v = c64[r * LD2 + c];
                    SA[b + sld * c] += (h & 1u) ? v : -v;
                }
            }
        }
        // park the FP32 Gram in the instance's Gram block
        float *Gp = (float *)I.G;
#pragma unroll
        for (int q = 0; q < 3; q++) {
            const int blk = tid + q * NT;
            if (blk < nblk) {
                int bi, bj;
                tile_of(blk, bi, bj);
#pragma unroll
                for (int a = 0; a < 4; a++)
#pragma unroll
                    for (int b = 0; b < 4; b++) {
                        const int i = 4 * bi + a, j = 4 * bj + b;
                        if (i < nn && j < nn) Gp[i + nmax * j] = acc[q][4 * a + b];
                    }
            }
        }
        __syncthreads();
        // ---- the sketch's R and its 1-norm condition number
        house_qr(ns, nn, SA, sld, c64);
        // ||R||_1 (column sums), then R^-1 in place (column j from the already
        // inverted leading block, as dtrti2 does) and ||R^-1||_1
        double cr = 0.0;
        for (int c = threadIdx.x; c < nn; c += NT) {
            double sum = 0.0;
            for (int r = 0; r <= c; r++) sum += fabs(SA[r + sld * c]);
            cr = fmax(cr, sum);
        }
        // R^-1 as bm::tri_inv_packed does it (one barrier per column, two
        // lanes per row, the reciprocals of the diagonal formed once), unless
        // a diagonal entry is zero or not finite
        __shared__ double colb[2][128], rdg[128];
        __shared__ int sing;
        if (threadIdx.x == 0) sing = 0;
        __syncthreads();
        for (int r = threadIdx.x; r < nn; r += NT) {
            const double d = SA[r + sld * r];
            if (d == 0.0 || !isfinite(d)) sing = 1;
            rdg[r] = 1.0 / d;
        }
        if (threadIdx.x == 0 && nn > 1) colb[1][0] = SA[sld];
        __syncthreads();
        if (!sing) {
            for (int r = threadIdx.x; r < nn; r += NT) SA[r + sld * r] = rdg[r];
            __syncthreads();
            const int r = threadIdx.x >> 1, hb = threadIdx.x & 1;
            for (int j = 1; j < nn; j++) {
                const double *cj = colb[j & 1];
                double v0 = 0.0, v1 = 0.0;
                if (r < j) {
                    int p = r + hb;
                    for (; p + 2 < j; p += 4) {
                        v0 = fma(SA[r + sld * p], cj[p], v0);
                        v1 = fma(SA[r + sld * (p + 2)], cj[p + 2], v1);
                    }
                    if (p < j) v0 = fma(SA[r + sld * p], cj[p], v0);
                }
                double v = v0 + v1;
                v += __shfl_xor_sync(0xffffffffu, v, 1);
                if (r < j && hb == 0) SA[r + sld * j] = -rdg[j] * v;
                if (j + 1 < nn)
                    for (int q = threadIdx.x; q <= j; q += NT) colb[(j + 1) & 1][q] = SA[q + sld * (j + 1)];
                __syncthreads();
            }
        }
        __syncthreads();
        double ci = 0.0;
        for (int c = threadIdx.x; c < nn; c += NT) {
            double sum = 0.0;
            for (int r = 0; r <= c; r++) sum += fabs(SA[r + sld * c]);
            ci = fmax(ci, sum);
        }
        if (sing || !(ci <= 1e300)) ci = INFINITY;  // singular R: no finite estimate
        red[threadIdx.x] = cr;
        red2[threadIdx.x] = ci;
        __syncthreads();
        for (int o = NT / 2; o > 0; o >>= 1) {
            if (threadIdx.x < o) {
                red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + o]);
                red2[threadIdx.x] = fmax(red2[threadIdx.x], red2[threadIdx.x + o]);
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            const double k1 = red[0] * red2[0];
            F[5 * t + 3] = (isfinite(k1) ? (float)fmin(log10(fmax(k1, 1.0)), 20.0) : 20.0f) / 10.0f;
        }
        __syncthreads();
        // ---- the FP32 Gram back (upper triangle, ld nmax): norms and FP32 Cholesky
        float *G = (float *)fsm;
        const int ldg = nmax;
        for (int c = tid >> 5; c < nn; c += NT / 32)
            for (int r = tid & 31; r <= c; r += 32) G[r + ldg * c] = Gp[r + nmax * c];
        __syncthreads();
        if (tid == 0) {
            float mx = 0.0f, mn = 3.4e38f;
            for (int j = 0; j < nn; j++) {
                const float v = sqrtf(fmaxf(G[j + ldg * j], 0.0f));
                mx = fmaxf(mx, v);
                mn = fminf(mn, v);
            }
            F[5 * t + 0] = log2f((float)mm) / 12.0f;
            F[5 * t + 1] = log2f((float)nn) / 7.0f;
            F[5 * t + 2] = mn > 0.0f ? fminf(log10f(mx / mn) / 4.0f, 4.0f) : 4.0f;
            bad = 0;
        }
        __syncthreads();
        for (int j = 0; j < nn; j++) {
            if (tid < 32) {
                float d = 0.0f;
                for (int p = tid; p < j; p += 32) d += G[p + ldg * j] * G[p + ldg * j];
                for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
                if (tid == 0) {
                    d = G[j + ldg * j] - d;
                    if (!(d > 0.0f))
                        bad = 1;
                    else
                        G[j + ldg * j] = sqrtf(d);
                }
            }
            __syncthreads();
            if (bad) break;
            const float dj = G[j + ldg * j];
            for (int c = j + 1 + tid; c < nn; c += NT) {
                float v = G[j + ldg * c];
                for (int p = 0; p < j; p++) v -= G[p + ldg * j] * G[p + ldg * c];
                G[j + ldg * c] = v / dj;
            }
            __syncthreads();
        }
        if (tid == 0) {
            float f4 = 2.0f;
            if (!bad) {
                float mx = 0.0f, mn = 3.4e38f;
                for (int j = 0; j < nn; j++) {
                    mx = fmaxf(mx, G[j + ldg * j]);
                    mn = fminf(mn, G[j + ldg * j]);
                }
                f4 = fminf(log10f(mx / mn) / 3.0f, 2.0f);
            }
            F[5 * t + 4] = f4;
        }
        __syncthreads();
    }
}

}  // namespace feat

struct BMHandle {
    int count, nrhs;
    std::vector<BMInst> h;
    BMInst *d_inst;
    int *d_list, *d_which, *d_flag;
    int *d_shifted;            // per instance: the trial factor of the last run chose the shift
    int *h_shifted;            // pinned host copy of d_shifted
    cudaEvent_t ev_shifted;    // recorded after the copy
    std::vector<int> shifted;  // the last run's trial choices (host)
    double trial_limit;        // condition limit of the trial factor
    OzGroup *d_groups;
    GramW *d_gjobs;
    RowExpJob *d_rjobs;
    int *d_prefix;
    int2 *d_tilemap;  // grouped GEMM tile table (tilemap_len entries)
    long long tilemap_len;
    MapItem *d_items;  // row-map work items (2 per instance at most)
    int *d_counter;
    double *d_orth;
    float *d_F;     // selector inputs, count x 5
    int *d_choice;  // selector output
    void *fp64_work;  // metadata of the FP64 Householder solver
    long long fp64_bytes;
    void *mem;
};

static size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// The mixed variants take n <= 128 (n + nrhs <= 136) and m >= 2n: the
// orthogonality check keeps X and T (2 n^2 doubles) in the instance's unused
// m x (n + nrhs) factor block.
static bool eligible(int m, int n, int nrhs) { return n <= BM_NMAX && n + nrhs <= BM_LD && m >= 2 * n; }

// One grouped Gram pass: instance list[k]'s matrix src(I) = {pointer, ld,
// columns}; G(0:min(cols,128), 0:cols) into I.G.
struct GramSrc {
    const double *p;
    int ld, cols;
};
// Uploads Gram jobs, the diagonal blocks computed from their own 64 columns
// first (see ozaki_grams), and launches them.
static void launch_grams(BMHandle *H, const std::vector<GramW> &jobs)
{
    if (jobs.empty()) return;
    std::vector<GramW> ordered;
    ordered.reserve(jobs.size());
    auto stacked = [](const GramW &j) { return (j.half == 0 && j.n <= 64) || j.half == 1; };
    for (const GramW &j : jobs)
        if (stacked(j)) ordered.push_back(j);
    const int ns = (int)ordered.size();
    for (const GramW &j : jobs)
        if (!stacked(j)) ordered.push_back(j);
    cudaMemcpyAsync(H->d_gjobs, ordered.data(), sizeof(GramW) * ordered.size(), cudaMemcpyHostToDevice, stream());
    ozaki_grams(H->d_gjobs, (int)ordered.size(), ns);
}

template <class F>
static void gram_pass(BMHandle *H, const std::vector<int> &list, F src)
{
    std::vector<GramW> jobs;
    jobs.reserve(list.size() * 2);
    for (int t : list) {
        const BMInst &I = H->h[t];
        const GramSrc g = src(I);
        for (int hf = 0; hf * 64 < g.cols; hf++)
            jobs.push_back(GramW{g.p, g.ld, I.m, g.cols, I.colexp, I.G, BM_LD, hf});
    }
    launch_grams(H, jobs);
}

// One grouped split-precision pass over the listed instances; make(t) gives
// instance t's product.
template <class F>
static void grouped_pass(BMHandle *H, const std::vector<int> &list, F make)
{
    const int n = (int)list.size();
    if (!n) return;
    std::vector<OzGroup> g(n);
    std::vector<int> pre(n + 1, 0);
    for (int k = 0; k < n; k++) {
        g[k] = make(H->h[list[k]]);
        pre[k + 1] = pre[k] + ozgemm_group_tiles(g[k].M, g[k].N);
    }
    cudaStream_t st = stream();
    cudaMemcpyAsync(H->d_groups, g.data(), sizeof(OzGroup) * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(H->d_prefix, pre.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, st);
    if (pre[n] > H->tilemap_len) return;  // cannot happen: sized for the largest pass at create
    ozgemm_groups(H->d_groups, H->d_prefix, n, pre[n], H->d_tilemap);
}

template <class F>
static void row_pass(BMHandle *H, const std::vector<int> &list, F make)
{
    const int n = (int)list.size();
    if (!n) return;
    std::vector<RowExpJob> j(n);
    for (int k = 0; k < n; k++) j[k] = make(H->h[list[k]]);
    cudaMemcpyAsync(H->d_rjobs, j.data(), sizeof(RowExpJob) * n, cudaMemcpyHostToDevice, stream());
    row_exponents(H->d_rjobs, n);
}

// One row-map pass over the listed instances: out = src X (X upper
// triangular, n x n), one work item per instance and 64-column block, the
// largest first.  src(I) gives {A, lda}, X(I) and out(I) (ld m) the rest.
template <class F>
static void map_pass(BMHandle *H, const std::vector<int> &list, F make)
{
    std::vector<MapItem> items;
    items.reserve(list.size() * 2);
    for (int t : list) {
        const BMInst &I = H->h[t];
        for (int c0 = 0; c0 < I.n; c0 += 64) {
            MapItem it = make(I);
            it.col0 = c0;
            it.ncols = std::min(64, I.n - c0);
            it.kend = std::min(I.n, c0 + 64);
            items.push_back(it);
        }
    }
    if (items.empty()) return;
    auto cost = [](const MapItem &it) { return (long long)((it.m + 127) / 128) * ((it.kend + 15) / 16); };
    std::stable_sort(items.begin(), items.end(), [&](const MapItem &a, const MapItem &b) { return cost(a) > cost(b); });
    cudaMemcpyAsync(H->d_items, items.data(), sizeof(MapItem) * items.size(), cudaMemcpyHostToDevice, stream());
    map_items(H->d_items, (int)items.size(), H->d_counter);
}

static MapItem map_item(const double *A, int lda, int m, const double *X, double *out, const int *rexp, const int *cexp)
{
    MapItem it;
    it.A = A;
    it.lda = lda;
    it.m = m;
    it.X = X;
    it.ldx = BM_LD;
    it.col0 = 0;
    it.ncols = 0;
    it.kend = 0;
    it.out = out;
    it.ldo = m;
    it.rexp = rexp;
    it.cexp = cexp;
    return it;
}


}  // namespace lg

namespace lg {
// Enqueues the mixed variants for the listed instances: g0 by Cholesky QR 2,
// g1 by shifted Cholesky QR 3 (flags and orthogonality left on the device).
// Default 1-norm condition number of the trial factor up to which an
// instance routed to Cholesky QR 2 keeps it.  Cholesky QR 2 passes its check
// up to kappa ~ 10^8.7; an unshifted factor of a Gram whose kappa is beyond
// 1/sqrt(u) saturates, and on 20,000 instances (kappa to 1e15, n <= 128)
// its estimate stayed above 3e8 but not always above 1e9.  1e8 keeps a
// factor of three below the lowest saturated value seen.
constexpr double kTrialLimit = 1e8;

// The passes of the mixed variants over g0 (Cholesky QR 2) and g1 (shifted
// Cholesky QR 3).  With `trial`, the first factor of a g0 instance is a trial
// (k_factor, shift 2): an instance whose trial chose the shift continues as
// shifted Cholesky QR 3 (its host flag is read back while the first row map
// runs).
static void mixed_passes(BMHandle *H, std::vector<int> g0, std::vector<int> g1, bool trial)
{
    const int count = H->count, nrhs = H->nrhs;
    cudaStream_t st = lg::stream();
    // the per-instance FP64 kernels run per size class (packed triangles of
    // n <= 32, 64, 96, 128), so small instances get more CTAs per SM
    auto cls = [&](int t) { const int nn = H->h[t].n; return nn <= 32 ? 0 : nn <= 64 ? 1 : nn <= 96 ? 2 : 3; };
    auto by_cls = [&](std::vector<int> &v) {
        std::stable_sort(v.begin(), v.end(), [&](int a, int b) { return cls(a) < cls(b); });
    };
    by_cls(g0);
    by_cls(g1);
    std::vector<int> mixed(g1);
    mixed.insert(mixed.end(), g0.begin(), g0.end());
    const int nm = (int)mixed.size();
    int n1 = (int)g1.size();
    const bool tried = trial && n1 < nm;
    // launch f(offset, count, smem) for every run of one size class in mixed[beg, end)
    auto per_class = [&](int beg, int end, auto f) {
        for (int a = beg; a < end;) {
            int b = a;
            while (b < end && cls(mixed[b]) == cls(mixed[a])) b++;
            f(a, b - a, bm::packed_bytes(32 * (cls(mixed[a]) + 1)));
            a = b;
        }
    };
    if (nm > 0) {
        const int smax = (int)bm::packed_bytes(BM_NMAX);
        cudaFuncSetAttribute(bm::k_factor, cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
        cudaFuncSetAttribute(bm::k_final_a, cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
        cudaMemcpyAsync(H->d_list, mixed.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, st);
        auto factor = [&](int beg, int end, int shift, int first) {
            per_class(beg, end, [&](int off, int cnt, size_t sm) {
                trace_begin();
                bm::k_factor<<<cnt, bm::NT, sm, st>>>(H->d_inst, H->d_list + off, shift, first, H->d_flag,
                                                      H->d_shifted, H->trial_limit);
                note_launch("bm_factor");
            });
        };
        // pass 1: G = A^T A; Rk = chol (shifted for group 1, listed first;
        // a trial for group 0 when `trial`); Q1 = A Rk^-1
        if (tried) cudaMemsetAsync(H->d_shifted, 0, sizeof(int) * count, st);
        gram_pass(H, mixed, [](const BMInst &I) { return GramSrc{I.A, I.lda, I.n}; });
        factor(0, n1, 1, 1);
        factor(n1, nm, tried ? 2 : 0, 1);
        if (tried) {
            cudaMemcpyAsync(H->h_shifted, H->d_shifted, sizeof(int) * count, cudaMemcpyDeviceToHost, st);
            cudaEventRecord(H->ev_shifted, st);
        }
        row_pass(H, mixed, [](const BMInst &I) { return RowExpJob{I.A, I.lda, I.m, I.n, I.rexp}; });
        map_pass(H, mixed, [](const BMInst &I) { return map_item(I.A, I.lda, I.m, I.X1, I.Q1, I.rexp, I.xcexp); });
        if (tried) {
            // instances whose trial chose the shift join group 1 for its second pass
            cudaEventSynchronize(H->ev_shifted);
            std::vector<int> keep;
            for (int t : g0) {
                H->shifted[t] = H->h_shifted[t];
                if (H->h_shifted[t])
                    g1.push_back(t);
                else
                    keep.push_back(t);
            }
            if ((int)g1.size() != n1) {
                g0.swap(keep);
                by_cls(g1);
                mixed.assign(g1.begin(), g1.end());
                mixed.insert(mixed.end(), g0.begin(), g0.end());
                n1 = (int)g1.size();
                cudaMemcpyAsync(H->d_list, mixed.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, st);
            }
        }
        // group 1: one more explicit pass, Q2 = Q1 Rk^-1
        if (n1) {
            gram_pass(H, g1, [](const BMInst &I) { return GramSrc{I.Q1, I.m, I.n}; });
            factor(0, n1, 0, 0);
            row_pass(H, g1, [](const BMInst &I) { return RowExpJob{I.Q1, I.m, I.m, I.n, I.rexp}; });
            map_pass(H, g1, [](const BMInst &I) { return map_item(I.Q1, I.m, I.m, I.X2, I.Q2, I.rexp, I.xcexp); });
        }
        // last pass on [Qf | b]: Qf = Q2 for group 1, Q1 for group 0
        std::vector<int> which(nm, 0);
        for (int k = 0; k < n1; k++) which[k] = 1;
        cudaMemcpyAsync(H->d_which, which.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, st);
        trace_begin();
        bm::k_copy_b<<<nm, 256, 0, st>>>(H->d_inst, H->d_list, H->d_which, nrhs);
        note_launch("bm_copy_b");
        {
            std::vector<GramW> jobs;
            for (int k = 0; k < nm; k++) {
                const BMInst &I = H->h[mixed[k]];
                const int cols = I.n + nrhs;
                for (int hf = 0; hf * 64 < cols; hf++)
                    jobs.push_back(GramW{which[k] ? I.Q2 : I.Q1, I.m, I.m, cols, I.colexp, I.G, BM_LD, hf});
            }
            launch_grams(H, jobs);
        }
        per_class(0, nm, [&](int off, int cnt, size_t sm) {
            trace_begin();
            bm::k_final_a<<<cnt, bm::NT, sm, st>>>(H->d_inst, H->d_list + off, H->d_which + off, nrhs, H->d_flag);
            note_launch("bm_final_a");
        });
        // the orthogonality check's products: T = G X, then I - X^T T over G(0:n, 0:n)
        std::vector<int> wof(count, 0);
        for (int k = 0; k < nm; k++) wof[mixed[k]] = which[k];
        grouped_pass(H, mixed, [&](const BMInst &I) {
            OzGroup g;
            double *Xs = bm::check_scratch(I, wof[&I - H->h.data()]);
            g.A = opnd(I.G, BM_LD, NT);
            g.B = opnd(Xs, I.n, NT, M_UPPER);
            g.C = Xs + (size_t)I.n * I.n;
            g.ldc = I.n;
            g.M = g.N = g.K = I.n;
            g.e = GemmEpi();
            g.rexp = g.cexp = nullptr;
            return g;
        });
        grouped_pass(H, mixed, [&](const BMInst &I) {
            OzGroup g;
            double *Xs = bm::check_scratch(I, wof[&I - H->h.data()]);
            g.A = opnd(Xs, I.n, TR, M_UPPER);
            g.B = opnd(Xs + (size_t)I.n * I.n, I.n, NT);
            g.C = I.G;
            g.ldc = BM_LD;
            g.M = g.N = g.K = I.n;
            g.e = GemmEpi();
            g.e.alpha = -1.0;
            g.e.add_diag = 1;
            g.rexp = g.cexp = nullptr;
            return g;
        });
        per_class(0, nm, [&](int off, int cnt, size_t sm) {
            trace_begin();
            (void)sm;
            bm::k_final_b<<<cnt, bm::NT, 0, st>>>(H->d_inst, H->d_list + off, H->d_which + off, nrhs, 50.0,
                                                   H->d_flag, H->d_orth);
            note_launch("bm_final_b");
        });
    }
}

}  // namespace lg

using namespace lg;

extern "C" {

void *lila_gels_mixed_create(int count, const int *m, const int *n, int nrhs, double *const *A, const int *lda,
                             double *const *B, const int *ldb)
{
    if (count <= 0 || nrhs < 1 || nrhs > 8) return nullptr;
    for (int t = 0; t < count; t++)
        if (m[t] < n[t] || n[t] < 1 || lda[t] < m[t] || ldb[t] < m[t]) return nullptr;
    BMHandle *H = new BMHandle();
    H->count = count;
    H->nrhs = nrhs;
    H->h.resize(count);
    // one device allocation: per instance Q1, Q2 (m x (n + nrhs)) for the
    // instances the mixed variants can take, G, R, X (BM_LD^2 each), then the
    // per-call metadata and the FP64 solver's description
    size_t bytes = 0;
    std::vector<size_t> qoff(count, 0), soff(count, 0);
    for (int t = 0; t < count; t++) {
        if (!eligible(m[t], n[t], nrhs)) continue;
        qoff[t] = bytes;
        bytes += align_up((size_t)m[t] * (n[t] + nrhs) * sizeof(double), 256) * 2;
    }
    for (int t = 0; t < count; t++) {
        if (!eligible(m[t], n[t], nrhs)) continue;
        soff[t] = bytes;
        bytes += 3 * (size_t)BM_LD * BM_LD * sizeof(double) + 2 * align_up(BM_LD * sizeof(int), 256) +
                 align_up((size_t)m[t] * sizeof(int), 256);
    }
    // tiles of the largest grouped pass: a row map (m x n) or a check product (n x n) per instance
    long long tiles = 0;
    for (int t = 0; t < count; t++)
        if (eligible(m[t], n[t], nrhs)) tiles += std::max(ozgemm_group_tiles(m[t], n[t]), ozgemm_group_tiles(n[t], n[t]));
    H->tilemap_len = tiles;
    const size_t meta_off = bytes;
    bytes += align_up(sizeof(int2) * (size_t)(tiles + 1), 256) + align_up(sizeof(MapItem) * 2 * (size_t)count, 256) +
             256 +
             align_up(sizeof(BMInst) * count, 256) + 5 * align_up(sizeof(int) * (count + 1), 256) +
             align_up(sizeof(OzGroup) * count, 256) + align_up(sizeof(GramW) * 3 * count, 256) +
             align_up(sizeof(RowExpJob) * count, 256) +
             align_up(sizeof(double) * count, 256) +
             align_up(sizeof(float) * 5 * count, 256);
    const size_t fp64_off = align_up(bytes, 256);
    H->fp64_bytes = lila_query_dgels_batched(count);
    bytes = fp64_off + (size_t)H->fp64_bytes;
    if (cudaMalloc(&H->mem, bytes) != cudaSuccess) {
        cudaGetLastError();
        delete H;
        return nullptr;
    }
    uint8_t *base = (uint8_t *)H->mem;
    for (int t = 0; t < count; t++) {
        BMInst &I = H->h[t];
        I.m = m[t];
        I.n = n[t];
        I.lda = lda[t];
        I.ldb = ldb[t];
        I.A = A[t];
        I.B = B[t];
        if (eligible(m[t], n[t], nrhs)) {
            const size_t qb = align_up((size_t)m[t] * (n[t] + nrhs) * sizeof(double), 256);
            I.Q1 = (double *)(base + qoff[t]);
            I.Q2 = (double *)(base + qoff[t] + qb);
            I.G = (double *)(base + soff[t]);
            I.X1 = I.G + BM_LD * BM_LD;
            I.X2 = I.X1 + BM_LD * BM_LD;
            I.colexp = (int *)(I.X2 + BM_LD * BM_LD);
            I.xcexp = (int *)((uint8_t *)I.colexp + align_up(BM_LD * sizeof(int), 256));
            I.rexp = (int *)((uint8_t *)I.xcexp + align_up(BM_LD * sizeof(int), 256));
        } else {
            I.Q1 = I.Q2 = I.G = I.X1 = I.X2 = nullptr;
            I.colexp = I.xcexp = I.rexp = nullptr;
        }
    }
    uint8_t *mp = base + meta_off;
    auto carve = [&](size_t sz) {
        uint8_t *r = mp;
        mp += align_up(sz, 256);
        return r;
    };
    H->d_inst = (BMInst *)carve(sizeof(BMInst) * count);
    H->d_list = (int *)carve(sizeof(int) * (count + 1));
    H->d_which = (int *)carve(sizeof(int) * (count + 1));
    H->d_flag = (int *)carve(sizeof(int) * (count + 1));
    H->d_prefix = (int *)carve(sizeof(int) * (count + 1));
    H->d_shifted = (int *)carve(sizeof(int) * (count + 1));
    H->d_groups = (OzGroup *)carve(sizeof(OzGroup) * count);
    H->d_gjobs = (GramW *)carve(sizeof(GramW) * 3 * count);
    H->d_rjobs = (RowExpJob *)carve(sizeof(RowExpJob) * count);
    H->d_tilemap = (int2 *)carve(sizeof(int2) * (size_t)(tiles + 1));
    H->d_items = (MapItem *)carve(sizeof(MapItem) * 2 * (size_t)count);
    H->d_counter = (int *)carve(sizeof(int));
    H->d_orth = (double *)carve(sizeof(double) * count);
    H->d_F = (float *)carve(sizeof(float) * 5 * count);
    H->d_choice = (int *)H->d_which;  // the selector's choices are read before any pass uses d_which
    H->fp64_work = base + fp64_off;
    H->shifted.assign(count, 0);
    H->trial_limit = kTrialLimit;
    if (cudaMallocHost(&H->h_shifted, sizeof(int) * count) != cudaSuccess ||
        cudaEventCreateWithFlags(&H->ev_shifted, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        if (H->h_shifted) cudaFreeHost(H->h_shifted);
        cudaFree(H->mem);
        delete H;
        return nullptr;
    }
    cudaMemcpy(H->d_inst, H->h.data(), sizeof(BMInst) * count, cudaMemcpyHostToDevice);
    return H;
}

int lila_gels_mixed_destroy(void *handle)
{
    BMHandle *H = (BMHandle *)handle;
    if (!H) return 0;
    cudaStreamSynchronize(lg::stream());
    cudaFree(H->mem);
    cudaFreeHost(H->h_shifted);
    cudaEventDestroy(H->ev_shifted);
    delete H;
    return 0;
}

int lila_gels_mixed_set_trial_limit(void *handle, double limit)
{
    BMHandle *H = (BMHandle *)handle;
    if (!H || !(limit > 0.0)) return -1;
    H->trial_limit = limit;
    return 0;
}

int lila_gels_mixed_shifted(void *handle, int *shifted)
{
    BMHandle *H = (BMHandle *)handle;
    if (!H) return -1;
    int c = 0;
    for (int t = 0; t < H->count; t++) {
        if (shifted) shifted[t] = H->shifted[t];
        c += H->shifted[t];
    }
    return c;
}

int lila_gels_mixed_run(void *handle, const int *route, int flags, int *info_host, double *orth_host)
{
    BMHandle *H = (BMHandle *)handle;
    if (!H) return -1;
    const int count = H->count, nrhs = H->nrhs;
    cudaStream_t st = lg::stream();
    std::vector<int> g0, g1, g2;
    for (int t = 0; t < count; t++) {
        int r = route[t];
        if ((r == 0 || r == 1) && !eligible(H->h[t].m, H->h[t].n, nrhs)) r = 2;
        (r == 0 ? g0 : r == 1 ? g1 : g2).push_back(t);
    }
    std::vector<int> mixed(g1);
    mixed.insert(mixed.end(), g0.begin(), g0.end());
    const int nm = (int)mixed.size();
    cudaMemsetAsync(H->d_flag, 0, sizeof(int) * count, st);
    std::fill(H->shifted.begin(), H->shifted.end(), 0);
    mixed_passes(H, g0, g1, !(flags & LILA_GELS_NO_TRIAL));
    std::vector<int> flag(count, 0);
    std::vector<double> orth(count, 0.0);
    cudaMemcpyAsync(flag.data(), H->d_flag, sizeof(int) * count, cudaMemcpyDeviceToHost, st);
    if (nm > 0) cudaMemcpyAsync(orth.data(), H->d_orth, sizeof(double) * count, cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return -3;
    std::vector<int> fp64(g2);
    int fallbacks = 0;
    for (int t = 0; t < count; t++) {
        info_host[t] = 0;
        if (orth_host) orth_host[t] = -2.0;
    }
    // instances whose Cholesky QR 2 failed get shifted Cholesky QR 3 first
    // (one more small grouped pass; not those the trial already sent through
    // it); only what fails again goes to FP64
    std::vector<int> retry;
    if (!(flags & LILA_GELS_NO_FALLBACK))
        for (int t : g0)
            if (flag[t] && !H->shifted[t]) retry.push_back(t);
    std::vector<int> flag2(flag);
    if (!retry.empty()) {
        for (int t : retry) flag2[t] = 0;
        cudaMemcpyAsync(H->d_flag, flag2.data(), sizeof(int) * count, cudaMemcpyHostToDevice, st);
        mixed_passes(H, std::vector<int>(), retry, false);
        cudaMemcpyAsync(flag2.data(), H->d_flag, sizeof(int) * count, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(orth.data(), H->d_orth, sizeof(double) * count, cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) return -3;
    }
    for (int t : mixed) {
        // the orthogonality of the variant that produced the solution (or failed last)
        const int f = flag2[t];
        if (orth_host) orth_host[t] = (f & (FL_BREAKDOWN | FL_FINAL_BREAKDOWN)) ? -1.0 : orth[t];
        if (flag[t]) {
            info_host[t] = 1;  // the routed variant failed its check
            fallbacks++;
        }
        if (f && !(flags & LILA_GELS_NO_FALLBACK)) fp64.push_back(t);
    }
    if (!fp64.empty()) {
        const int nf = (int)fp64.size();
        std::vector<int> fm(nf), fn(nf), fla(nf), flb(nf);
        std::vector<double *> fA(nf), fB(nf);
        for (int k = 0; k < nf; k++) {
            const BMInst &I = H->h[fp64[k]];
            fm[k] = I.m;
            fn[k] = I.n;
            fla[k] = I.lda;
            flb[k] = I.ldb;
            fA[k] = I.A;
            fB[k] = I.B;
        }
        int rc = lila_dgels_batched_prepare(nf, fm.data(), fn.data(), nrhs, fA.data(), fla.data(), fB.data(),
                                            flb.data(), H->fp64_work, H->fp64_bytes);
        if (rc != 0) return -2;
        int *d_info = H->d_flag;  // reused as the FP64 path's info (indices of the subset)
        lila_dgels_batched_run(nf, nrhs, H->fp64_work, d_info);
        std::vector<int> inf(nf);
        cudaMemcpyAsync(inf.data(), d_info, sizeof(int) * nf, cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        for (int k = 0; k < nf; k++)
            if (inf[k]) info_host[fp64[k]] = -inf[k];
    }
    return fallbacks;
}

int lila_gels_mixed_features(void *handle, float *F)
{
    BMHandle *H = (BMHandle *)handle;
    if (!H) return -1;
    // instances the mixed variants cannot take keep zero features (the
    // solve routes them to the FP64 solver whatever the selector says); the
    // others run one launch per size class (n <= 32, 64, 96, 128) with that
    // class's shared memory, so that small instances share an SM
    cudaStream_t st = lg::stream();
    cudaMemsetAsync(F, 0, sizeof(float) * 5 * (size_t)H->count, st);
    std::vector<int> order;
    for (int t = 0; t < H->count; t++)
        if (eligible(H->h[t].m, H->h[t].n, H->nrhs)) order.push_back(t);
    const int ne = (int)order.size();
    if (ne == 0) return 0;
    auto cls = [&](int t) { return (H->h[t].n - 1) >> 5; };
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cls(a) < cls(b); });
    cudaMemcpyAsync(H->d_list, order.data(), sizeof(int) * ne, cudaMemcpyHostToDevice, st);
    cudaFuncSetAttribute(feat::k_features, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)feat::smem_bytes(BM_NMAX));
    for (int a = 0; a < ne;) {
        int b = a;
        while (b < ne && cls(order[b]) == cls(order[a])) b++;
        const int nmax = 32 * (cls(order[a]) + 1);
        const size_t sm = feat::smem_bytes(nmax);
        int per_sm = 1;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, feat::k_features, feat::NT, sm) != cudaSuccess ||
            per_sm < 1) {
            cudaGetLastError();
            per_sm = 1;
        }
        const int grid = std::min(b - a, per_sm * sm_count());
        trace_begin();
        feat::k_features<<<grid, feat::NT, sm, st>>>(H->d_inst, H->d_list + a, b - a, nmax, F);
        note_launch("gels_features");
        a = b;
    }
    return 0;
}

// Features -> selector -> routed solve.  route_out (host, may be NULL) gets
// the variant the selector picked for each instance (2 where the instance is
// not eligible for the mixed variants).
int lila_gels_mixed_solve(void *handle, const float *params, int flags, int *info, double *orth, int *route_out)
{
    BMHandle *H = (BMHandle *)handle;
    if (!H) return -1;
    if (!params) return -2;
    const int count = H->count;
    if (lila_gels_mixed_features(handle, H->d_F) != 0) return -1;
    lila_sel_infer(count, params, H->d_F, nullptr, H->d_choice);
    std::vector<int> route(count);
    cudaStream_t st = lg::stream();
    cudaMemcpyAsync(route.data(), H->d_choice, sizeof(int) * count, cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return -3;
    for (int t = 0; t < count; t++) {
        if (!eligible(H->h[t].m, H->h[t].n, H->nrhs)) route[t] = 2;
        if (route_out) route_out[t] = route[t];
    }
    return lila_gels_mixed_run(handle, route.data(), flags, info, orth);
}

}  // extern "C"
