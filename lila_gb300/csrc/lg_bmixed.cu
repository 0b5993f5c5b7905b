// lg_bmixed.cu -- batched least squares with split-precision Cholesky QR
// variants, per-instance routing and a checked fallback to FP64 Householder.
//
// Variants (chosen per instance by the caller, e.g. the learned selector):
//   0  Cholesky QR 2 with FP64-grade tensor-core products
//   1  shifted Cholesky QR 3 (a shifted first pass, then Cholesky QR 2)
//   2  FP64 Householder (the persistent batched solver of lg_batched.cu)
// Variants 0/1 need n + nrhs <= 64.  They only read A and B until the final
// step: the formed factor lives in a scratch block [Q | b] (m x 64), whose
// Gram gives Q^T Q and Q^T b together.  The last Cholesky pass is implicit
// (least squares needs Q^T b, not Q), and its factor's orthogonality is
// measured on the device from that Gram.  The solution is written to
// B(0:n, :) only when no Cholesky broke down and the orthogonality is at most
// 50 n 2^-53; other instances are re-solved by variant 2 from their
// untouched A and B (or, with LILA_GELS_NO_FALLBACK, left as they are).
#include <math.h>
#include <stdint.h>

#include <vector>

#include "lg_common.cuh"
#include "../../include/lila_gpu.h"

namespace lg {

struct BMInst {
    int m, n, lda, ldb;
    double *A, *B;
    double *Q;          // scratch m x 64, ld m
    double *G, *R, *X;  // 64 x 64, ld 64
    int *colexp;        // 64
    long long *partial; // 8192
};

namespace bm {

constexpr int NT = 128;

// Upper Cholesky of the n x n leading block of S (ld 64) in shared memory;
// returns false on a non-positive pivot.
__device__ bool chol_smem(int n, double *S)
{
    __shared__ int bad;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    for (int j = 0; j < n; j++) {
        if (threadIdx.x == 0) {
            double d = S[j + 64 * j];
            for (int p = 0; p < j; p++) d -= S[p + 64 * j] * S[p + 64 * j];
            if (!(d > 0.0) || !isfinite(d)) {
                bad = 1;
                d = 1.0;
            }
            S[j + 64 * j] = sqrt(d);
        }
        __syncthreads();
        const double dj = S[j + 64 * j];
        for (int c = j + 1 + threadIdx.x; c < n; c += NT) {
            double t = S[j + 64 * c];
            for (int p = 0; p < j; p++) t -= S[p + 64 * j] * S[p + 64 * c];
            S[j + 64 * c] = t / dj;
        }
        __syncthreads();
    }
    for (int idx = threadIdx.x; idx < 64 * 64; idx += NT) {
        const int r = idx & 63, c = idx >> 6;
        if (r > c || r >= n || c >= n) S[idx] = 0.0;
    }
    __syncthreads();
    return bad == 0;
}

// X = R^-1 (upper, n x n, ld 64), one column per thread.
__device__ void tri_inv_smem(int n, const double *R, double *X)
{
    for (int idx = threadIdx.x; idx < 64 * 64; idx += NT) X[idx] = 0.0;
    __syncthreads();
    for (int c = threadIdx.x; c < n; c += NT) {
        X[c + 64 * c] = 1.0 / R[c + 64 * c];
        for (int r = c - 1; r >= 0; r--) {
            double s = 0.0;
            for (int p = r + 1; p <= c; p++) s += R[r + 64 * p] * X[p + 64 * c];
            X[r + 64 * c] = -s / R[r + 64 * r];
        }
    }
    __syncthreads();
}

// C = A B for upper triangular n x n A, B (ld 64) into C (C may not alias).
__device__ void trmm_uu(int n, const double *A, const double *B, double *C)
{
    for (int idx = threadIdx.x; idx < 64 * 64; idx += NT) {
        const int r = idx & 63, c = idx >> 6;
        double s = 0.0;
        if (r < n && c < n && r <= c)
            for (int p = r; p <= c; p++) s += A[r + 64 * p] * B[p + 64 * c];
        C[idx] = s;
    }
    __syncthreads();
}

// One factor pass: Rk = chol(G [+ shift]), X = Rk^-1, R = Rk R (or Rk).
__global__ void __launch_bounds__(NT) k_factor(const BMInst *inst, const int *list, int cnt, int shift, int first,
                                               int *flag)
{
    extern __shared__ double sm[];
    double *S = sm, *Xs = sm + 4096, *Rs = sm + 8192, *Cs = sm + 12288;
    const int t = list[blockIdx.x];
    const BMInst I = inst[t];
    const int n = I.n;
    for (int idx = threadIdx.x; idx < 4096; idx += NT) S[idx] = I.G[idx];
    __syncthreads();
    if (shift && threadIdx.x == 0) {
        double tr = 0.0;
        for (int k = 0; k < n; k++) tr += S[k + 64 * k];
        const double sig = 11.0 * ((double)I.m * n + (double)n * (n + 1)) * 1.1102230246251565e-16 * tr;
        for (int k = 0; k < n; k++) S[k + 64 * k] += sig;
    }
    __syncthreads();
    const bool ok = chol_smem(n, S);
    if (!ok && threadIdx.x == 0) flag[t] = 1;
    tri_inv_smem(n, S, Xs);
    if (first) {
        for (int idx = threadIdx.x; idx < 4096; idx += NT) Rs[idx] = S[idx];
    } else {
        for (int idx = threadIdx.x; idx < 4096; idx += NT) Cs[idx] = I.R[idx];
        __syncthreads();
        trmm_uu(n, S, Cs, Rs);
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < 4096; idx += NT) {
        I.X[idx] = Xs[idx];
        I.R[idx] = Rs[idx];
    }
}

// b -> Q(:, n : n + nrhs)
__global__ void k_copy_b(const BMInst *inst, const int *list, int cnt, int nrhs)
{
    const int t = list[blockIdx.x];
    const BMInst I = inst[t];
    for (int j = 0; j < nrhs; j++)
        for (int r = threadIdx.x; r < I.m; r += blockDim.x)
            I.Q[(size_t)r + (size_t)(I.n + j) * I.m] = I.B[(size_t)r + (size_t)j * I.ldb];
}

// Last pass: G = [Q b]^T [Q b] (Q = Q_k, the last formed factor).
// Rk = chol(G(0:n,0:n)), X = Rk^-1; the factor the solve uses is the implicit
// Q_{k+1} = Q_k X, whose orthogonality ||I - X^T G(0:n,0:n) X||_F is measured
// here in FP64 (the Gram is FP64-grade) and compared with climit * n * 2^-53.
// On success: R = Rk R, y = X^T Q_k^T b = Q_{k+1}^T b, x = R^-1 y into B(0:n, :).
__global__ void __launch_bounds__(NT) k_final(const BMInst *inst, const int *list, int cnt, int nrhs, double climit,
                                              int *flag, double *orth)
{
    extern __shared__ double sm[];
    double *S = sm, *Xs = sm + 4096, *Rs = sm + 8192, *Cs = sm + 12288;
    __shared__ double y[64 * 8];
    __shared__ double red[NT];
    __shared__ int fail;
    const int t = list[blockIdx.x];
    const BMInst I = inst[t];
    const int n = I.n;
    for (int idx = threadIdx.x; idx < 4096; idx += NT) {
        const double g = I.G[idx];
        S[idx] = g;
        Cs[idx] = g;
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < n * nrhs; idx += NT) {
        const int r = idx % n, j = idx / n;
        y[r + 64 * j] = S[r + 64 * (n + j)];
    }
    __syncthreads();
    const bool ok = chol_smem(n, S);
    tri_inv_smem(n, S, Xs);
    // Rs = G X (G symmetric, upper part stored in Cs), then E = X^T Rs - I
    for (int idx = threadIdx.x; idx < 4096; idx += NT) {
        const int r = idx & 63, c = idx >> 6;
        double s = 0.0;
        if (r < n && c < n)
            for (int p = 0; p <= c; p++) s += Cs[(r <= p) ? r + 64 * p : p + 64 * r] * Xs[p + 64 * c];
        Rs[idx] = s;
    }
    __syncthreads();
    double part = 0.0;
    for (int idx = threadIdx.x; idx < n * n; idx += NT) {
        const int r = idx % n, c = idx / n;
        double s = 0.0;
        for (int p = 0; p <= r; p++) s += Xs[p + 64 * r] * Rs[p + 64 * c];
        const double e = s - (r == c ? 1.0 : 0.0);
        part += e * e;
    }
    red[threadIdx.x] = part;
    __syncthreads();
    for (int o = NT / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double e = sqrt(red[0]);
        orth[t] = ok ? e : -1.0;
        // an earlier pass that broke down (flag 1) fails the instance too
        fail = flag[t] ? flag[t] : ((!ok || !(e <= climit * n * 1.1102230246251565e-16)) ? 2 : 0);
        if (fail) flag[t] = fail;
    }
    for (int idx = threadIdx.x; idx < 4096; idx += NT) Cs[idx] = I.R[idx];
    __syncthreads();
    if (fail) return;
    trmm_uu(n, S, Cs, Rs);  // R = Rk R
    // y = X^T y, then x = R^-1 y
    if (threadIdx.x < nrhs) {
        double *yj = y + 64 * threadIdx.x;
        for (int r = n - 1; r >= 0; r--) {
            double s = 0.0;
            for (int p = 0; p <= r; p++) s += Xs[p + 64 * r] * yj[p];
            yj[r] = s;
        }
        for (int r = n - 1; r >= 0; r--) {
            double s = yj[r];
            for (int p = r + 1; p < n; p++) s -= Rs[r + 64 * p] * yj[p];
            yj[r] = s / Rs[r + 64 * r];
        }
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < n * nrhs; idx += NT) {
        const int r = idx % n, j = idx / n;
        I.B[(size_t)r + (size_t)j * I.ldb] = y[r + 64 * j];
    }
    for (int idx = threadIdx.x; idx < 4096; idx += NT) I.R[idx] = Rs[idx];
}

}  // namespace bm

// ---------------------------------------------------------------------------
// Selector features, FP32 outputs, n <= 128 (one CTA per instance at a time):
//   f0 log2(m) / 12, f1 log2(n) / 7,
//   f2 log10(max / min column norm) / 4 (clipped to 4),
//   f3 log10 of the 1-norm condition number of the FP64 Householder R of a
//      2n x n sparse sign sketch C A (C: row r of A goes to bucket h(r) mod 2n
//      with sign s(r), so C A costs m n additions), divided by 10 and clipped
//      to 2 (2 also for an exactly singular R, and for n > 64, where the
//      instance is not eligible for the mixed variants),
//   f4 log10(max / min pivot) / 3 of the FP32 Cholesky of A^T A
//      (2 when the FP32 factorization breaks down).
// A dense Gaussian sketch would cost 2 m n^2 FP64 flops, as much as the FP64
// solve itself; the sparse sketch keeps the estimate in FP64 (it must resolve
// condition numbers up to 1e16) at the cost of one pass over A.
// ---------------------------------------------------------------------------
namespace feat {

constexpr int NT = 256, CH = 32, LDC = 132, CH2 = 16, LD2 = 66, SLD = 128;
constexpr size_t SMEM_A = (size_t)CH * LDC * 4 + 128 * 128 * 4;
constexpr size_t SMEM_B = (size_t)SLD * 64 * 8 + (size_t)CH2 * LD2 * 8;
constexpr size_t SMEM = SMEM_A > SMEM_B ? SMEM_A : SMEM_B;

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

__global__ void __launch_bounds__(NT) k_features(const BMInst *inst, int count, float *F)
{
    extern __shared__ __align__(16) uint8_t fsm[];
    __shared__ double red[NT], red2[NT];
    __shared__ int bad;
    for (int t = blockIdx.x; t < count; t += gridDim.x) {
        const BMInst I = inst[t];
        const int mm = I.m, nn = I.n, ns = 2 * nn;
        // ---- phase A: FP32 Gram (4 x 4 register tiles), norms, FP32 Cholesky
        float *ch = (float *)fsm;
        float *G = ch + CH * LDC;  // 128 x 128, ld 128
        const int nb = (nn + 3) >> 2, nblk = nb * (nb + 1) / 2;
        float acc[3][16];
#pragma unroll
        for (int q = 0; q < 3; q++)
#pragma unroll
            for (int e = 0; e < 16; e++) acc[q][e] = 0.0f;
        for (int r0 = 0; r0 < mm; r0 += CH) {
            __syncthreads();
            for (int idx = threadIdx.x; idx < CH * LDC; idx += NT) {
                const int r = idx % CH, c = idx / CH;
                float v = 0.0f;
                if (c < nn && r0 + r < mm) v = (float)I.A[(size_t)(r0 + r) + (size_t)c * I.lda];
                ch[r * LDC + c] = v;
            }
            __syncthreads();
#pragma unroll
            for (int q = 0; q < 3; q++) {
                const int blk = threadIdx.x + q * NT;
                if (blk < nblk) {
                    int bi, bj;
                    tile_of(blk, bi, bj);
                    for (int r = 0; r < CH; r++) {
                        const float4 x = *(const float4 *)(ch + r * LDC + 4 * bi);
                        const float4 y = *(const float4 *)(ch + r * LDC + 4 * bj);
                        const float xs[4] = {x.x, x.y, x.z, x.w}, ys[4] = {y.x, y.y, y.z, y.w};
#pragma unroll
                        for (int a = 0; a < 4; a++)
#pragma unroll
                            for (int b = 0; b < 4; b++) acc[q][4 * a + b] = fmaf(xs[a], ys[b], acc[q][4 * a + b]);
                    }
                }
            }
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 3; q++) {
            const int blk = threadIdx.x + q * NT;
            if (blk < nblk) {
                int bi, bj;
                tile_of(blk, bi, bj);
#pragma unroll
                for (int a = 0; a < 4; a++)
#pragma unroll
                    for (int b = 0; b < 4; b++) {
                        const int i = 4 * bi + a, j = 4 * bj + b;
                        if (i < nn && j < nn) G[i + 128 * j] = acc[q][4 * a + b];
                    }
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            float mx = 0.0f, mn = 3.4e38f;
            for (int j = 0; j < nn; j++) {
                const float v = sqrtf(fmaxf(G[j + 128 * j], 0.0f));
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
            if (threadIdx.x == 0) {
                float d = G[j + 128 * j];
                for (int p = 0; p < j; p++) d -= G[p + 128 * j] * G[p + 128 * j];
                if (!(d > 0.0f))
                    bad = 1;
                else
                    G[j + 128 * j] = sqrtf(d);
            }
            __syncthreads();
            if (bad) break;
            const float dj = G[j + 128 * j];
            for (int c = j + 1 + threadIdx.x; c < nn; c += NT) {
                float v = G[j + 128 * c];
                for (int p = 0; p < j; p++) v -= G[p + 128 * j] * G[p + 128 * c];
                G[j + 128 * c] = v / dj;
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            float f4 = 2.0f;
            if (!bad) {
                float mx = 0.0f, mn = 3.4e38f;
                for (int j = 0; j < nn; j++) {
                    mx = fmaxf(mx, G[j + 128 * j]);
                    mn = fminf(mn, G[j + 128 * j]);
                }
                f4 = fminf(log10f(mx / mn) / 3.0f, 2.0f);
            }
            F[5 * t + 4] = f4;
            if (nn > 64) F[5 * t + 3] = 2.0f;
        }
        __syncthreads();
        if (nn > 64) continue;
        // ---- phase B: FP64 sparse sign sketch (2n x n, ld SLD) and its R
        double *SA = (double *)fsm;
        double *c64 = SA + SLD * 64;
        for (int idx = threadIdx.x; idx < SLD * 64; idx += NT) SA[idx] = 0.0;
        for (int r0 = 0; r0 < mm; r0 += CH2) {
            __syncthreads();
            for (int idx = threadIdx.x; idx < CH2 * 64; idx += NT) {
                const int r = idx % CH2, c = idx / CH2;
                double v = 0.0;
                if (c < nn && r0 + r < mm) v = I.A[(size_t)(r0 + r) + (size_t)c * I.lda];
                c64[r * LD2 + c] = v;
            }
            __syncthreads();
            if (threadIdx.x < nn) {
                const int c = threadIdx.x;
                for (int r = 0; r < CH2 && r0 + r < mm; r++) {
                    const uint32_t h = mix32((uint32_t)(r0 + r) * 0x9E3779B9u + 0x3C6EF372u);
                    const int b = (int)((h >> 1) % (uint32_t)ns);
                    const double v = c64[r * LD2 + c];
                    SA[b + SLD * c] += (h & 1u) ? v : -v;
                }
            }
        }
        __syncthreads();
        for (int k = 0; k < nn; k++) {
            double part = 0.0;
            for (int r = k + 1 + threadIdx.x; r < ns; r += NT) part += SA[r + SLD * k] * SA[r + SLD * k];
            red[threadIdx.x] = part;
            __syncthreads();
            for (int o = NT / 2; o > 0; o >>= 1) {
                if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
                __syncthreads();
            }
            const double alpha = SA[k + SLD * k];
            const double xn = sqrt(red[0]);
            const double beta = -copysign(sqrt(alpha * alpha + xn * xn), alpha);
            const double tau = beta != 0.0 ? (beta - alpha) / beta : 0.0;
            const double sc = (alpha - beta) != 0.0 ? 1.0 / (alpha - beta) : 0.0;
            __syncthreads();
            for (int r = k + 1 + threadIdx.x; r < ns; r += NT) SA[r + SLD * k] *= sc;
            __syncthreads();
            if (threadIdx.x == 0) SA[k + SLD * k] = beta;
            for (int c = k + 1 + threadIdx.x; c < nn; c += NT) {
                double w = SA[k + SLD * c];
                for (int r = k + 1; r < ns; r++) w += SA[r + SLD * k] * SA[r + SLD * c];
                w *= tau;
                SA[k + SLD * c] -= w;
                for (int r = k + 1; r < ns; r++) SA[r + SLD * c] -= w * SA[r + SLD * k];
            }
            __syncthreads();
        }
        // ||R||_1, ||R^-1||_1: thread c owns column c; R^-1(:, c) goes to rows 64.. of column c
        double cr = 0.0, ci = 0.0;
        if (threadIdx.x < nn) {
            const int c = threadIdx.x;
            double *x = SA + 64 + SLD * c;
            for (int r = 0; r <= c; r++) cr += fabs(SA[r + SLD * c]);
            for (int r = c; r >= 0; r--) {
                double v = (r == c) ? 1.0 : 0.0;
                for (int p = r + 1; p <= c; p++) v -= SA[r + SLD * p] * x[p];
                x[r] = v / SA[r + SLD * r];
                ci += fabs(x[r]);
            }
            if (!(ci <= 1e300)) ci = INFINITY;  // singular R: no finite estimate
        }
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
    }
}

}  // namespace feat

struct BMHandle {
    int count, nrhs;
    std::vector<BMInst> h;
    BMInst *d_inst;
    int *d_list, *d_flag;
    GramJob *d_gj;
    MapJob *d_mj;
    double **d_G;
    double *d_orth;
    float *d_F;     // selector inputs, count x 5
    int *d_choice;  // selector output
    void *fp64_work;  // metadata of the FP64 Householder solver
    long long fp64_bytes;
    void *mem;
};

}  // namespace lg

using namespace lg;

extern "C" {

void *lila_gels_mixed_create(int count, const int *m, const int *n, int nrhs, double *const *A, const int *lda,
                             double *const *B, const int *ldb)
{
    if (count <= 0 || nrhs < 1 || nrhs > 8) return nullptr;
    BMHandle *H = new BMHandle();
    H->count = count;
    H->nrhs = nrhs;
    H->h.resize(count);
    // one device allocation: per instance Q (m x 64), G, R, X (3 x 4096), colexp, partial
    size_t bytes = 0;
    std::vector<size_t> qoff(count);
    for (int t = 0; t < count; t++) {
        qoff[t] = bytes;
        bytes += (size_t)m[t] * 64 * sizeof(double);
    }
    const size_t small_off = bytes;
    bytes += (size_t)count * (3 * 4096 * sizeof(double) + 64 * sizeof(int) + 8192 * sizeof(long long));
    const size_t meta_off = bytes;
    bytes += (size_t)count * (sizeof(BMInst) + 3 * sizeof(int) + sizeof(GramJob) + sizeof(MapJob) + 2 * sizeof(double *) +
                              5 * sizeof(float)) + 64;
    bytes += 1024;
    const size_t fp64_off = (bytes + 255) & ~(size_t)255;
    H->fp64_bytes = lila_query_dgels_batched(count);
    bytes = fp64_off + (size_t)H->fp64_bytes;
    if (cudaMalloc(&H->mem, bytes) != cudaSuccess) {
        delete H;
        return nullptr;
    }
    uint8_t *base = (uint8_t *)H->mem;
    uint8_t *sp = base + small_off;
    for (int t = 0; t < count; t++) {
        BMInst &I = H->h[t];
        I.m = m[t];
        I.n = n[t];
        I.lda = lda[t];
        I.ldb = ldb[t];
        I.A = A[t];
        I.B = B[t];
        I.Q = (double *)(base + qoff[t]);
        I.G = (double *)sp;
        I.R = I.G + 4096;
        I.X = I.R + 4096;
        sp += 3 * 4096 * sizeof(double);
        I.colexp = (int *)sp;
        sp += 64 * sizeof(int);
        I.partial = (long long *)sp;
        sp += 8192 * sizeof(long long);
    }
    uint8_t *mp = base + meta_off;
    H->d_inst = (BMInst *)mp;
    mp += (size_t)count * sizeof(BMInst);
    H->d_list = (int *)mp;
    mp += (size_t)count * sizeof(int);
    H->d_flag = (int *)mp;
    mp += (size_t)count * sizeof(int);
    mp = (uint8_t *)(((uintptr_t)mp + 15) & ~(uintptr_t)15);
    H->d_gj = (GramJob *)mp;
    mp += (size_t)count * sizeof(GramJob);
    mp = (uint8_t *)(((uintptr_t)mp + 15) & ~(uintptr_t)15);
    H->d_mj = (MapJob *)mp;
    mp += (size_t)count * sizeof(MapJob);
    mp = (uint8_t *)(((uintptr_t)mp + 15) & ~(uintptr_t)15);
    H->d_G = (double **)mp;
    mp += (size_t)count * sizeof(double *);
    H->d_orth = (double *)mp;
    mp += (size_t)count * sizeof(double);
    H->d_F = (float *)mp;
    mp += (size_t)count * 5 * sizeof(float);
    mp = (uint8_t *)(((uintptr_t)mp + 15) & ~(uintptr_t)15);
    H->d_choice = (int *)mp;
    H->fp64_work = base + fp64_off;
    cudaMemcpy(H->d_inst, H->h.data(), sizeof(BMInst) * count, cudaMemcpyHostToDevice);
    return H;
}

int lila_gels_mixed_destroy(void *handle)
{
    BMHandle *H = (BMHandle *)handle;
    if (!H) return 0;
    cudaStreamSynchronize(lg::stream());
    cudaFree(H->mem);
    delete H;
    return 0;
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
        if ((r == 0 || r == 1) && H->h[t].n + nrhs > 64) r = 2;
        (r == 0 ? g0 : r == 1 ? g1 : g2).push_back(t);
    }
    std::vector<int> mixed(g1);
    mixed.insert(mixed.end(), g0.begin(), g0.end());
    const int nm = (int)mixed.size(), n1 = (int)g1.size();
    cudaMemsetAsync(H->d_flag, 0, sizeof(int) * count, st);
    std::vector<GramJob> gj(nm);
    std::vector<MapJob> mj(nm);
    std::vector<double *> gp(nm);
    if (nm > 0) {
        cudaMemcpyAsync(H->d_list, mixed.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, st);
        // pass 1: Gram of A
        for (int k = 0; k < nm; k++) {
            const BMInst &I = H->h[mixed[k]];
            gj[k] = GramJob{I.A, I.lda, I.n, 0, I.m, I.colexp, I.partial};
            gp[k] = I.G;
            mj[k] = MapJob{I.A, I.lda, I.m, I.n, I.X, 64, I.n, I.Q, I.m};
        }
        cudaMemcpyAsync(H->d_gj, gj.data(), sizeof(GramJob) * nm, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(H->d_G, gp.data(), sizeof(double *) * nm, cudaMemcpyHostToDevice, st);
        ozaki_gram_jobs(H->d_gj, nm, H->d_G);
        const size_t fsm = 4 * 4096 * sizeof(double);
        cudaFuncSetAttribute(bm::k_factor, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsm);
        cudaFuncSetAttribute(bm::k_final, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsm);
        // shifted first pass for group 1 (listed first), plain for group 0
        if (n1) {
            bm::k_factor<<<n1, bm::NT, fsm, st>>>(H->d_inst, H->d_list, n1, 1, 1, H->d_flag);
            note_launch("bm_factor");
        }
        if (nm - n1) {
            bm::k_factor<<<nm - n1, bm::NT, fsm, st>>>(H->d_inst, H->d_list + n1, nm - n1, 0, 1, H->d_flag);
            note_launch("bm_factor");
        }
        // Q = A X
        cudaMemcpyAsync(H->d_mj, mj.data(), sizeof(MapJob) * nm, cudaMemcpyHostToDevice, st);
        ozaki_map_jobs(H->d_mj, nm);
        // group 1: one more unshifted pass on Q, Q = Q X in place
        if (n1) {
            std::vector<GramJob> g1j(n1);
            std::vector<MapJob> m1j(n1);
            std::vector<double *> g1p(n1);
            for (int k = 0; k < n1; k++) {
                const BMInst &I = H->h[mixed[k]];
                g1j[k] = GramJob{I.Q, I.m, I.n, 0, I.m, I.colexp, I.partial};
                g1p[k] = I.G;
                m1j[k] = MapJob{I.Q, I.m, I.m, I.n, I.X, 64, I.n, I.Q, I.m};
            }
            cudaMemcpyAsync(H->d_gj, g1j.data(), sizeof(GramJob) * n1, cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(H->d_G, g1p.data(), sizeof(double *) * n1, cudaMemcpyHostToDevice, st);
            ozaki_gram_jobs(H->d_gj, n1, H->d_G);
            bm::k_factor<<<n1, bm::NT, fsm, st>>>(H->d_inst, H->d_list, n1, 0, 0, H->d_flag);
            note_launch("bm_factor");
            cudaMemcpyAsync(H->d_mj, m1j.data(), sizeof(MapJob) * n1, cudaMemcpyHostToDevice, st);
            ozaki_map_jobs(H->d_mj, n1);
        }
        // last pass on [Q | b]
        bm::k_copy_b<<<nm, 256, 0, st>>>(H->d_inst, H->d_list, nm, nrhs);
        note_launch("bm_copy_b");
        for (int k = 0; k < nm; k++) {
            const BMInst &I = H->h[mixed[k]];
            gj[k] = GramJob{I.Q, I.m, I.n + nrhs, 0, I.m, I.colexp, I.partial};
            gp[k] = I.G;
        }
        cudaMemcpyAsync(H->d_gj, gj.data(), sizeof(GramJob) * nm, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(H->d_G, gp.data(), sizeof(double *) * nm, cudaMemcpyHostToDevice, st);
        ozaki_gram_jobs(H->d_gj, nm, H->d_G);
        bm::k_final<<<nm, bm::NT, fsm, st>>>(H->d_inst, H->d_list, nm, nrhs, 50.0, H->d_flag, H->d_orth);
        note_launch("bm_final");
    }
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
    for (int t : mixed) {
        if (orth_host) orth_host[t] = flag[t] == 1 ? -1.0 : orth[t];
        if (flag[t]) {
            info_host[t] = 1;
            fallbacks++;
            if (!(flags & LILA_GELS_NO_FALLBACK)) fp64.push_back(t);
        }
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
        cudaMemcpyAsync(inf.data(), d_info, sizeof(int) * fp64.size(), cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        for (size_t k = 0; k < fp64.size(); k++)
            if (inf[k]) info_host[fp64[k]] = -inf[k];
    }
    return fallbacks;
}

int lila_gels_mixed_features(void *handle, float *F)
{
    BMHandle *H = (BMHandle *)handle;
    if (!H) return -1;
    for (int t = 0; t < H->count; t++)
        if (H->h[t].n > 128) return -1;
    cudaFuncSetAttribute(feat::k_features, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)feat::SMEM);
    int grid = 2 * sm_count();
    if (grid > H->count) grid = H->count;
    trace_begin();
    feat::k_features<<<grid, feat::NT, feat::SMEM, lg::stream()>>>(H->d_inst, H->count, F);
    note_launch("gels_features");
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
        if (H->h[t].n + H->nrhs > 64) route[t] = 2;
        if (route_out) route_out[t] = route[t];
    }
    return lila_gels_mixed_run(handle, route.data(), flags, info, orth);
}

}  // extern "C"
