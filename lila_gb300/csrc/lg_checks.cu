// lg_checks.cu -- on-device accuracy checks of a factorization, the GPU form of
// the packaged library's test metrics (lila-c-lila_param/lila/src/
// lila_test_qq_orth_1.c:3-19 and lila_test_qr_repres_1.c:3-27):
//   lila_test_qq_orth_1   = ||I - Q^T Q||_F         over Q(i:m, i:i+n)
//   lila_test_qr_repres_1 = ||A - Q R||_F / ||A||_F  over the block at (i, i)
// Products are FP64-grade: the split-precision Gram / row map for n <= 64,
// the FP64 GEMM otherwise.  Both synchronise and return the value.
#include <math.h>

#include <vector>

#include "lg_common.cuh"
#include "../../include/lila_gpu.h"

namespace lg {

// Frobenius norm of (G - I) for an n x n G (one CTA), scaled sum of squares.
__global__ void k_fro_minus_identity(int n, const double *G, int ldg, double *out)
{
    __shared__ double sh[256];
    double s = 0.0, c = 0.0;
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
        const int r = idx % n, col = idx / n;
        double v = G[(size_t)r + (size_t)col * ldg] - (r == col ? 1.0 : 0.0);
        double y = v * v - c, t = s + y;
        c = (t - s) - y;
        s = t;
    }
    sh[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot = 0.0;
        for (int k = 0; k < blockDim.x; k++) tot += sh[k];
        *out = sqrt(tot);
    }
}

// sum over the m x n block of (X - A)^2 and of A^2, per-CTA partials.
__global__ void k_diff_sq(int m, int n, const double *X, int ldx, const double *A, int lda, double *part)
{
    __shared__ double s1[256], s2[256];
    double a = 0.0, b = 0.0;
    const size_t total = (size_t)m * n;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        const size_t r = idx % m, c = idx / m;
        const double av = A[r + c * lda];
        const double d = X[r + c * ldx] - av;
        a = fma(d, d, a);
        b = fma(av, av, b);
    }
    s1[threadIdx.x] = a;
    s2[threadIdx.x] = b;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            s1[threadIdx.x] += s1[threadIdx.x + o];
            s2[threadIdx.x] += s2[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = s1[0];
        part[2 * blockIdx.x + 1] = s2[0];
    }
}

static double *g_check_buf = nullptr;
static long long g_check_len = 0;

static double *check_scratch(long long len)
{
    if (len > g_check_len) {
        if (g_check_buf) {
            cudaStreamSynchronize(stream());
            cudaFree(g_check_buf);
        }
        g_check_buf = nullptr;
        g_check_len = 0;
        if (cudaMalloc(&g_check_buf, (size_t)len * sizeof(double)) != cudaSuccess) return nullptr;
        g_check_len = len;
    }
    return g_check_buf;
}

// G = Q^T Q (n x n, ld n) at FP64 grade into buf; returns false on failure.
static bool gram_fp64_grade(int m, int n, const double *Q, int ldq, double *G, double *wk, long long wklen)
{
    if (n <= 64) return ozaki_gram(m, n, Q, ldq, G, n, wk, wklen) == 0;
    GemmEpi e;
    gemm(n, n, m, opnd(Q, ldq, TR), opnd(Q, ldq), G, n, e, wk, wklen, "check_gram");
    return true;
}

}  // namespace lg

using namespace lg;

extern "C" {

double lila_test_qq_orth_1(int m, int n, int i, double *Q, int ldq)
{
    const int ml = m - i;
    if (ml <= 0 || n <= 0) return 0.0;
    const long long wk = ozaki_gram_work(sm_count()) + 64LL * n * n + 4096;
    double *buf = check_scratch((long long)n * n + 1 + wk);
    if (!buf) return NAN;
    double *G = buf, *out = buf + (size_t)n * n, *w = out + 1;
    const double *Qii = Q + i + (size_t)i * ldq;
    if (!gram_fp64_grade(ml, n, Qii, ldq, G, w, wk)) return NAN;
    k_fro_minus_identity<<<1, 256, 0, stream()>>>(n, G, n, out);
    note_launch("check_orth");
    double v = NAN;
    cudaMemcpyAsync(&v, out, sizeof(double), cudaMemcpyDeviceToHost, stream());
    cudaStreamSynchronize(stream());
    return v;
}

double lila_test_qr_repres_1(int m, int n, int i, double *A, int lda, double *Q, int ldq, double *R, int ldr)
{
    const int ml = m - i;
    if (ml <= 0 || n <= 0) return 0.0;
    const int parts = 4 * sm_count();
    double *buf = check_scratch((long long)ml * n + 2LL * parts + 64LL * 64);
    if (!buf) return NAN;
    double *X = buf, *part = buf + (size_t)ml * n, *Ru = part + 2 * parts;
    const double *Aii = A + i + (size_t)i * lda;
    const double *Qii = Q + i + (size_t)i * ldq;
    const double *Rii = R + i + (size_t)i * ldr;
    // X = Q triu(R) at FP64 grade
    if (n <= 64) {
        copy2d(n, n, Rii, ldr, Ru, n);
        set2d(n, n, 0.0, 0.0, Ru, n, 2);
        ozaki_map(ml, n, Qii, ldq, Ru, n, n, X, ml);
    } else {
        GemmEpi e;
        gemm(ml, n, n, opnd(Qii, ldq), opnd(Rii, ldr, NT, M_UPPER), X, ml, e, nullptr, 0, "check_qr");
    }
    k_diff_sq<<<parts, 256, 0, stream()>>>(ml, n, X, ml, Aii, lda, part);
    note_launch("check_repres");
    std::vector<double> h(2 * parts);
    cudaMemcpyAsync(h.data(), part, sizeof(double) * 2 * parts, cudaMemcpyDeviceToHost, stream());
    cudaStreamSynchronize(stream());
    double num = 0.0, den = 0.0;
    for (int p = 0; p < parts; p++) {
        num += h[2 * p];
        den += h[2 * p + 1];
    }
    return den > 0.0 ? sqrt(num / den) : sqrt(num);
}

}  // extern "C"
