// lg_debug.cu -- C entry points onto the individual FP64 device primitives,
// for unit tests of each kernel against a host computation (include/lila_prim.h).
#include "lg_common.cuh"
#include "../../include/lila_prim.h"

using namespace lg;

extern "C" {

int lila_prim_gemm(int M, int N, int K, const double *A, int lda, int transA, int maskA,
                   const double *B, int ldb, int transB, int maskB, double *C, int ldc, double alpha,
                   double beta, int zero_rows, int add_diag, int upper_only, double *part,
                   long long part_len)
{
    GemmEpi e;
    e.alpha = alpha;
    e.beta = beta;
    e.zero_rows = zero_rows;
    e.add_diag = add_diag;
    e.upper_only = upper_only;
    gemm(M, N, K, opnd(A, lda, transA, maskA), opnd(B, ldb, transB, maskB), C, ldc, e, part, part_len);
    return 0;
}

int lila_prim_gemm_splits(int M, int N, int K, long long part_len) { return gemm_splits(M, N, K, part_len); }

int lila_prim_ozgemm(int M, int N, int K, const double *A, int lda, int transA, int maskA, const double *B, int ldb,
                     int transB, int maskB, double *C, int ldc, double alpha, double beta, int zero_rows,
                     int add_diag, int upper_only, double *part, long long part_len)
{
    GemmEpi e;
    e.alpha = alpha;
    e.beta = beta;
    e.zero_rows = zero_rows;
    e.add_diag = add_diag;
    e.upper_only = upper_only;
    ozgemm(M, N, K, opnd(A, lda, transA, maskA), opnd(B, ldb, transB, maskB), C, ldc, e, part, part_len);
    return 0;
}

int lila_prim_ozgemm_splits(int M, int N, int K, long long part_len) { return ozgemm_splits(M, N, K, part_len); }

int lila_prim_trsm_right_upper(int M, int N, double alpha, const double *U, int ldu, double *B,
                               int ldb, const double *S)
{
    trsm_right_upper(M, N, alpha, U, ldu, B, ldb, S);
    return 0;
}

int lila_prim_trsm_left_lower_unit(int M, int N, const double *L, int ldl, double *B, int ldb)
{
    trsm_left_lower_unit(M, N, L, ldl, B, ldb);
    return 0;
}

int lila_prim_trsm_right_lower_unit_trans(int M, int N, double alpha, const double *L, int ldl,
                                          double *B, int ldb)
{
    trsm_right_lower_unit_trans(M, N, alpha, L, ldl, B, ldb);
    return 0;
}

int lila_prim_potrf_upper(int n, double *A, int lda)
{
    potrf_upper(n, A, lda);
    return 0;
}

int lila_prim_lu_sign(int n, double *T, int ldt, double *S)
{
    lu_sign(n, T, ldt, S);
    return 0;
}

int lila_prim_larfg(int m, double *x, double *tau)
{
    larfg(m, x, tau);
    return 0;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// FP64 throughput probes: the measured denominators for the plain-FP64
// kernels' roofline.  Each thread runs independent FMA chains; one value per
// thread is written so the work is not optimised away.
// ---------------------------------------------------------------------------
__global__ void k_probe_dfma(double *out, int iters, double a, double b)
{
    double x0 = threadIdx.x * 1e-9, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; i++) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void k_probe_dmma(double *out, int iters, double a, double b)
{
    double c[8];
    for (int k = 0; k < 8; k++) c[k] = 0.0;
    double fa = a + threadIdx.x * 1e-12, fb = b;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k += 2) {
            asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%4,%5};\n"
                         : "=d"(c[k]), "=d"(c[k + 1])
                         : "d"(fa), "d"(fb), "d"(c[k]), "d"(c[k + 1]));
        }
    }
    double s = 0.0;
    for (int k = 0; k < 8; k++) s += c[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

extern "C" {
// Runs the probe (kind 0: DFMA, 1: DMMA m8n8k4) with blocks x threads and
// returns achieved FP64 GFLOP/s (device timing with events); out must hold
// blocks*threads doubles.
double lila_prim_fp64_probe(int kind, double *out, int blocks, int threads, int iters)
{
    cudaStream_t st = stream();
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int rep = 0; rep < 2; rep++) {
        cudaEventRecord(e0, st);
        if (kind == 0)
            k_probe_dfma<<<blocks, threads, 0, st>>>(out, iters, 0.999999, 1e-7);
        else
            k_probe_dmma<<<blocks, threads, 0, st>>>(out, iters, 0.999999, 1e-7);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
    }
    note_launch("fp64_probe");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    double flops = kind == 0 ? 2.0 * 8 * iters * (double)blocks * threads
                             : 512.0 * 4 * iters * (double)blocks * (threads / 32);
    return flops / (ms * 1e-3) / 1e9;
}
}
