/*
 * lila_prim.h -- the GB300 library's FP64 device primitives, exported one by
 * one so each kernel can be unit-tested against a host computation.  They
 * have no counterpart in the reference (which calls CBLAS/LAPACKE: dgemm,
 * dtrsm, dpotrf, dlarfg; lila-c/lila.h:6-7).  Pointers are device pointers;
 * calls are enqueued on the library stream (include/lila_gpu.h).
 * Trans: 0 = no transpose, 1 = transpose.  Mask of the stored operand:
 * 0 full, 1 unit lower trapezoid, 2 upper, 3 lower, 4 unit upper.
 */
#ifndef LILA_GB300_LILA_PRIM_H
#define LILA_GB300_LILA_PRIM_H
#ifdef __cplusplus
extern "C" {
#endif
int lila_prim_gemm(int M, int N, int K, const double *A, int lda, int transA, int maskA,
                   const double *B, int ldb, int transB, int maskB, double *C, int ldc, double alpha,
                   double beta, int zero_rows, int add_diag, int upper_only, double *part,
                   long long part_len);
int lila_prim_gemm_splits(int M, int N, int K, long long part_len);
/* The same product at FP64 grade on the BF16 tensor cores (tcgen05). */
int lila_prim_ozgemm(int M, int N, int K, const double *A, int lda, int transA, int maskA,
                     const double *B, int ldb, int transB, int maskB, double *C, int ldc,
                     double alpha, double beta, int zero_rows, int add_diag, int upper_only,
                     double *part, long long part_len);
int lila_prim_ozgemm_splits(int M, int N, int K, long long part_len);
int lila_prim_trsm_right_upper(int M, int N, double alpha, const double *U, int ldu, double *B,
                               int ldb, const double *S);
int lila_prim_trsm_left_lower_unit(int M, int N, const double *L, int ldl, double *B, int ldb);
int lila_prim_trsm_right_lower_unit_trans(int M, int N, double alpha, const double *L, int ldl,
                                          double *B, int ldb);
int lila_prim_potrf_upper(int n, double *A, int lda);
int lila_prim_lu_sign(int n, double *T, int ldt, double *S);
int lila_prim_larfg(int m, double *x, double *tau);
/* The pivot step of the split leaf's FP64 factor: out[k] = 1 / sqrt(d[k])
 * (Newton-Raphson from a single-precision estimate, within about 1.5 ulp);
 * 0 where d[k] is not positive and finite. */
int lila_prim_rsqrt(int n, const double *d, double *out);
/* One pass's factor of the split leaf (n <= 64): from the Gram G the upper
 * Rk with Rk^T Rk = G (+ sigma I, sigma = shift_factor trace(G), when the
 * trial factor breaks down, its diagonal ratio or its 1-norm condition
 * estimate ||Rk||_1 ||Rk^-1||_1 exceeds cond_limit, or for variant 2) and
 * X = Rk^-1, both n x n with their strictly lower parts zero.  variant 1:
 * no trial, never shifted.  Returns 1 when the shift was taken, 0 when not,
 * negative for an argument error; breakdown of the factor that is kept sets
 * LILA_ST_CHOL_BREAKDOWN in the status word. */
int lila_prim_factor_pass(int n, const double *G, int ldg, double *Rk, int ldk, double *X, int ldx, int variant,
                          double shift_factor, double cond_limit);
/* FP64 throughput probe (kind 0: DFMA chains, 1: DMMA mma.sync m8n8k4);
 * returns GFLOP/s; out holds blocks*threads doubles. */
double lila_prim_fp64_probe(int kind, double *out, int blocks, int threads, int iters);
/* One-tile tcgen05 check: D(128 x N, row-major FP32) = A(128 x 64) * B(N x 64)^T with
 * A, B row-major BF16; N in {16, 32, ..., 256}. */
int lila_prim_tc_selftest(const void *A, const void *B, float *D, int N, int swap);
/* FP64-grade G = A^T A (n <= 64) on the BF16 tensor cores (split-precision);
 * work holds lila_prim_ozaki_gram_work() doubles. */
long long lila_prim_ozaki_gram_work(void);
int lila_prim_ozaki_gram(int m, int n, const double *A, int lda, double *G, int ldg, double *work,
                         long long lwork);
/* Same with the rows handled per CTA forced (diagnostics of the pipeline). */
int lila_prim_ozaki_gram_rows(int m, int n, const double *A, int lda, double *G, int ldg, double *work,
                              long long lwork, int rows_per);
/* FP64-grade out = A X (n, nout <= 64) on the BF16 tensor cores; out may be A itself. */
int lila_prim_ozaki_map(int m, int n, const double *A, int lda, const double *X, int ldx, int nout,
                        double *out, int ldo);
/* Which kernels the tall Gram and row map take (TMA-fed ones only where A is
 * 16-byte aligned with an even lda): 0 (default) the TMA-fed Gram and the
 * register-fed row map; 1 both register-fed; 2 / 3 the TMA-fed Gram and the
 * TMA-fed warp-specialised row map on transposed 32-row tiles (double-buffered
 * tensor memory) assembling its FP64 outputs through the FP64-pipe
 * int64 -> double conversion (2) or integer instructions (3), the same bits.
 * Returns the previous setting. */
int lila_prim_ozaki_map_path(int path);
/* Failure-path test of the cooperative panel's grid barrier: runs the panel
 * of an m x nb matrix (dgeqr3's one-launch panel) with every barrier waiting
 * for `extra` arrivals that never come, so each wait runs out after the
 * lila_gpu_set_wait_limit cycles, sets LILA_ST_WAIT_TIMEOUT and the kernel
 * returns; A and T are left meaningless.  1 when the launch ran, 0 when the
 * panel does not apply to the shape.  work: lila_prim_panel_work(nb) doubles. */
int lila_prim_panel_phantom(int m, int nb, double *A, int lda, double *T, int ldt, double *work, int extra);
long long lila_prim_panel_work(int nb);
#ifdef __cplusplus
}
#endif
#endif
