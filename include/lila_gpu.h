/*
 * lila_gpu.h -- GB300 runtime controls of the LILA library (no counterpart in
 * the reference, which is synchronous host code: lila-c/lila.h has no stream,
 * status or device concepts).
 */
#ifndef LILA_GB300_LILA_GPU_H
#define LILA_GB300_LILA_GPU_H

#define LILA_GPU_VERSION 1

/* Status bits returned by lila_gpu_status(). */
#define LILA_ST_CHOL_BREAKDOWN 1  /* non-positive pivot in a Cholesky factorization */
#define LILA_ST_LU_ZERO_PIVOT 2   /* zero pivot in the reconstruction LU */
#define LILA_ST_NONFINITE 4       /* a non-finite value reached a checked output */
#define LILA_ST_CHECK_FAILED 8    /* an on-device accuracy check exceeded its bound */
#define LILA_ST_WAIT_TIMEOUT 16   /* a bounded device-side wait gave up */
#define LILA_ST_LAUNCH_ERROR 32   /* a kernel launch failed (host side) */

#ifdef __cplusplus
extern "C" {
#endif

/* Stream on which the calling host thread's lila calls are enqueued
 * (a cudaStream_t passed as void*; NULL = legacy default stream). */
int lila_gpu_set_stream(void *stream);
void *lila_gpu_get_stream(void);
/* Wait for the calling thread's stream; 0 or -cudaError. */
int lila_gpu_sync(void);
/* Synchronise the stream and return the OR of the status bits above. */
int lila_gpu_status(void);
int lila_gpu_clear_status(void);
int lila_gpu_version(void);
/* Number of kernels this library has launched in this process. */
unsigned long long lila_gpu_launch_count(void);
/* CUDA-event timing of every launch (on: 1) and its per-kernel summary as
 * "name launches total_ms" lines; off by default. */
int lila_gpu_trace(int on);
int lila_gpu_trace_summary(char *buf, int len);

/* Split-precision form of lila_dgeqrf_w03_mt_hr (lila-c/lila.h:53): the same
 * outputs (V and S*R in A, T tiles, Q*S in Q) computed by Cholesky QR 2 (or
 * shifted Cholesky QR 3 for ill-conditioned leaves) whose tall products run
 * on the BF16 tensor cores at FP64-grade accuracy; n <= 64.  The same leaf is
 * selected inside lila_dgeqrf_w03_recursive / _levelx / _mt by
 * lila_param[1] = 3.  Passes are adaptive: a pass whose trial Cholesky breaks
 * down or is too ill-conditioned is shifted, and the leaf ends after two
 * unshifted passes.  The _v form picks 0 adaptive, 1 Cholesky QR 2 only,
 * 2 shifted first pass; lila_gpu_last_variant() reports 1 (no shift) or
 * 2 (shifted passes were used). */
int lila_dgeqrf_w03_mt_hr_mixed(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                                double *Q, int ldq, double *work, int lwork);
int lila_dgeqrf_w03_mt_hr_mixed_v(int variant, int m, int n, int i, int mt, double *A, int lda,
                                  double *T, int ldt, double *Q, int ldq, double *work, int lwork);
int lila_query_dgeqrf_w03_mt_hr_mixed(int m, int n, int i, int mt, double *A, int lda, double *T,
                                      int ldt, double *Q, int ldq, double *work, int lwork);
int lila_gpu_last_variant(void);
/* Number of Gram passes the last split-precision leaf took. */
int lila_gpu_last_passes(void);

/* Tall-skinny leaf by a TSQR reduction tree (row blocks of mb <= 256 rows,
 * groups of `arity` R factors per tree node, Q by a backward sweep) followed
 * by the Householder reconstruction of lila_dgeqrf_w03_mt_hr (lila-c/lila.h:53):
 * same outputs (V and S R in A, T tiles, Q S in Q), FP64, stable at any
 * condition number.  The reference's tree QR is LAPACK's dlatsqr
 * (tsqr/main_test_tsqr.c:234-395).  mb = 0 / arity = 0 take the values found
 * by lila_gpu_tsqr_autotune for the shape (else 256 / 4); mb*n and
 * arity*n*n must not exceed 16384. */
int lila_dgeqrf_w03_tsqr(int mb, int arity, int m, int n, int i, int mt, double *A, int lda, double *T,
                         int ldt, double *Q, int ldq, double *work, int lwork);
int lila_query_dgeqrf_w03_tsqr(int mb, int arity, int m, int n, int i, int mt);
int lila_gpu_tsqr_autotune(int m, int n, double *A, int lda, double *T, int ldt, double *Q, int ldq,
                           double *work, int lwork);

/* Batched least squares: count independent problems min ||A_t x - B_t||
 * (A_t m_t x n_t with m_t >= n_t, nrhs <= 8 right-hand sides), the reference's
 * least-squares driver per instance (least-squares/main_ls_qr3.c:94-119) in
 * one persistent launch.  m, n, lda, ldb and the pointer arrays A, B (device
 * addresses) are host arrays; x overwrites B_t(0:n_t, :), V and R overwrite
 * A_t, info[t] (device) is 0 or k when R(k,k) is exactly zero.  prepare uploads
 * the batch description into work (lila_query_dgels_batched(count) bytes);
 * run is one capturable launch; graph captures run into a CUDA graph that
 * lila_gpu_graph_launch replays. */
long long lila_query_dgels_batched(int count);
int lila_dgels_batched_prepare(int count, const int *m, const int *n, int nrhs, double *const *A,
                               const int *lda, double *const *B, const int *ldb, void *work,
                               long long work_bytes);
int lila_dgels_batched_run(int count, int nrhs, void *work, int *info);
void *lila_dgels_batched_graph(int count, int nrhs, void *work, int *info);
int lila_gpu_graph_launch(void *exec);
int lila_gpu_graph_destroy(void *exec);
/* Autotuner of the persistent launch (threads per CTA, CTAs per SM): times the
 * candidates on the prepared batch, restoring A and B from the saved copies
 * before each, and keeps the fastest; returns threads * 100 + CTAs per SM. */
int lila_gpu_gels_autotune(int count, int nrhs, void *work, int *info, double *const *Asave,
                           double *const *A, const long long *bytesA, double *const *Bsave,
                           double *const *B, const long long *bytesB);
int lila_gpu_gels_config(int threads, int per_sm);

/* lila_dormqrf_w03 without a workspace argument, for callers that cannot
 * allocate device memory (a fixed pre-reserved memory pool, or a solver loop
 * that must not let cudaMalloc synchronise the device).  No counterpart in
 * the reference.  Its scratch is a fixed device array of
 * LILA_NOALLOC_SCRATCH_DOUBLES doubles held by every GPU that loads the
 * library; 2 * min(mt, k) * n must not exceed it (else
 * LILA_NOALLOC_TOO_LARGE, nothing enqueued).  All calls share the array:
 * calls that overlap on the GPU race.  The first call on a device looks up
 * the array's address and should come before any stream capture. */
#define LILA_NOALLOC_SCRATCH_DOUBLES 524288
#define LILA_NOALLOC_TOO_LARGE (-101)
#define LILA_NOALLOC_NO_DEVICE (-102)
int lila_dormqrf_w03_noalloc(int m, int n, int k, int i, int j, int mt, double *A, int lda, double *T,
                             int ldt);

#ifdef __cplusplus
}
#endif

#endif
