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
/* Clock-cycle limit of the device-side grid-barrier waits of the cooperative
 * Householder panel (default 4e9, about 2 s at 2 GHz): a wait that reaches it
 * sets LILA_ST_WAIT_TIMEOUT and its kernel returns.  cycles <= 0 keeps the
 * setting.  Returns the previous limit. */
long long lila_gpu_set_wait_limit(long long cycles);
/* Number of kernels this library has launched in this process. */
unsigned long long lila_gpu_launch_count(void);
/* CUDA-event timing of every launch (on: 1) and its per-kernel summary as
 * "name launches total_ms" lines; off by default. */
int lila_gpu_trace(int on);
int lila_gpu_trace_summary(char *buf, int len);

/* Precision of the library's large products (FP64 GEMMs of the block
 * reflector updates, panels, explicit Q; products with M, N, K >= 64 and
 * M N K >= 2^27): LILA_PRECISION_FP64 (default) runs them on the FP64 CUDA
 * cores; LILA_PRECISION_SPLIT runs them as FP64-grade split-precision products
 * on the BF16 tensor cores (eight base-128 digits per value, exact integer
 * accumulation, error below 2^-50 (max|a| sum|b| + sum|a| max|b|) per entry).
 * Returns the previous mode; other values only query. */
#define LILA_PRECISION_FP64 0
#define LILA_PRECISION_SPLIT 1
int lila_gpu_set_precision(int mode);

/* Graph mode (off by default).  When on, a public factorization or update
 * call (the recursive, levelx, mt, mt_hh, mt_l, mt_hr, dgeqr2_w03, dormqrf,
 * dormqrbz, ormhr2_w03_hr and dorgh2_3 entries) whose arguments -- sizes,
 * pointers, lwork and the lila_param / nb_lvl contents -- equal those of an
 * earlier call on the same device replays the CUDA graph captured from that
 * earlier call (one launch instead of one per kernel).  The first call of a
 * key pays the capture.  Calls that cannot be captured (host synchronisation
 * inside, as in the adaptive split-precision leaf) run directly.  Up to 64
 * graphs are kept (least recently used evicted).  graph_mode returns the
 * previous mode (on < 0 only queries); cache_clear frees the graphs and
 * returns how many there were; graph_replays counts replays. */
int lila_gpu_graph_mode(int on);
int lila_gpu_graph_cache_clear(void);
unsigned long long lila_gpu_graph_replays(void);

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
/* On-device accuracy check of the split-precision leaf (no counterpart in the
 * reference, whose drivers measure accuracy on the host afterwards with
 * lila_test_qq_orth_1 / lila_test_qr_repres_1,
 * lila-c-lila_param/lila/src/lila_test_qq_orth_1.c:3-19,
 * lila_test_qr_repres_1.c:3-27).  After its passes the leaf measures
 * ||I - Q^T Q||_F and ||A - Q R||_F / ||A||_F of its result and compares both
 * with 50 n 2^-53:
 *   level 0  no check;
 *   level 1  (default) the orthogonality from the last pass's Gram (the
 *            output Q is that pass's candidate C times an n x n matrix M, so
 *            Q^T Q = M^T (C^T C) M up to the rounding of the FP64-grade map),
 *            the residual over a sample of rows (every ceil(ml / 8192)-th row
 *            of the leaf, kept before A is overwritten);
 *   level 2  the orthogonality from one more split-precision Gram of the
 *            output Q, the same residual sample.
 * A failed check, or passes that never reached two unshifted ones in a row,
 * re-solves the leaf in FP64: the TSQR leaf (lila_dgeqrf_w03_tsqr) factors
 * the computed Q S = Q' R', and the outputs become its V, T and Q' with
 * R' S R as R (A = Q S S R holds to the residual check, so no copy of A is
 * kept).  The fallback needs the workspace lila_query_dgeqrf_w03_mt_hr_mixed
 * returns; with less (at least the leaf's own part) or with non-finite input
 * the failure is reported instead: LILA_ST_CHECK_FAILED in the status word
 * and a return value of 1.  set_check returns the previous level (level < 0
 * or > 2 only queries); last_check gives the last checked leaf's residual and
 * orthogonality (-1 when it was not checked; returns -1 then, else 0);
 * last_fallback is 1 when the last leaf was re-solved in FP64. */
int lila_gpu_set_check(int level);
int lila_gpu_last_check(double *res, double *orth);
int lila_gpu_last_fallback(void);

/* Autotuner of lila_dgeqrf_w03_recursive's panel width mt and recursion
 * cutoff nx for one shape (no counterpart in the reference, whose drivers
 * take both as parameters): with leaf and panel from lila_param, every
 * candidate mt in {32, 64, 128, 256} x nx in {32, .., 512} that T (ldt) and
 * work (lwork) can hold factors a copy of A in Ascratch (same lda), once to
 * warm up and once timed; A is not modified, Ascratch, T and Q are scratch.
 * The fastest is written to lila_param[3] and *mt; returns its time in
 * microseconds, -12 when no candidate fits, -k for a bad argument. */
int lila_gpu_recursive_autotune(int *lila_param, int m, int n, const double *A, int lda, double *Ascratch,
                                double *T, int ldt, double *Q, int ldq, double *work, int lwork, int *mt);

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

/* Out-of-core tall-skinny QR (no counterpart in the reference): the
 * split-precision leaf lila_dgeqrf_w03_mt_hr_mixed at i = 0 for an m x n
 * matrix (n <= 64) that stays in HOST memory.  A (lda) and Q (ldq) are host
 * arrays (page-locked, e.g. cudaHostAlloc / cudaHostRegister, for copies
 * that overlap the work; on Grace they cross NVLink-C2C), T (mt x n, ldt)
 * and work are device arrays.  On return A holds V and S R, T the tiles and
 * Q the orthonormal factor times S, as from the in-core leaf.  The rows go
 * through the device in chunks of rows_per_chunk rows (0: 1,048,576;
 * rounded up to a multiple of 128 and at least n): every Cholesky QR pass
 * reads A once, and the last one also writes V and Q (device memory:
 * about 6 chunk buffers).  query returns the workspace in doubles (0 for
 * arguments it cannot take); the call returns 0, -k for a bad argument k
 * (-12 too little workspace) or -100 on a CUDA error. */
long long lila_gpu_query_dgeqrf_tall_host(int m, int n, int rows_per_chunk);
int lila_gpu_dgeqrf_tall_host(int m, int n, int mt, double *A, int lda, double *T, int ldt, double *Q,
                              int ldq, int rows_per_chunk, double *work, long long lwork);

/* Batched least squares with per-instance variants (no counterpart in the
 * reference): 0 Cholesky QR 2 and 1 shifted Cholesky QR 3, both with
 * FP64-grade split-precision tensor-core products (n <= 128, n + nrhs <= 136
 * and m >= 2n, else the instance goes to variant 2; every pass is one grouped
 * launch over the routed instances),
 * and 2 the FP64 Householder solver above.  Variants 0/1 check on the device
 * that no Cholesky broke down and that the orthogonality of the final implicit
 * Q is at most 50 n 2^-53; an instance that fails is re-solved by variant 2
 * (unless flags has LILA_GELS_NO_FALLBACK).  The first Cholesky factor of a
 * variant-0 instance is a trial (unless flags has LILA_GELS_NO_TRIAL): when
 * it breaks down or its 1-norm condition number exceeds 1e8 the instance
 * continues as variant 1 (the shift applied to the same Gram), and
 * lila_gels_mixed_shifted reports it (set_trial_limit replaces the 1e8;
 * -1 unless limit > 0).  create takes host arrays like
 * lila_dgels_batched_prepare (nrhs <= 8), allocates the scratch (two
 * m_t x (n_t + nrhs) blocks and three 136 x 136 blocks of doubles per
 * eligible instance) and returns a handle, NULL on error.
 * run takes the host route array, writes info[t] (host): 0 solved as routed,
 * 1 the routed variant's check failed (unless NO_FALLBACK the instance was
 * then solved by variant 1 if it had been routed to variant 0, that
 * passed and the trial had not already chosen variant 1, else by variant
 * 2), -k R(k,k) == 0 in variant 2; orth[t] (host,
 * may be NULL) gets the orthogonality measured by the last mixed variant run
 * on it (-1 Cholesky breakdown, -2 variant 2 only).  It returns the number of
 * failed checks of the routed variants.  x overwrites B_t(0:n_t, :); A_t is
 * overwritten only by variant 2.
 * features writes 5 FP32 selector inputs per instance to F (device, count x
 * 5); instances the mixed variants cannot take (n_t > 128, n_t + nrhs > 136
 * or m_t < 2 n_t) get zeros and are always solved by variant 2. */
#define LILA_GELS_NO_FALLBACK 1
#define LILA_GELS_NO_TRIAL 2
void *lila_gels_mixed_create(int count, const int *m, const int *n, int nrhs, double *const *A,
                             const int *lda, double *const *B, const int *ldb);
int lila_gels_mixed_run(void *handle, const int *route, int flags, int *info, double *orth);
int lila_gels_mixed_features(void *handle, float *F);
int lila_gels_mixed_destroy(void *handle);
/* The instances of the last run whose trial factor chose the shift: the
 * count, and per instance 0/1 into shifted (host, may be NULL). */
int lila_gels_mixed_shifted(void *handle, int *shifted);
int lila_gels_mixed_set_trial_limit(void *handle, double limit);
/* features -> lila_sel_infer(params) -> run; route_out (host, may be NULL)
 * receives the variant used per instance. */
int lila_gels_mixed_solve(void *handle, const float *params, int flags, int *info, double *orth,
                          int *route_out);

/* Learned variant selector: a 5-64-64-64-3 FP32 perceptron (ReLU, softmax;
 * parameter layout W1 64x5 | b1 | W2 64x64 | b2 | W3 64x64 | b3 | W4 3x64 | b4,
 * W row-major) with its own inference, gradient and Adam kernels.  All arrays
 * are device arrays except loss_host.  grad: the gradient of the class-weighted
 * mean cross entropy over count samples (idx selects them, NULL = 0..count-1),
 * loss its value; work: lila_sel_grad_work(count) floats.  train runs
 * mini-batch Adam (a std::mt19937(seed) permutation per epoch). */
#define LILA_SEL_PARAMS 8899
int lila_sel_params(void);
int lila_sel_init(float *params, unsigned seed);
int lila_sel_infer(int count, const float *params, const float *F, float *logits, int *choice);
long long lila_sel_grad_work(int count);
int lila_sel_grad(int count, const float *params, const float *F, const int *label, const int *idx,
                  const float *cw, float *grad, float *loss, float *work, long long lwork);
int lila_sel_adam(const float *grad, float *params, float *m1, float *m2, int step, float lr);
long long lila_sel_train_work(int n, int batch);
int lila_sel_train(int n, const float *F, const int *label, const float *cw, float *params, int epochs,
                   int batch, float lr, unsigned seed, float *work, long long lwork, float *loss_host);

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
