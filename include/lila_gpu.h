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

#ifdef __cplusplus
}
#endif

#endif
