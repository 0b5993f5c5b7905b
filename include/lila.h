/*
 * lila.h -- C ABI of the GB300 (sm_103a) LILA Householder-QR library.
 *
 * Drop-in for the w03 interface of the reference's lila-c/lila.h: the same
 * names, argument lists and argument meanings, the same column-major FP64
 * layout and the same global-index T layout (T is mt x (n+i); the compact-WY
 * factor of the reflectors [a, b) sharing the tile floor(a/mt) sits at
 * T + (a % mt) + a*ldt).  Differences a caller must know:
 *
 *   * A, T, Q, B, work, tau and S are DEVICE pointers (cudaMalloc'd or
 *     managed); lila_param and nb_lvl stay host pointers.
 *   * Every call is asynchronous and stream-ordered on the calling thread's
 *     library stream (lila_gpu_set_stream, default: the legacy default
 *     stream).  Use lila_gpu_sync() before reading results on the host.
 *   * Return value: 0 on success, -k when argument k is invalid (1-based,
 *     LAPACK style), including a workspace smaller than the matching
 *     lila_query_* result.  The reference always returns 0.
 *   * Numerical breakdowns (Cholesky of a non-positive Gram, a zero LU pivot)
 *     do not trap; they set bits in the device status word read by
 *     lila_gpu_status() (include/lila_gpu.h).
 *   * lila_query_* return the workspace size in doubles that THIS library
 *     needs (it can differ from the reference's counts); the query arguments
 *     are the reference's, pointers may be NULL and lwork may be -1.
 *   * The CholQR + Householder-reconstruction routines keep the sign vector S
 *     apart from their scratch, so leaves of any number of mt tiles are exact
 *     (the reference aliases the two when a leaf spans 3 or more tiles).
 *
 * Reference prototypes are cited as lila-c/lila.h:<line>.
 */
#ifndef LILA_GB300_LILA_H
#define LILA_GB300_LILA_H

#ifdef __cplusplus
extern "C" {
#endif

/* Recursive Householder QR of an m x n panel, n x n T (lila-c/lila.h:9). */
int dgeqr3(int m, int n, double *A, int lda, double *T, int ldt);

/* Apply H^T of reflectors [i,i+k) to A(i:m, j:j+n) in place (lila-c/lila.h:30). */
int lila_dormqrf_w03(int m, int n, int k, int i, int j, int mt, double *A, int lda, double *T,
                     int ldt, double *work, int lwork);
/* Same, to a separate block B(i:m, j:j+n) (lila-c/lila.h:31). */
int lila_dormqrf_z03(int m, int n, int k, int i, int j, int mt, double *A, int lda, double *T,
                     int ldt, double *B, int ldb, double *work, int lwork);
/* Q(i:m, j:j+n) := H_[i,i+k) [0; Q(i+k:m, j:j+n)] (lila-c/lila.h:34; argument
 * order of the definition lila-c/lila_dormqrbz_w03.c:3, Q before T, which is
 * how every caller passes them). */
int lila_dormqrbz_w03(int m, int n, int k, int i, int j, int mt, double *A, int lda, double *Q,
                      int ldq, double *T, int ldt, double *work, int lwork);

/* Householder reconstruction of an m x n orthonormal block (lila-c/lila.h:39). */
int lila_dorgh2_3(int m, int n, double *A, int lda, double *T, int ldt, double *Q, int ldq,
                  double *work, int lwork, double *S);
/* Tile form: reconstruct tile j of a leaf starting at i from Q (lila-c/lila.h:38;
 * the reference's lila_dorgh2.c does not match this prototype, so this library
 * gives it the contract of lila_ormhr2_w03_hr). */
int lila_dorgh2(int m, int n, int i, int j, int mt, double *A, int lda, double *T, int ldt,
                double *Q, int ldq, double *work, int lwork, double *S);
/* Tile j of a CholQR leaf starting at i (lila-c/lila.h:40). */
int lila_ormhr2_w03_hr(int m, int n, int i, int j, int l, int mt, double *A, int lda, double *T,
                       int ldt, double *Q, int ldq, double *work, int lwork, double *S);

/* T coupling inside one mt tile (lila-c/lila.h:43). */
int lila_dlarft_connect_w03(int m, int n, int i, int j, int mt, double *A, int lda, double *T,
                            int ldt);
/* T tiles from V and tau (lila-c/lila.h:44). */
int lila_dlarft_w03(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                    double *tau);

/* Drivers (lila-c/lila.h:46-56). */
int lila_dgeqrf_w03_levelx(int *lila_param, int n_lvl, int i_lvl, int *nb_lvl, int m, int n,
                           int i, int mt, double *A, int lda, double *T, int ldt, double *Q,
                           int ldq, double *work, int lwork);
int lila_dgeqrf_w03_recursive(int *lila_param, int m, int n, int i, int mt, double *A, int lda,
                              double *T, int ldt, double *Q, int ldq, double *work, int lwork);
int lila_dgeqr2_w03(int *lila_param, int m, int n, int i, int mt, double *A, int lda, double *T,
                    int ldt, double *Q, int ldq, double *work, int lwork);
int lila_dgeqrf_w03_mt(int *lila_param, int m, int n, int i, int mt, double *A, int lda, double *T,
                       int ldt, double *Q, int ldq, double *work, int lwork);
int lila_dgeqrf_w03_mt_hh(int *lila_param, int m, int n, int i, int mt, double *A, int lda,
                          double *T, int ldt, double *Q, int ldq, double *work, int lwork);
int lila_dgeqrf_w03_mt_l(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                         double *Q, int ldq, double *work, int lwork);
int lila_dgeqrf_w03_mt_hr(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                          double *Q, int ldq, double *work, int lwork);
int lila_dgeqr2_w03_l(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                      double *Q, int ldq, double *work, int lwork);
int lila_dgeqr2_w03_3(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                      double *Q, int ldq, double *work, int lwork);
int lila_dgeqr2_w03_hr(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                       double *Q, int ldq, double *work, int lwork);

/* Workspace queries, counts of doubles (lila-c/lila.h:58-71). */
int lila_query_dgeqrf_w03_levelx(int *lila_param, int n_lvl, int i_lvl, int *nb_lvl, int m, int n,
                                 int i, int mt, double *A, int lda, double *T, int ldt, double *Q,
                                 int ldq, double *work, int lwork);
int lila_query_dgeqrf_w03_recursive(int *lila_param, int m, int n, int i, int mt, double *A,
                                    int lda, double *T, int ldt, double *Q, int ldq, double *work,
                                    int lwork);
int lila_query_dgeqrf_w03_mt(int *lila_param, int m, int n, int i, int mt, double *A, int lda,
                             double *T, int ldt, double *Q, int ldq, double *work, int lwork);
int lila_query_dgeqrf_w03_mt_hh(int *lila_param, int m, int n, int i, int mt, double *A, int lda,
                                double *T, int ldt, double *Q, int ldq, double *work, int lwork);
int lila_query_dormqrbz_w03(int m, int n, int k, int i, int j, int mt, double *A, int lda,
                            double *Q, int ldq, double *T, int ldt, double *work, int lwork);
int lila_query_dgeqrf_w03_mt_hr(int m, int n, int i, int mt, double *A, int lda, double *T,
                                int ldt, double *Q, int ldq, double *work, int lwork);
int lila_query_dgeqrf_w03_mt_l(int m, int n, int i, int mt, double *A, int lda, double *T,
                               int ldt, double *Q, int ldq, double *work, int lwork);
int lila_query_dgeqr2_w03_hr(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                             double *Q, int ldq, double *work, int lwork);
int lila_query_dgeqr2_w03_3(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                            double *Q, int ldq, double *work, int lwork);
int lila_query_dgeqr2_w03_l(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                            double *Q, int ldq, double *work, int lwork);
int lila_query_ormhr2_w03_hr(int m, int n, int i, int j, int l, int mt, double *A, int lda,
                             double *T, int ldt, double *Q, int ldq, double *work, int lwork,
                             double *S);
int lila_query_dorgh2_3(int m, int n, double *A, int lda, double *T, int ldt, double *Q, int ldq,
                        double *work, int lwork, double *S);
int lila_query_dormqrf_w03(int m, int n, int k, int i, int j, int mt, double *A, int lda,
                           double *T, int ldt, double *work, int lwork);

/* tau from T or from V (lila-c/lila.h:92-93). */
int lila_dT2tau_w03(int m, int n, int i, int mt, double *T, int ldt, double *tau);
int lila_dV2tau_w03(int m, int n, int i, int mt, double *A, int lda, double *tau);

/* Factor n appended columns against k existing ones (lila-c/lila.h:101). */
int lila_dgeqrf_w03_appendcols(int *lila_param, int m, int k, int n, int mt, double *A, int lda,
                               double *Q, int ldq, double *T, int ldt, double *work, int lwork);

/* V, R and T without Q (v03), and Q from the V and T they leave (q03):
 * lila-c/lila.h:74-90.  v03 runs the w03 factorization without forming Q;
 * q03 forms Q(i:m, i:i+n) = H_i .. H_{i+n-1} [I; 0] from A's reflectors and
 * T's tiles.  Both recursions stop at n < nx (w03: n <= nx).  As in the
 * reference, leaf 2 does nothing and panel 2 factors nothing (the tile
 * updates around it still run); leaf 3 is rejected.  The w03 query of the
 * same arguments is enough workspace. */
int lila_dgeqrf_v03_levelx(int *lila_param, int n_lvl, int i_lvl, int *nb_lvl, int m, int n, int i,
                           int mt, double *A, int lda, double *T, int ldt, double *work, int lwork);
int lila_dgeqrf_v03_recursive(int *lila_param, int m, int n, int i, int mt, double *A, int lda,
                              double *T, int ldt, double *work, int lwork);
int lila_dgeqrf_v03_mt(int *lila_param, int m, int n, int i, int mt, double *A, int lda, double *T,
                       int ldt, double *work, int lwork);
int lila_dgeqr2_v03(int *lila_param, int m, int n, int i, int mt, double *A, int lda, double *T,
                    int ldt, double *work, int lwork);
int lila_dgeqrf_v03_mt_hh(int *lila_param, int m, int n, int i, int mt, double *A, int lda,
                          double *T, int ldt, double *work, int lwork);
int lila_dgeqrf_v03_mt_l(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                         double *work, int lwork);
int lila_dgeqr2_v03_l(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                      double *work, int lwork);
int lila_dgeqr2_v03_3(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                      double *work, int lwork);
int lila_dgeqrf_q03_levelx(int *lila_param, int n_lvl, int i_lvl, int *nb_lvl, int m, int n, int i,
                           int mt, double *A, int lda, double *T, int ldt, double *Q, int ldq,
                           double *work, int lwork);
int lila_dgeqrf_q03_recursive(int *lila_param, int m, int n, int i, int mt, double *A, int lda,
                              double *T, int ldt, double *Q, int ldq, double *work, int lwork);
int lila_dgeqrf_q03_mt_hh(int *lila_param, int m, int n, int i, int mt, double *A, int lda,
                          double *T, int ldt, double *Q, int ldq, double *work, int lwork);
int lila_dgeqrf_q03_mt(int *lila_param, int m, int n, int i, int mt, double *A, int lda, double *T,
                       int ldt, double *Q, int ldq, double *work, int lwork);
int lila_dgeqrf_q03_mt_l(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                         double *Q, int ldq, double *work, int lwork);
int lila_dgeqr2_q03(int *lila_param, int m, int n, int i, int mt, double *A, int lda, double *T,
                    int ldt, double *Q, int ldq, double *work, int lwork);
int lila_dgeqr2_q03_l(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                      double *Q, int ldq, double *work, int lwork);
int lila_dgeqr2_q03_3(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                      double *Q, int ldq, double *work, int lwork);

/* Accuracy checks of the packaged library, computed on the device at FP64
 * grade (lila-c-lila_param/lila/include/lila.h:117-121;
 * src/lila_test_qq_orth_1.c:3-19, src/lila_test_qr_repres_1.c:3-27):
 * ||I - Q^T Q||_F and ||A - Q R||_F / ||A||_F over the block at (i, i).
 * Device pointers; both synchronise the library stream. */
double lila_test_qq_orth_1(int m, int n, int i, double *Q, int ldq);
double lila_test_qr_repres_1(int m, int n, int i, double *A, int lda, double *Q, int ldq, double *R,
                             int ldr);

#ifdef __cplusplus
}
#endif

#endif /* LILA_GB300_LILA_H */
