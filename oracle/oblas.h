/* oblas.h -- the oracle's FP64 BLAS/LAPACK subset (test infrastructure only). */
#ifndef ORACLE_OBLAS_H
#define ORACLE_OBLAS_H

enum { OB_N = 0, OB_T = 1 };
enum { OB_UPPER = 0, OB_LOWER = 1 };
enum { OB_NONUNIT = 0, OB_UNIT = 1 };
enum { OB_LEFT = 0, OB_RIGHT = 1 };

void ob_dgemm(int ta, int tb, int m, int n, int k, double alpha, const double *A, int lda,
              const double *B, int ldb, double beta, double *C, int ldc);
void ob_dtrmm(int side, int uplo, int ta, int diag, int m, int n, double alpha, const double *A,
              int lda, double *B, int ldb);
void ob_dtrsm(int side, int uplo, int ta, int diag, int m, int n, double alpha, const double *A,
              int lda, double *B, int ldb);
void ob_dsyrk(int uplo, int ta, int n, int k, double alpha, const double *A, int lda, double beta,
              double *C, int ldc);
void ob_dger(int m, int n, double alpha, const double *x, int incx, const double *y, int incy,
             double *A, int lda);
double ob_ddot(int n, const double *x, int incx, const double *y, int incy);
double ob_dnrm2(int n, const double *x, int incx);
double ob_dlapy2(double x, double y);
void ob_dlarfg(int n, double *alpha, double *x, int incx, double *tau);
void ob_dgeqr2(int m, int n, double *A, int lda, double *tau);
void ob_dlarft_fc(int n, int k, const double *V, int ldv, const double *tau, double *T, int ldt);
void ob_dorg2r(int m, int n, int k, double *A, int lda, const double *tau);
int ob_dpotrf_upper(int n, double *A, int lda);
void ob_dlacpy(int m, int n, const double *A, int lda, double *B, int ldb);
double ob_dlange_fro(int m, int n, const double *A, int lda);

#endif
#ifndef ORACLE_OBLAS_DD
#define ORACLE_OBLAS_DD
double ob_ddot_dd(int n, const double *x, int incx, const double *y, int incy);
void ob_dgemm_dd(int ta, int m, int n, int k, const double *A, int lda, const double *B, int ldb,
                 double *C, int ldc);
#endif
