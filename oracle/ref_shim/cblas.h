/* Minimal CBLAS declarations used only to compile the reference's C sources
 * (lila-c/*.c) into oracle/_ref/ for parity checking.  The enum values are the
 * standard CBLAS ones; each routine is mapped onto the scipy_-prefixed LP64
 * symbols exported by scipy's bundled OpenBLAS.  Test infrastructure only. */
#ifndef ORACLE_REF_SHIM_CBLAS_H
#define ORACLE_REF_SHIM_CBLAS_H
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
enum CBLAS_UPLO { CblasUpper = 121, CblasLower = 122 };
enum CBLAS_DIAG { CblasNonUnit = 131, CblasUnit = 132 };
enum CBLAS_SIDE { CblasLeft = 141, CblasRight = 142 };
typedef enum CBLAS_ORDER CBLAS_LAYOUT;

#define cblas_dgemm scipy_cblas_dgemm
#define cblas_dtrmm scipy_cblas_dtrmm
#define cblas_dtrsm scipy_cblas_dtrsm
#define cblas_dsyrk scipy_cblas_dsyrk
#define cblas_dger  scipy_cblas_dger
#define cblas_ddot  scipy_cblas_ddot
#define cblas_dnrm2 scipy_cblas_dnrm2

void cblas_dgemm(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, enum CBLAS_TRANSPOSE, int, int, int,
                 double, const double *, int, const double *, int, double, double *, int);
void cblas_dtrmm(enum CBLAS_ORDER, enum CBLAS_SIDE, enum CBLAS_UPLO, enum CBLAS_TRANSPOSE,
                 enum CBLAS_DIAG, int, int, double, const double *, int, double *, int);
void cblas_dtrsm(enum CBLAS_ORDER, enum CBLAS_SIDE, enum CBLAS_UPLO, enum CBLAS_TRANSPOSE,
                 enum CBLAS_DIAG, int, int, double, const double *, int, double *, int);
void cblas_dsyrk(enum CBLAS_ORDER, enum CBLAS_UPLO, enum CBLAS_TRANSPOSE, int, int,
                 double, const double *, int, double, double *, int);
void cblas_dger(enum CBLAS_ORDER, int, int, double, const double *, int, const double *, int,
                double *, int);
double cblas_ddot(int, const double *, int, const double *, int);
double cblas_dnrm2(int, const double *, int);
#endif
