/* Minimal LAPACKE declarations used only to compile the reference's C sources
 * into oracle/_ref/ (test infrastructure).  Names map onto scipy's bundled
 * OpenBLAS (LP64, scipy_ prefix). */
#ifndef ORACLE_REF_SHIM_LAPACKE_H
#define ORACLE_REF_SHIM_LAPACKE_H
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
typedef int lapack_int;

#define LAPACKE_dgeqrf_work scipy_LAPACKE_dgeqrf_work
#define LAPACKE_dlacpy      scipy_LAPACKE_dlacpy
#define LAPACKE_dlacpy_work scipy_LAPACKE_dlacpy_work
#define LAPACKE_dlange_work scipy_LAPACKE_dlange_work
#define LAPACKE_dlantr_work scipy_LAPACKE_dlantr_work
#define LAPACKE_dlarfg_work scipy_LAPACKE_dlarfg_work
#define LAPACKE_dlarft_work scipy_LAPACKE_dlarft_work
#define LAPACKE_dlaset      scipy_LAPACKE_dlaset
#define LAPACKE_dorgqr_work scipy_LAPACKE_dorgqr_work
#define LAPACKE_dormqr_work scipy_LAPACKE_dormqr_work
#define LAPACKE_dpotrf      scipy_LAPACKE_dpotrf
#define LAPACKE_dlapy2      oracle_ref_dlapy2

lapack_int LAPACKE_dgeqrf_work(int, lapack_int, lapack_int, double *, lapack_int, double *, double *, lapack_int);
lapack_int LAPACKE_dlacpy(int, char, lapack_int, lapack_int, const double *, lapack_int, double *, lapack_int);
lapack_int LAPACKE_dlacpy_work(int, char, lapack_int, lapack_int, const double *, lapack_int, double *, lapack_int);
double LAPACKE_dlange_work(int, char, lapack_int, lapack_int, const double *, lapack_int, double *);
double LAPACKE_dlantr_work(int, char, char, char, lapack_int, lapack_int, const double *, lapack_int, double *);
lapack_int LAPACKE_dlarfg_work(lapack_int, double *, double *, lapack_int, double *);
lapack_int LAPACKE_dlarft_work(int, char, char, lapack_int, lapack_int, const double *, lapack_int, const double *, double *, lapack_int);
lapack_int LAPACKE_dlaset(int, char, lapack_int, lapack_int, double, double, double *, lapack_int);
lapack_int LAPACKE_dorgqr_work(int, lapack_int, lapack_int, lapack_int, double *, lapack_int, const double *, double *, lapack_int);
lapack_int LAPACKE_dormqr_work(int, char, char, lapack_int, lapack_int, lapack_int, const double *, lapack_int, const double *, double *, lapack_int, double *, lapack_int);
lapack_int LAPACKE_dpotrf(int, char, lapack_int, double *, lapack_int);
#include <math.h>
static inline double oracle_ref_dlapy2(double x, double y) { return hypot(x, y); }
#endif
