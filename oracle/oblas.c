/*
 * oblas.c -- the oracle's own small FP64 BLAS/LAPACK subset.
 *
 * TEST INFRASTRUCTURE ONLY.  This file belongs to the CPU oracle: it is
 * compiled into oracle/liblila_oracle*.so and loaded by tests/ and by
 * bench.py's cpu_baseline leg; the GPU product never links or calls it.
 *
 * The reference (lila-c/*.c) is written on top of CBLAS + LAPACKE.  Those
 * libraries are not part of the reference checkout, so the oracle restates
 * the published algorithms of the routines it calls (column-major, LP64):
 *   BLAS-3  dgemm, dtrmm, dtrsm, dsyrk      (reference BLAS semantics)
 *   BLAS-2  dger
 *   BLAS-1  ddot, dnrm2 (scaled sum of squares)
 *   LAPACK  dlarfg, dgeqr2, dlarft('F','C'), dorg2r, dpotrf('U'), dlapy2
 * With -DORACLE_EXTERNAL_BLAS the BLAS-3/2/1 routines forward to scipy's
 * bundled OpenBLAS (scipy_cblas_*), which is only used to time the CPU
 * baseline at large sizes; the LAPACK-level routines stay the restatement.
 */
#include "oblas.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef ORACLE_EXTERNAL_BLAS
/* scipy's OpenBLAS, standard CBLAS enum values. */
void scipy_cblas_dgemm(int, int, int, int, int, int, double, const double *, int, const double *,
                       int, double, double *, int);
void scipy_cblas_dtrmm(int, int, int, int, int, int, int, double, const double *, int, double *,
                       int);
void scipy_cblas_dtrsm(int, int, int, int, int, int, int, double, const double *, int, double *,
                       int);
void scipy_cblas_dsyrk(int, int, int, int, int, double, const double *, int, double, double *, int);
void scipy_cblas_dger(int, int, int, double, const double *, int, const double *, int, double *,
                      int);
double scipy_cblas_ddot(int, const double *, int, const double *, int);
#define CB_COL 102
#define CB_T(t) ((t) == OB_T ? 112 : 111)
#define CB_UPLO(u) ((u) == OB_UPPER ? 121 : 122)
#define CB_DIAG(d) ((d) == OB_UNIT ? 132 : 131)
#define CB_SIDE(s) ((s) == OB_LEFT ? 141 : 142)
#endif

#define IDX(M, r, c, ld) ((M)[(size_t)(r) + (size_t)(c) * (size_t)(ld)])

/* C := alpha*op(A)*op(B) + beta*C ; op(A) is m x k, op(B) is k x n. */
void ob_dgemm(int ta, int tb, int m, int n, int k, double alpha, const double *A, int lda,
              const double *B, int ldb, double beta, double *C, int ldc)
{
    if (m <= 0 || n <= 0) return;
#ifdef ORACLE_EXTERNAL_BLAS
    if (k > 0) {
        scipy_cblas_dgemm(CB_COL, CB_T(ta), CB_T(tb), m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
        return;
    }
#endif
#pragma omp parallel for schedule(static) if ((double)m * n * (k + 1) > 4e6)
    for (int j = 0; j < n; j++) {
        double *cj = &IDX(C, 0, j, ldc);
        if (beta == 0.0) {
            for (int i = 0; i < m; i++) cj[i] = 0.0;
        } else if (beta != 1.0) {
            for (int i = 0; i < m; i++) cj[i] *= beta;
        }
        if (alpha == 0.0 || k <= 0) continue;
        if (ta == OB_N) {
            for (int p = 0; p < k; p++) {
                double b = (tb == OB_N) ? IDX(B, p, j, ldb) : IDX(B, j, p, ldb);
                double s = alpha * b;
                if (s == 0.0) continue;
                const double *ap = &IDX(A, 0, p, lda);
                for (int i = 0; i < m; i++) cj[i] += s * ap[i];
            }
        } else {
            for (int i = 0; i < m; i++) {
                const double *ai = &IDX(A, 0, i, lda);
                double s = 0.0;
                if (tb == OB_N) {
                    const double *bj = &IDX(B, 0, j, ldb);
                    for (int p = 0; p < k; p++) s += ai[p] * bj[p];
                } else {
                    for (int p = 0; p < k; p++) s += ai[p] * IDX(B, j, p, ldb);
                }
                cj[i] += alpha * s;
            }
        }
    }
}

/* Element of op(Tri) with triangle/diag conventions applied (k x k). */
static inline double tri_el(int uplo, int trans, int diag, const double *A, int lda, int r, int c)
{
    int sr = trans == OB_T ? c : r;
    int sc = trans == OB_T ? r : c;
    if (sr == sc) return diag == OB_UNIT ? 1.0 : IDX(A, sr, sc, lda);
    if (uplo == OB_UPPER ? (sr < sc) : (sr > sc)) return IDX(A, sr, sc, lda);
    return 0.0;
}

/* B := alpha*op(A)*B (side L) or alpha*B*op(A) (side R), A triangular. */
void ob_dtrmm(int side, int uplo, int ta, int diag, int m, int n, double alpha, const double *A,
              int lda, double *B, int ldb)
{
    if (m <= 0 || n <= 0) return;
#ifdef ORACLE_EXTERNAL_BLAS
    scipy_cblas_dtrmm(CB_COL, CB_SIDE(side), CB_UPLO(uplo), CB_T(ta), CB_DIAG(diag), m, n, alpha,
                      A, lda, B, ldb);
    return;
#endif
    if (side == OB_LEFT) {
        /* effective op(A) is lower when (uplo==L, N) or (uplo==U, T) */
        int eff_lower = (uplo == OB_LOWER) == (ta == OB_N);
        double *col = (double *)malloc(sizeof(double) * (size_t)m);
        for (int j = 0; j < n; j++) {
            double *bj = &IDX(B, 0, j, ldb);
            for (int r = 0; r < m; r++) {
                double s = 0.0;
                int lo = eff_lower ? 0 : r, hi = eff_lower ? r : m - 1;
                for (int c = lo; c <= hi; c++) s += tri_el(uplo, ta, diag, A, lda, r, c) * bj[c];
                col[r] = alpha * s;
            }
            memcpy(bj, col, sizeof(double) * (size_t)m);
        }
        free(col);
    } else {
        int eff_lower = (uplo == OB_LOWER) == (ta == OB_N);
        double *row = (double *)malloc(sizeof(double) * (size_t)n);
        for (int i = 0; i < m; i++) {
            for (int c = 0; c < n; c++) {
                double s = 0.0;
                int lo = eff_lower ? c : 0, hi = eff_lower ? n - 1 : c;
                for (int r = lo; r <= hi; r++)
                    s += IDX(B, i, r, ldb) * tri_el(uplo, ta, diag, A, lda, r, c);
                row[c] = alpha * s;
            }
            for (int c = 0; c < n; c++) IDX(B, i, c, ldb) = row[c];
        }
        free(row);
    }
}

/* Solve op(A)*X = alpha*B (side L) or X*op(A) = alpha*B (side R); X overwrites B. */
void ob_dtrsm(int side, int uplo, int ta, int diag, int m, int n, double alpha, const double *A,
              int lda, double *B, int ldb)
{
    if (m <= 0 || n <= 0) return;
#ifdef ORACLE_EXTERNAL_BLAS
    scipy_cblas_dtrsm(CB_COL, CB_SIDE(side), CB_UPLO(uplo), CB_T(ta), CB_DIAG(diag), m, n, alpha,
                      A, lda, B, ldb);
    return;
#endif
    int eff_lower = (uplo == OB_LOWER) == (ta == OB_N);
    if (side == OB_LEFT) {
        for (int j = 0; j < n; j++) {
            double *x = &IDX(B, 0, j, ldb);
            for (int r = 0; r < m; r++) x[r] *= alpha;
            if (eff_lower) {
                for (int r = 0; r < m; r++) {
                    double s = x[r];
                    for (int c = 0; c < r; c++) s -= tri_el(uplo, ta, diag, A, lda, r, c) * x[c];
                    x[r] = s / tri_el(uplo, ta, diag, A, lda, r, r);
                }
            } else {
                for (int r = m - 1; r >= 0; r--) {
                    double s = x[r];
                    for (int c = r + 1; c < m; c++) s -= tri_el(uplo, ta, diag, A, lda, r, c) * x[c];
                    x[r] = s / tri_el(uplo, ta, diag, A, lda, r, r);
                }
            }
        }
    } else {
#pragma omp parallel for schedule(static) if ((double)m * n * n > 4e6)
        for (int i = 0; i < m; i++) {
            /* row vector x solves x*op(A) = alpha*b */
            if (!eff_lower) {
                for (int c = 0; c < n; c++) {
                    double s = alpha * IDX(B, i, c, ldb);
                    for (int r = 0; r < c; r++)
                        s -= IDX(B, i, r, ldb) * tri_el(uplo, ta, diag, A, lda, r, c);
                    IDX(B, i, c, ldb) = s / tri_el(uplo, ta, diag, A, lda, c, c);
                }
            } else {
                for (int c = n - 1; c >= 0; c--) {
                    double s = alpha * IDX(B, i, c, ldb);
                    for (int r = c + 1; r < n; r++)
                        s -= IDX(B, i, r, ldb) * tri_el(uplo, ta, diag, A, lda, r, c);
                    IDX(B, i, c, ldb) = s / tri_el(uplo, ta, diag, A, lda, c, c);
                }
            }
        }
    }
}

/* C := alpha*A^T*A + beta*C (trans==T, A is k x n) on the 'uplo' triangle of C (n x n). */
void ob_dsyrk(int uplo, int ta, int n, int k, double alpha, const double *A, int lda, double beta,
              double *C, int ldc)
{
    if (n <= 0) return;
#ifdef ORACLE_EXTERNAL_BLAS
    scipy_cblas_dsyrk(CB_COL, CB_UPLO(uplo), CB_T(ta), n, k, alpha, A, lda, beta, C, ldc);
    return;
#endif
#pragma omp parallel for schedule(dynamic) if ((double)n * n * k > 4e6)
    for (int j = 0; j < n; j++) {
        int lo = uplo == OB_UPPER ? 0 : j, hi = uplo == OB_UPPER ? j : n - 1;
        for (int i = lo; i <= hi; i++) {
            double s = 0.0;
            if (ta == OB_T) {
                const double *ai = &IDX(A, 0, i, lda), *aj = &IDX(A, 0, j, lda);
                for (int p = 0; p < k; p++) s += ai[p] * aj[p];
            } else {
                for (int p = 0; p < k; p++) s += IDX(A, i, p, lda) * IDX(A, j, p, lda);
            }
            double c = beta == 0.0 ? 0.0 : beta * IDX(C, i, j, ldc);
            IDX(C, i, j, ldc) = c + alpha * s;
        }
    }
}

/* A := alpha*x*y^T + A, x length m (stride incx), y length n (stride incy). */
void ob_dger(int m, int n, double alpha, const double *x, int incx, const double *y, int incy,
             double *A, int lda)
{
    if (m <= 0 || n <= 0) return;
#ifdef ORACLE_EXTERNAL_BLAS
    scipy_cblas_dger(CB_COL, m, n, alpha, x, incx, y, incy, A, lda);
    return;
#endif
    for (int j = 0; j < n; j++) {
        double s = alpha * y[(size_t)j * incy];
        for (int i = 0; i < m; i++) IDX(A, i, j, lda) += x[(size_t)i * incx] * s;
    }
}

double ob_ddot(int n, const double *x, int incx, const double *y, int incy)
{
#ifdef ORACLE_EXTERNAL_BLAS
    return scipy_cblas_ddot(n, x, incx, y, incy);
#endif
    double s = 0.0;
    for (int i = 0; i < n; i++) s += x[(size_t)i * incx] * y[(size_t)i * incy];
    return s;
}

/* Euclidean norm by the scaled sum of squares (reference BLAS dnrm2 method). */
double ob_dnrm2(int n, const double *x, int incx)
{
    double scale = 0.0, ssq = 1.0;
    for (int i = 0; i < n; i++) {
        double v = x[(size_t)i * incx];
        if (v != 0.0) {
            double a = fabs(v);
            if (scale < a) {
                ssq = 1.0 + ssq * (scale / a) * (scale / a);
                scale = a;
            } else {
                ssq += (a / scale) * (a / scale);
            }
        }
    }
    return scale * sqrt(ssq);
}

double ob_dlapy2(double x, double y)
{
    double xa = fabs(x), ya = fabs(y);
    double w = xa > ya ? xa : ya, z = xa > ya ? ya : xa;
    if (w == 0.0 || z == 0.0) return w;
    return w * sqrt(1.0 + (z / w) * (z / w));
}

/*
 * Elementary reflector H = I - tau*[1;v]*[1;v]^T with H*[alpha;x] = [beta;0]
 * (LAPACK dlarfg: beta = -sign(alpha)*||[alpha;x]||, tau = (beta-alpha)/beta,
 * v = x/(alpha-beta); tau = 0 when x == 0).  Includes LAPACK's rescaling for
 * |beta| below the safe minimum.
 */
void ob_dlarfg(int n, double *alpha, double *x, int incx, double *tau)
{
    if (n <= 1) {
        *tau = 0.0;
        return;
    }
    double xnorm = ob_dnrm2(n - 1, x, incx);
    if (xnorm == 0.0) {
        *tau = 0.0;
        return;
    }
    double beta = -copysign(ob_dlapy2(*alpha, xnorm), *alpha);
    const double safmin = 2.2250738585072014e-308 / 1.1102230246251565e-16;
    int knt = 0;
    if (fabs(beta) < safmin) {
        double rsafmn = 1.0 / safmin;
        do {
            knt++;
            for (int i = 0; i < n - 1; i++) x[(size_t)i * incx] *= rsafmn;
            beta *= rsafmn;
            *alpha *= rsafmn;
        } while (fabs(beta) < safmin && knt < 20);
        xnorm = ob_dnrm2(n - 1, x, incx);
        beta = -copysign(ob_dlapy2(*alpha, xnorm), *alpha);
    }
    *tau = (beta - *alpha) / beta;
    double s = 1.0 / (*alpha - beta);
    for (int i = 0; i < n - 1; i++) x[(size_t)i * incx] *= s;
    for (int j = 0; j < knt; j++) beta *= safmin;
    *alpha = beta;
}

/* Unblocked Householder QR (LAPACK dgeqr2 algorithm); tau has min(m,n) entries. */
void ob_dgeqr2(int m, int n, double *A, int lda, double *tau)
{
    int k = m < n ? m : n;
    double *w = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < k; i++) {
        double *aii = &IDX(A, i, i, lda);
        int nx = i + 1 < m ? i + 1 : m - 1;
        ob_dlarfg(m - i, aii, &IDX(A, nx, i, lda), 1, &tau[i]);
        if (i + 1 < n && tau[i] != 0.0) {
            /* apply H_i to A[i:m, i+1:n] from the left: w = A^T v ; A -= tau v w^T */
            double save = *aii;
            *aii = 1.0;
            int nc = n - i - 1;
            for (int c = 0; c < nc; c++)
                w[c] = ob_ddot(m - i, aii, 1, &IDX(A, i, i + 1 + c, lda), 1);
            for (int c = 0; c < nc; c++) {
                double s = tau[i] * w[c];
                double *ac = &IDX(A, i, i + 1 + c, lda);
                for (int r = 0; r < m - i; r++) ac[r] -= aii[r] * s;
            }
            *aii = save;
        }
    }
    free(w);
}

/*
 * Triangular factor T (k x k, upper) of H(1)...H(k) = I - V*T*V^T, forward
 * direction, columnwise storage (LAPACK dlarft 'F','C').  V is n x k with
 * unit diagonal implied; entries above the diagonal are not referenced.
 */
void ob_dlarft_fc(int n, int k, const double *V, int ldv, const double *tau, double *T, int ldt)
{
    for (int i = 0; i < k; i++) {
        if (tau[i] == 0.0) {
            for (int r = 0; r <= i; r++) IDX(T, r, i, ldt) = 0.0;
            continue;
        }
        /* T(0:i, i) = -tau(i) * V(i:n, 0:i)^T * V(i:n, i)  (V(i,i) = 1) */
        for (int r = 0; r < i; r++) {
            double s = IDX(V, i, r, ldv); /* row i of column r times the implied 1 */
            for (int p = i + 1; p < n; p++) s += IDX(V, p, r, ldv) * IDX(V, p, i, ldv);
            IDX(T, r, i, ldt) = -tau[i] * s;
        }
        /* T(0:i, i) = T(0:i, 0:i) * T(0:i, i) (upper triangular, non-unit) */
        for (int r = 0; r < i; r++) {
            double s = 0.0;
            for (int c = r; c < i; c++) s += IDX(T, r, c, ldt) * IDX(T, c, i, ldt);
            IDX(T, r, i, ldt) = s;
        }
        IDX(T, i, i, ldt) = tau[i];
    }
}

/* Explicit Q (m x n) from the first k reflectors stored in A (LAPACK dorg2r algorithm). */
void ob_dorg2r(int m, int n, int k, double *A, int lda, const double *tau)
{
    if (n <= 0) return;
    for (int j = k; j < n; j++) {
        for (int l = 0; l < m; l++) IDX(A, l, j, lda) = 0.0;
        IDX(A, j, j, lda) = 1.0;
    }
    double *w = (double *)malloc(sizeof(double) * (size_t)n);
    for (int i = k - 1; i >= 0; i--) {
        if (i < n - 1) {
            /* apply H(i) to A(i:m, i+1:n) from the left */
            IDX(A, i, i, lda) = 1.0;
            int nc = n - i - 1;
            for (int c = 0; c < nc; c++)
                w[c] = ob_ddot(m - i, &IDX(A, i, i, lda), 1, &IDX(A, i, i + 1 + c, lda), 1);
            for (int c = 0; c < nc; c++) {
                double s = tau[i] * w[c];
                for (int r = 0; r < m - i; r++) IDX(A, i + r, i + 1 + c, lda) -= IDX(A, i + r, i, lda) * s;
            }
        }
        if (i < m - 1)
            for (int r = i + 1; r < m; r++) IDX(A, r, i, lda) *= -tau[i];
        IDX(A, i, i, lda) = 1.0 - tau[i];
        for (int l = 0; l < i; l++) IDX(A, l, i, lda) = 0.0;
    }
    free(w);
}

/* Cholesky A = U^T U, upper triangle in place (LAPACK dpotrf 'U', unblocked). Returns info. */
int ob_dpotrf_upper(int n, double *A, int lda)
{
    for (int j = 0; j < n; j++) {
        double d = IDX(A, j, j, lda);
        for (int p = 0; p < j; p++) d -= IDX(A, p, j, lda) * IDX(A, p, j, lda);
        if (!(d > 0.0)) {
            IDX(A, j, j, lda) = d;
            return j + 1;
        }
        d = sqrt(d);
        IDX(A, j, j, lda) = d;
        for (int c = j + 1; c < n; c++) {
            double s = IDX(A, j, c, lda);
            for (int p = 0; p < j; p++) s -= IDX(A, p, j, lda) * IDX(A, p, c, lda);
            IDX(A, j, c, lda) = s / d;
        }
    }
    return 0;
}

void ob_dlacpy(int m, int n, const double *A, int lda, double *B, int ldb)
{
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++) IDX(B, i, j, ldb) = IDX(A, i, j, lda);
}

double ob_dlange_fro(int m, int n, const double *A, int lda)
{
    double scale = 0.0, ssq = 1.0;
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++) {
            double a = fabs(IDX(A, i, j, lda));
            if (a != 0.0) {
                if (scale < a) {
                    ssq = 1.0 + ssq * (scale / a) * (scale / a);
                    scale = a;
                } else {
                    ssq += (a / scale) * (a / scale);
                }
            }
        }
    return scale * sqrt(ssq);
}

/*
 * Double-double accumulation of dot products (TwoProd by fma, TwoSum), used by
 * the oracle to produce reference values accurate to ~2^-100 for checking the
 * split-precision products; result rounded to double.
 */
static inline void two_sum(double a, double b, double *s, double *e)
{
    double x = a + b, z = x - a;
    *e = (a - (x - z)) + (b - z);
    *s = x;
}

double ob_ddot_dd(int n, const double *x, int incx, const double *y, int incy)
{
    double sh = 0.0, sl = 0.0;
    for (int i = 0; i < n; i++) {
        double a = x[(size_t)i * incx], b = y[(size_t)i * incy];
        double p = a * b, pe = fma(a, b, -p);
        double t, te;
        two_sum(sh, p, &t, &te);
        sl += te + pe;
        two_sum(t, sl, &sh, &sl);
    }
    return sh + sl;
}

/* C = op(A) * B with every entry a double-double dot product (A^T if ta). */
void ob_dgemm_dd(int ta, int m, int n, int k, const double *A, int lda, const double *B, int ldb,
                 double *C, int ldc)
{
#pragma omp parallel for schedule(static)
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++) {
            const double *ai = ta ? &A[(size_t)i * lda] : &A[i];
            int inca = ta ? 1 : lda;
            C[(size_t)i + (size_t)j * ldc] = ob_ddot_dd(k, ai, inca, &B[(size_t)j * ldb], 1);
        }
}
