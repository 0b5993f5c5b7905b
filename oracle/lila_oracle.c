/*
 * lila_oracle.c -- CPU restatement of the reference's w03 Householder-QR family.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle: tests/, __graft_entry__.smoke()
 * and bench.py's cpu_baseline / reference leg are the only callers.  It is the
 * checker, never the product; the GPU library (lila_gb300/) does not link it.
 *
 * Every routine restates the algorithm of the reference routine named in its
 * comment (file:line in the langou/lila checkout), in column-major FP64 with
 * LP64 ints, with the same argument lists and the same global-index T layout:
 * T is mt x (n+ii); the compact-WY factor of the reflectors [a, b) that share
 * the global tile floor(a/mt) sits at T + (a % mt) + a*ldt.
 *
 * BLAS/LAPACK calls go to the oracle's own subset (oblas.c).  Known defects
 * of the reference are NOT reproduced; each difference is listed here:
 *   - lila_dgeqrf_w03_mt_hr.c:8 / lila_ormhr2_w03_hr.c:10 put the sign vector
 *     S and the scratch work2 at the same address, which corrupts S once a
 *     leaf spans >= 3 mt tiles.  Here S lives at work[0 : i+n] and the tile
 *     routine's scratch starts after it, so they never overlap.
 *   - lila_query_dgeqrf_w03_mt_hr.c:16 under-counts (it omits S); the query
 *     here adds i+n doubles for S.
 * Parity with the reference is pinned by tests/test_oracle_pin.py (against
 * the reference compiled into oracle/_ref/ in the development container) and
 * by the committed fixtures in tests/golden/.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oblas.h"

#define EL(M, r, c, ld) ((M)[(size_t)(r) + (size_t)(c) * (size_t)(ld)])

static int imin(int a, int b) { return a < b ? a : b; }
static int imax(int a, int b) { return a > b ? a : b; }

/* End of the reflector tile that starts at column a, clipped to `end`. */
static int tile_end(int a, int end, int mt)
{
    int b = (a / mt + 1) * mt;
    return b < end ? b : end;
}

/* ------------------------------------------------------------------------ */
/* Block reflector applications                                             */
/* ------------------------------------------------------------------------ */

/*
 * C := H^T C for the reflectors [i, i+k) stored in A (unit lower trapezoid),
 * tile by tile in increasing order; C is addressed with the global row index
 * (row r of the block is C[r]).  One tile [a, b) is the LAPACK 'L','T'
 * forward-columnwise block-reflector step:
 *   W = V^T C(a:m) ; W = T^T W ; C(a:m) -= V W.
 * Restates lila-c/lila_dormqrf_w03.c:15-76 and lila_dormqrf_z03.c:11-67.
 */
static void apply_qt_tiles(int m, int n, int k, int i, int mt, const double *A, int lda,
                           const double *T, int ldt, double *C, int ldc, double *W)
{
    for (int a = i; a < i + k;) {
        int b = tile_end(a, i + k, mt), vb = b - a;
        const double *V = &EL(A, a, a, lda);
        const double *Tt = &EL(T, a % mt, a, ldt);
        double *Ct = C + a;
        ob_dlacpy(vb, n, Ct, ldc, W, mt);
        ob_dtrmm(OB_LEFT, OB_LOWER, OB_T, OB_UNIT, vb, n, 1.0, V, lda, W, mt);
        ob_dgemm(OB_T, OB_N, vb, n, m - b, 1.0, V + vb, lda, Ct + vb, ldc, 1.0, W, mt);
        ob_dtrmm(OB_LEFT, OB_UPPER, OB_T, OB_NONUNIT, vb, n, 1.0, Tt, ldt, W, mt);
        ob_dgemm(OB_N, OB_N, m - b, n, vb, -1.0, V + vb, lda, W, mt, 1.0, Ct + vb, ldc);
        ob_dtrmm(OB_LEFT, OB_LOWER, OB_N, OB_UNIT, vb, n, 1.0, V, lda, W, mt);
        for (int c = 0; c < n; c++)
            for (int r = 0; r < vb; r++) EL(Ct, r, c, ldc) -= EL(W, r, c, mt);
        a = b;
    }
}

/* lila-c/lila_dormqrf_w03.c:3 -- apply H^T to A(i:m, j:j+n) in place. */
int oracle_dormqrf_w03(int m, int n, int k, int i, int j, int mt, double *A, int lda, double *T,
                       int ldt, double *work, int lwork)
{
    (void)lwork;
    apply_qt_tiles(m, n, k, i, mt, A, lda, T, ldt, A + (size_t)j * lda, lda, work);
    return 0;
}

/* lila-c/lila_dormqrf_z03.c:3 -- apply H^T to a separate block B(i:m, j:j+n). */
int oracle_dormqrf_z03(int m, int n, int k, int i, int j, int mt, double *A, int lda, double *T,
                       int ldt, double *B, int ldb, double *work, int lwork)
{
    (void)lwork;
    apply_qt_tiles(m, n, k, i, mt, A, lda, T, ldt, B + (size_t)j * ldb, ldb, work);
    return 0;
}

/*
 * Q(i:m, j:j+n) := H [0 ; Q(i+k:m, j:j+n)] for the reflectors [i, i+k), tiles
 * in decreasing order.  Rows [a, b) of the tile being applied are still zero,
 * so each step is  W = V(b:m)^T X(b:m) ; W = T W ; X(a:b) = -V1 W ;
 * X(b:m) -= V(b:m) W.   Restates lila-c/lila_dormqrbz_w03.c:12-62.
 * Argument order follows the definition (Q before T), as every caller does.
 */
int oracle_dormqrbz_w03(int m, int n, int k, int i, int j, int mt, double *A, int lda, double *Q,
                        int ldq, double *T, int ldt, double *work, int lwork)
{
    (void)lwork;
    if (k <= 0) return 0;
    int ntile = 0;
    for (int a = i; a < i + k; a = tile_end(a, i + k, mt)) ntile++;
    int *starts = (int *)malloc(sizeof(int) * (size_t)(ntile + 1));
    ntile = 0;
    for (int a = i; a < i + k; a = tile_end(a, i + k, mt)) starts[ntile++] = a;
    starts[ntile] = i + k;
    double *X = Q + (size_t)j * ldq;
    int ldw = k;
    for (int t = ntile - 1; t >= 0; t--) {
        int a = starts[t], b = starts[t + 1], vb = b - a;
        const double *Vtop = &EL(A, a, a, lda);
        const double *Vbot = &EL(A, b, a, lda);
        const double *Tt = &EL(T, a % mt, a, ldt);
        ob_dgemm(OB_T, OB_N, vb, n, m - b, 1.0, Vbot, lda, X + b, ldq, 0.0, work, ldw);
        ob_dtrmm(OB_LEFT, OB_UPPER, OB_N, OB_NONUNIT, vb, n, 1.0, Tt, ldt, work, ldw);
        ob_dlacpy(vb, n, work, ldw, X + a, ldq);
        ob_dtrmm(OB_LEFT, OB_LOWER, OB_N, OB_UNIT, vb, n, -1.0, Vtop, lda, X + a, ldq);
        ob_dgemm(OB_N, OB_N, m - b, n, vb, -1.0, Vbot, lda, work, ldw, 1.0, X + b, ldq);
    }
    free(starts);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* T factors                                                                */
/* ------------------------------------------------------------------------ */

/*
 * Couple the reflectors [i, i+vb) (vb = part of the block [i, i+n) in i's
 * tile) to the earlier reflectors [i-wb, i) of the same tile:
 *   T12 = -T11 (V1^T V2) T22.
 * wb reaches back to j when j shares i's tile, else to the tile start.
 * Restates lila-c/lila_dlarft_connect_w03.c:3-32.
 */
int oracle_dlarft_connect_w03(int m, int n, int i, int j, int mt, double *A, int lda, double *T,
                              int ldt)
{
    int vb = imin(mt - i % mt, n);
    int wb = (j / mt == i / mt) ? i - j : i % mt;
    if (wb == mt) wb = 1;
    if (wb <= 0 || vb <= 0) return 0;
    const double *Aii = &EL(A, i, i, lda);
    const double *Aij = &EL(A, i, i - wb, lda);
    double *Tki = &EL(T, i % mt, i, ldt);
    double *Tji = &EL(T, i % mt - wb, i, ldt);
    double *Tjj = &EL(T, i % mt - wb, i - wb, ldt);
    for (int c = 0; c < vb; c++)
        for (int r = 0; r < wb; r++) EL(Tji, r, c, ldt) = EL(Aij, c, r, lda);
    ob_dtrmm(OB_RIGHT, OB_LOWER, OB_N, OB_UNIT, wb, vb, 1.0, Aii, lda, Tji, ldt);
    ob_dgemm(OB_T, OB_N, wb, vb, m - vb - i, 1.0, Aij + vb, lda, Aii + vb, lda, 1.0, Tji, ldt);
    ob_dtrmm(OB_LEFT, OB_UPPER, OB_N, OB_NONUNIT, wb, vb, -1.0, Tjj, ldt, Tji, ldt);
    ob_dtrmm(OB_RIGHT, OB_UPPER, OB_N, OB_NONUNIT, wb, vb, 1.0, Tki, ldt, Tji, ldt);
    return 0;
}

/*
 * T tiles of the reflectors [i, i+n) from V and tau, one LAPACK dlarft('F','C')
 * per tile segment.  Restates lila-c/lila_dlarft_w03.c:3-55.
 */
int oracle_dlarft_w03(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                      double *tau)
{
    for (int a = i; a < i + n;) {
        int b = tile_end(a, i + n, mt);
        ob_dlarft_fc(m - a, b - a, &EL(A, a, a, lda), lda, tau + (a - i), &EL(T, a % mt, a, ldt), ldt);
        a = b;
    }
    return 0;
}

/* tau = diag(T) per tile.  Restates lila-c/lila_dT2tau_w03.c:3-35. */
int oracle_dT2tau_w03(int m, int n, int i, int mt, double *T, int ldt, double *tau)
{
    (void)m;
    for (int c = i; c < i + n; c++) tau[c - i] = EL(T, c % mt, c, ldt);
    return 0;
}

/* tau = 2 / (1 + ||v||^2).  Restates lila-c/lila_dV2tau_w03.c:3-34. */
int oracle_dV2tau_w03(int m, int n, int i, int mt, double *A, int lda, double *tau)
{
    (void)mt;
    for (int c = i; c < i + n; c++) {
        const double *v = &EL(A, c + 1, c, lda);
        tau[c - i] = 2.0 / (1.0 + ob_ddot(m - c - 1, v, 1, v, 1));
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Panels                                                                   */
/* ------------------------------------------------------------------------ */

/*
 * Recursive Householder QR of an m x n panel with its n x n T (Elmroth and
 * Gustavson).  T's strictly upper part doubles as the workspace W of the
 * left-half update.  Restates lila-c/dgeqr3.c:3-114.
 */
int oracle_dgeqr3(int m, int n, double *A, int lda, double *T, int ldt)
{
    if (n <= 0) return 0;
    if (n == 1) {
        int nx = m > 1 ? 1 : 0;
        ob_dlarfg(m, &A[0], &A[nx], 1, &T[0]);
        return 0;
    }
    int n1 = n / 2, n2 = n - n1;
    oracle_dgeqr3(m, n1, A, lda, T, ldt);
    double *W = &EL(T, 0, n1, ldt);
    /* A(:, n1:n) := H1^T A(:, n1:n) */
    for (int c = 0; c < n2; c++)
        for (int r = 0; r < n1; r++) EL(W, r, c, ldt) = EL(A, r, n1 + c, lda);
    ob_dtrmm(OB_LEFT, OB_LOWER, OB_T, OB_UNIT, n1, n2, 1.0, A, lda, W, ldt);
    ob_dgemm(OB_T, OB_N, n1, n2, m - n1, 1.0, &EL(A, n1, 0, lda), lda, &EL(A, n1, n1, lda), lda, 1.0, W, ldt);
    ob_dtrmm(OB_LEFT, OB_UPPER, OB_T, OB_NONUNIT, n1, n2, 1.0, T, ldt, W, ldt);
    ob_dgemm(OB_N, OB_N, m - n1, n2, n1, -1.0, &EL(A, n1, 0, lda), lda, W, ldt, 1.0, &EL(A, n1, n1, lda), lda);
    ob_dtrmm(OB_LEFT, OB_LOWER, OB_N, OB_UNIT, n1, n2, 1.0, A, lda, W, ldt);
    for (int c = 0; c < n2; c++)
        for (int r = 0; r < n1; r++) EL(A, r, n1 + c, lda) -= EL(W, r, c, ldt);
    oracle_dgeqr3(m - n1, n2, &EL(A, n1, n1, lda), lda, &EL(T, n1, n1, ldt), ldt);
    /* T12 = -T1 (Y1^T Y2) T2 */
    for (int r = 0; r < n1; r++)
        for (int c = 0; c < n2; c++) EL(T, r, n1 + c, ldt) = EL(A, n1 + c, r, lda);
    ob_dtrmm(OB_RIGHT, OB_LOWER, OB_N, OB_UNIT, n1, n2, 1.0, &EL(A, n1, n1, lda), lda, &EL(T, 0, n1, ldt), ldt);
    ob_dgemm(OB_T, OB_N, n1, n2, m - n, 1.0, &EL(A, n, 0, lda), lda, &EL(A, n, n1, lda), lda, 1.0, &EL(T, 0, n1, ldt), ldt);
    ob_dtrmm(OB_LEFT, OB_UPPER, OB_N, OB_NONUNIT, n1, n2, -1.0, T, ldt, &EL(T, 0, n1, ldt), ldt);
    ob_dtrmm(OB_RIGHT, OB_UPPER, OB_N, OB_NONUNIT, n1, n2, 1.0, &EL(T, n1, n1, ldt), ldt, &EL(T, 0, n1, ldt), ldt);
    return 0;
}

/*
 * Panel via LAPACK: dgeqrf + dlarft + explicit Q by dorgqr.  tau in work[0:n].
 * Restates lila-c/lila_dgeqr2_w03_l.c:3-26.
 */
int oracle_dgeqr2_w03_l(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                        double *Q, int ldq, double *work, int lwork)
{
    (void)lwork;
    int ml = m - i;
    double *tau = work;
    double *Aii = &EL(A, i, i, lda), *Qii = &EL(Q, i, i, ldq);
    ob_dgeqr2(ml, n, Aii, lda, tau);
    ob_dlarft_fc(ml, n, Aii, lda, tau, &EL(T, i % mt, i, ldt), ldt);
    ob_dlacpy(ml, n, Aii, lda, Qii, ldq);
    ob_dorg2r(ml, n, n, Qii, ldq, tau);
    return 0;
}

/*
 * Panel via the recursive dgeqr3 plus explicit Q = [I;0] - V (T V1^T).
 * Restates lila-c/lila_dgeqr2_w03_3.c:3-34; work holds the n x n product.
 */
int oracle_dgeqr2_w03_3(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                        double *Q, int ldq, double *work, int lwork)
{
    (void)lwork;
    int ml = m - i;
    double *Aii = &EL(A, i, i, lda), *Qii = &EL(Q, i, i, ldq), *Tki = &EL(T, i % mt, i, ldt);
    oracle_dgeqr3(ml, n, Aii, lda, Tki, ldt);
    ob_dlacpy(ml, n, Aii, lda, Qii, ldq);
    for (int c = 0; c < n; c++)
        for (int r = 0; r <= c && r < ml; r++) EL(Qii, r, c, ldq) = (r == c) ? 1.0 : 0.0;
    for (int c = 0; c < n; c++)
        for (int r = 0; r < n; r++) EL(work, r, c, n) = (r <= c) ? EL(Tki, r, c, ldt) : 0.0;
    ob_dtrmm(OB_RIGHT, OB_LOWER, OB_T, OB_UNIT, n, n, 1.0, Aii, lda, work, n);
    ob_dtrmm(OB_RIGHT, OB_UPPER, OB_N, OB_NONUNIT, ml, n, -1.0, work, n, Qii, ldq);
    for (int c = 0; c < n; c++) EL(Qii, c, c, ldq) += 1.0;
    return 0;
}

/*
 * Householder reconstruction of an m x n orthonormal Q: LU without pivoting of
 * Q1 - S, where S(k) = -1 when |1 - t_kk| < |1 + t_kk| picks the larger pivot.
 * On entry T (n x n) holds Q(0:n, :) and A(n:m, :) holds Q(n:m, :); on exit
 * A holds V below the diagonal and S*R on and above it, T = -U L^-T, Q = Q S.
 * Restates lila-c/lila_dorgh2_3.c:3-55.
 */
int oracle_dorgh2_3(int m, int n, double *A, int lda, double *T, int ldt, double *Q, int ldq,
                    double *work, int lwork, double *S)
{
    (void)work;
    (void)lwork;
    for (int k = 0; k < n; k++) {
        double *tkk = &EL(T, k, k, ldt);
        if (fabs(1.0 - *tkk) < fabs(1.0 + *tkk)) {
            for (int r = 0; r < n; r++) EL(T, r, k, ldt) = -EL(T, r, k, ldt);
            S[k] = -1.0;
        } else {
            S[k] = 1.0;
        }
        *tkk -= 1.0;
        for (int r = k + 1; r < n; r++) EL(T, r, k, ldt) /= *tkk;
        ob_dger(n - k - 1, n - k - 1, -1.0, tkk + 1, 1, tkk + ldt, ldt, tkk + 1 + ldt, ldt);
    }
    for (int k = 0; k < n; k++)
        if (S[k] == -1.0)
            for (int r = n; r < m; r++) EL(A, r, k, lda) = -EL(A, r, k, lda);
    ob_dtrsm(OB_RIGHT, OB_UPPER, OB_N, OB_NONUNIT, m - n, n, 1.0, T, ldt, A + n, lda);
    for (int k = 0; k < n; k++)
        if (S[k] == -1.0)
            for (int c = k; c < n; c++) EL(A, k, c, lda) = -EL(A, k, c, lda);
    for (int k = 0; k < n; k++)
        if (S[k] == -1.0)
            for (int r = 0; r < m; r++) EL(Q, r, k, ldq) = -EL(Q, r, k, ldq);
    for (int k = 0; k < n; k++)
        for (int c = 0; c < k; c++) EL(A, k, c, lda) = EL(T, k, c, ldt);
    for (int k = 0; k < n; k++)
        for (int c = 0; c < k; c++) EL(T, k, c, ldt) = 0.0;
    ob_dtrsm(OB_RIGHT, OB_LOWER, OB_T, OB_UNIT, n, n, -1.0, A, lda, T, ldt);
    return 0;
}

/*
 * Householder reconstruction of tile j of a leaf that starts at column i:
 * rows [i, j) of R are sign-corrected with the earlier tiles' S, the tile's
 * Q columns are reduced by the earlier reflectors (using the zero top block:
 * W = V1^-1 Q(i:j)), then LU with sign choice as in lila_dorgh2_3.
 * work[0 : (j-i)*n] is scratch; S is indexed by the global column.
 * Restates lila-c/lila_ormhr2_w03_hr.c:3-84 (scratch no longer aliases S).
 */
int oracle_ormhr2_w03_hr(int m, int n, int i, int j, int l, int mt, double *A, int lda, double *T,
                         int ldt, double *Q, int ldq, double *work, int lwork, double *S)
{
    (void)l;
    (void)lwork;
    int it = j % mt, jw = j - i;
    double *Qij = &EL(Q, i, j, ldq), *Qjj = &EL(Q, j, j, ldq);
    double *Tjj = &EL(T, it, j, ldt);
    double *A0j = &EL(A, 0, j, lda), *Aii = &EL(A, i, i, lda), *Ajj = &EL(A, j, j, lda);
    double *Aji = &EL(A, j, i, lda);
    double *work2 = work;
    int ldw2 = jw > 0 ? jw : 1;
    for (int k = i; k < j; k++)
        if (S[k] == -1.0)
            for (int c = 0; c < n; c++) EL(A0j, k, c, lda) = -EL(A0j, k, c, lda);
    ob_dlacpy(jw, n, Qij, ldq, work2, ldw2);
    ob_dlacpy(n, n, Qjj, ldq, Tjj, ldt);
    ob_dlacpy(m - j - n, n, Qjj + n, ldq, Ajj + n, lda);
    if (jw != 0) {
        ob_dtrsm(OB_LEFT, OB_LOWER, OB_N, OB_UNIT, jw, n, 1.0, Aii, lda, work2, ldw2);
        ob_dgemm(OB_N, OB_N, n, n, jw, -1.0, Aji, lda, work2, ldw2, 1.0, Tjj, ldt);
        ob_dgemm(OB_N, OB_N, m - j - n, n, jw, -1.0, Aji + n, lda, work2, ldw2, 1.0, Ajj + n, lda);
    }
    for (int k = 0; k < n; k++) {
        double *tkk = &EL(Tjj, k, k, ldt);
        if (fabs(1.0 - *tkk) < fabs(1.0 + *tkk)) {
            for (int r = 0; r < n; r++) EL(Tjj, r, k, ldt) = -EL(Tjj, r, k, ldt);
            S[k + j] = -1.0;
        } else {
            S[k + j] = 1.0;
        }
        *tkk -= 1.0;
        for (int r = k + 1; r < n; r++) EL(Tjj, r, k, ldt) /= *tkk;
        ob_dger(n - k - 1, n - k - 1, -1.0, tkk + 1, 1, tkk + ldt, ldt, tkk + 1 + ldt, ldt);
    }
    for (int k = 0; k < n; k++)
        if (S[k + j] == -1.0)
            for (int c = k; c < n; c++) EL(Ajj, k, c, lda) = -EL(Ajj, k, c, lda);
    for (int k = 0; k < n; k++)
        if (S[k + j] == -1.0)
            for (int r = n; r < m - j; r++) EL(Ajj, r, k, lda) = -EL(Ajj, r, k, lda);
    for (int k = 0; k < n; k++)
        if (S[k + j] == -1.0)
            for (int r = 0; r < m - i; r++) EL(Qij, r, k, ldq) = -EL(Qij, r, k, ldq);
    for (int k = 0; k < n; k++)
        for (int c = 0; c < k; c++) EL(Ajj, k, c, lda) = EL(Tjj, k, c, ldt);
    for (int k = 0; k < n; k++)
        for (int c = 0; c < k; c++) EL(Tjj, k, c, ldt) = 0.0;
    ob_dtrsm(OB_RIGHT, OB_UPPER, OB_N, OB_NONUNIT, m - j - n, n, 1.0, Tjj, ldt, Ajj + n, lda);
    ob_dtrsm(OB_RIGHT, OB_LOWER, OB_T, OB_UNIT, n, n, -1.0, Ajj, lda, Tjj, ldt);
    return 0;
}

/* Tile form named in lila-c/lila.h:38 (the reference's lila_dorgh2.c does not
 * compile against that prototype): same contract as oracle_ormhr2_w03_hr. */
int oracle_dorgh2(int m, int n, int i, int j, int mt, double *A, int lda, double *T, int ldt,
                  double *Q, int ldq, double *work, int lwork, double *S)
{
    return oracle_ormhr2_w03_hr(m, n, i, j, -1, mt, A, lda, T, ldt, Q, ldq, work, lwork, S);
}

/*
 * Panel via Cholesky QR + Householder reconstruction: Q = A, G = Q^T Q into
 * A's top block, R = chol(G), Q = Q R^-1, then lila_dorgh2_3 on the panel.
 * S = work[0:n].  Restates lila-c/lila_dgeqr2_w03_hr.c:3-29.
 */
int oracle_dgeqr2_w03_hr(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                         double *Q, int ldq, double *work, int lwork)
{
    int ml = m - i;
    double *S = work;
    double *Aii = &EL(A, i, i, lda), *Qii = &EL(Q, i, i, ldq), *Tki = &EL(T, i % mt, i, ldt);
    ob_dlacpy(ml, n, Aii, lda, Qii, ldq);
    ob_dsyrk(OB_UPPER, OB_T, n, ml, 1.0, Qii, ldq, 0.0, Aii, lda);
    ob_dpotrf_upper(n, Aii, lda);
    ob_dtrsm(OB_RIGHT, OB_UPPER, OB_N, OB_NONUNIT, ml, n, 1.0, Aii, lda, Qii, ldq);
    ob_dlacpy(ml - n, n, Qii + n, ldq, Aii + n, lda);
    ob_dlacpy(n, n, Qii, ldq, Tki, ldt);
    oracle_dorgh2_3(ml, n, Aii, lda, Tki, ldt, Qii, ldq, work + n, lwork - n, S);
    return 0;
}

/* Panel dispatcher on lila_param[2].  Restates lila-c/lila_dgeqr2_w03.c:3-19. */
int oracle_dgeqr2_w03(int *lila_param, int m, int n, int i, int mt, double *A, int lda, double *T,
                      int ldt, double *Q, int ldq, double *work, int lwork)
{
    switch (lila_param[2]) {
    case 0: return oracle_dgeqr2_w03_l(m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork);
    case 1: return oracle_dgeqr2_w03_3(m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork);
    case 2: return oracle_dgeqr2_w03_hr(m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork);
    default: return 0;
    }
}

/* ------------------------------------------------------------------------ */
/* Leaves                                                                   */
/* ------------------------------------------------------------------------ */

/*
 * Leaf as a sequence of mt tiles: update the tile by the leaf's earlier
 * reflectors, factor it with the panel, extend its Q by the earlier reflectors.
 * Restates lila-c/lila_dgeqrf_w03_mt_hh.c:3-35.
 */
int oracle_dgeqrf_w03_mt_hh(int *lila_param, int m, int n, int i, int mt, double *A, int lda,
                            double *T, int ldt, double *Q, int ldq, double *work, int lwork)
{
    int vb = imin(mt - i % mt, n);
    oracle_dgeqr2_w03(lila_param, m, vb, i, mt, A, lda, T, ldt, Q, ldq, work, lwork);
    for (int j = i + vb; j < i + n; j += vb) {
        vb = imin(mt, i + n - j);
        int l = j - i;
        oracle_dormqrf_w03(m, vb, l, i, j, mt, A, lda, T, ldt, work, lwork);
        oracle_dgeqr2_w03(lila_param, m, vb, j, mt, A, lda, T, ldt, Q, ldq, work, lwork);
        oracle_dormqrbz_w03(m, vb, l, i, j, mt, A, lda, Q, ldq, T, ldt, work, lwork);
    }
    return 0;
}

/* Leaf via LAPACK: dgeqrf, lila_dlarft_w03, dorgqr.  tau = work + n.
 * Restates lila-c/lila_dgeqrf_w03_mt_l.c:3-22. */
int oracle_dgeqrf_w03_mt_l(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                           double *Q, int ldq, double *work, int lwork)
{
    (void)lwork;
    int ml = m - i;
    double *tau = work + n;
    double *Aii = &EL(A, i, i, lda), *Qii = &EL(Q, i, i, ldq);
    ob_dgeqr2(ml, n, Aii, lda, tau);
    oracle_dlarft_w03(m, n, i, mt, A, lda, T, ldt, tau);
    ob_dlacpy(ml, n, Aii, lda, Qii, ldq);
    ob_dorg2r(ml, n, n, Qii, ldq, tau);
    return 0;
}

/*
 * Leaf via Cholesky QR of the whole leaf followed by tile-wise Householder
 * reconstruction.  S = work[0 : i+n] (global index); the tile routine's
 * scratch is work + (i+n).  Restates lila-c/lila_dgeqrf_w03_mt_hr.c:3-33.
 */
int oracle_dgeqrf_w03_mt_hr(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                            double *Q, int ldq, double *work, int lwork)
{
    int ml = m - i;
    double *S = work;
    double *scratch = work + (i + n);
    double *Aii = &EL(A, i, i, lda), *Qii = &EL(Q, i, i, ldq);
    ob_dlacpy(ml, n, Aii, lda, Qii, ldq);
    ob_dsyrk(OB_UPPER, OB_T, n, ml, 1.0, Qii, ldq, 0.0, Aii, lda);
    ob_dpotrf_upper(n, Aii, lda);
    ob_dtrsm(OB_RIGHT, OB_UPPER, OB_N, OB_NONUNIT, ml, n, 1.0, Aii, lda, Qii, ldq);
    for (int j = i; j < i + n;) {
        int vb = imin(tile_end(j, i + n, mt) - j, n);
        oracle_ormhr2_w03_hr(m, vb, i, j, -1, mt, A, lda, T, ldt, Q, ldq, scratch, lwork - (i + n), S);
        j += vb;
    }
    return 0;
}

/* Leaf dispatcher on lila_param[1].  Restates lila-c/lila_dgeqrf_w03_mt.c:3-19. */
int oracle_dgeqrf_w03_mt(int *lila_param, int m, int n, int i, int mt, double *A, int lda,
                         double *T, int ldt, double *Q, int ldq, double *work, int lwork)
{
    switch (lila_param[1]) {
    case 0: return oracle_dgeqrf_w03_mt_l(m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork);
    case 1: return oracle_dgeqrf_w03_mt_hh(lila_param, m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork);
    case 2: return oracle_dgeqrf_w03_mt_hr(m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork);
    default: return 0;
    }
}

/* ------------------------------------------------------------------------ */
/* Drivers                                                                  */
/* ------------------------------------------------------------------------ */

/* Column recursion down to nx = lila_param[3].
 * Restates lila-c/lila_dgeqrf_w03_recursive.c:3-29. */
int oracle_dgeqrf_w03_recursive(int *lila_param, int m, int n, int i, int mt, double *A, int lda,
                                double *T, int ldt, double *Q, int ldq, double *work, int lwork)
{
    if (n <= lila_param[3])
        return oracle_dgeqrf_w03_mt(lila_param, m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork);
    int nb1 = n / 2, nb2 = n - nb1;
    oracle_dgeqrf_w03_recursive(lila_param, m, nb1, i, mt, A, lda, T, ldt, Q, ldq, work, lwork);
    oracle_dormqrf_w03(m, nb2, nb1, i, i + nb1, mt, A, lda, T, ldt, work, lwork);
    oracle_dgeqrf_w03_recursive(lila_param, m, nb2, i + nb1, mt, A, lda, T, ldt, Q, ldq, work, lwork);
    oracle_dlarft_connect_w03(m, nb2, i + nb1, i, mt, A, lda, T, ldt);
    oracle_dormqrbz_w03(m, nb2, nb1, i, i + nb1, mt, A, lda, Q, ldq, T, ldt, work, lwork);
    return 0;
}

/* Multi-level column blocking nb_lvl[i_lvl], leaves at the last level.
 * Restates lila-c/lila_dgeqrf_w03_levelx.c:3-52. */
int oracle_dgeqrf_w03_levelx(int *lila_param, int n_lvl, int i_lvl, int *nb_lvl, int m, int n,
                             int i, int mt, double *A, int lda, double *T, int ldt, double *Q,
                             int ldq, double *work, int lwork)
{
    int nb = nb_lvl[i_lvl];
    int last = (i_lvl == n_lvl - 1);
    int k = 0, j = i;
    while (j < i + n) {
        int vb = imin(nb, i + n - j);
        if (k > 0) oracle_dormqrf_w03(m, vb, k, i, j, mt, A, lda, T, ldt, work, lwork);
        if (last)
            oracle_dgeqrf_w03_mt(lila_param, m, vb, j, mt, A, lda, T, ldt, Q, ldq, work, lwork);
        else
            oracle_dgeqrf_w03_levelx(lila_param, n_lvl, i_lvl + 1, nb_lvl, m, vb, j, mt, A, lda, T,
                                     ldt, Q, ldq, work, lwork);
        if (k > 0) {
            oracle_dlarft_connect_w03(m, vb, j, i, mt, A, lda, T, ldt);
            oracle_dormqrbz_w03(m, vb, k, i, j, mt, A, lda, Q, ldq, T, ldt, work, lwork);
        }
        k += vb;
        j += vb;
    }
    return 0;
}

/* Factor n new columns against k existing ones (V, T, Q already in place).
 * Restates lila-c/lila_dgeqrf_w03_appendcols.c:3-14. */
int oracle_dgeqrf_w03_appendcols(int *lila_param, int m, int k, int n, int mt, double *A, int lda,
                                 double *Q, int ldq, double *T, int ldt, double *work, int lwork)
{
    if (k != 0) oracle_dormqrf_w03(m, n, k, 0, k, mt, A, lda, T, ldt, work, lwork);
    oracle_dgeqrf_w03_recursive(lila_param, m, n, k, mt, A, lda, T, ldt, Q, ldq, work, lwork);
    if (k != 0) oracle_dlarft_connect_w03(m, n, k, 0, mt, A, lda, T, ldt);
    if (k != 0) oracle_dormqrbz_w03(m, n, k, 0, k, mt, A, lda, Q, ldq, T, ldt, work, lwork);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* V, R, T without Q (v03) and Q from V, T (q03)                            */
/* ------------------------------------------------------------------------ */
/*
 * Both recursions stop at n < nx (the w03 one at n <= nx).  With nx = 1 the
 * reference's recursion on a single column never ends; here a single column
 * is always a leaf.  Leaf 2 and panel 2 are not implemented in the reference
 * (lila_dgeqrf_v03_mt.c:14-16, lila_dgeqr2_v03.c:13-15 and their q03 twins):
 * leaf 2 does nothing, panel 2 factors nothing while the tile loop around it
 * still runs, as here.
 */

/* Panel via dgeqr3.  Restates lila-c/lila_dgeqr2_v03_3.c:3-34, whose product
 * T V1^T into the workspace is never read and is left out. */
int oracle_dgeqr2_v03_3(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                        double *work, int lwork)
{
    (void)work;
    (void)lwork;
    return oracle_dgeqr3(m - i, n, &EL(A, i, i, lda), lda, &EL(T, i % mt, i, ldt), ldt);
}

/* Panel via dgeqrf + dlarft, tau in work[0:n].  Restates lila-c/lila_dgeqr2_v03_l.c:3-27. */
int oracle_dgeqr2_v03_l(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                        double *work, int lwork)
{
    (void)lwork;
    int ml = m - i;
    double *Aii = &EL(A, i, i, lda);
    ob_dgeqr2(ml, n, Aii, lda, work);
    ob_dlarft_fc(ml, n, Aii, lda, work, &EL(T, i % mt, i, ldt), ldt);
    return 0;
}

/* lila-c/lila_dgeqr2_v03.c:3-19 */
int oracle_dgeqr2_v03(int *lila_param, int m, int n, int i, int mt, double *A, int lda, double *T,
                      int ldt, double *work, int lwork)
{
    switch (lila_param[2]) {
    case 0: return oracle_dgeqr2_v03_l(m, n, i, mt, A, lda, T, ldt, work, lwork);
    case 1: return oracle_dgeqr2_v03_3(m, n, i, mt, A, lda, T, ldt, work, lwork);
    default: return 0;
    }
}

/* Tiles: update by the leaf's earlier reflectors, then factor.
 * Restates lila-c/lila_dgeqrf_v03_mt_hh.c:3-35. */
int oracle_dgeqrf_v03_mt_hh(int *lila_param, int m, int n, int i, int mt, double *A, int lda,
                            double *T, int ldt, double *work, int lwork)
{
    int vb = imin(mt - i % mt, n);
    oracle_dgeqr2_v03(lila_param, m, vb, i, mt, A, lda, T, ldt, work, lwork);
    for (int j = i + vb; j < i + n; j += vb) {
        vb = imin(mt, i + n - j);
        oracle_dormqrf_w03(m, vb, j - i, i, j, mt, A, lda, T, ldt, work, lwork);
        oracle_dgeqr2_v03(lila_param, m, vb, j, mt, A, lda, T, ldt, work, lwork);
    }
    return 0;
}

/* dgeqrf of the leaf and lila_dlarft_w03, tau = work + n.
 * Restates lila-c/lila_dgeqrf_v03_mt_l.c:3-19. */
int oracle_dgeqrf_v03_mt_l(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                           double *work, int lwork)
{
    (void)lwork;
    double *tau = work + n;
    ob_dgeqr2(m - i, n, &EL(A, i, i, lda), lda, tau);
    return oracle_dlarft_w03(m, n, i, mt, A, lda, T, ldt, tau);
}

/* lila-c/lila_dgeqrf_v03_mt.c:3-19 */
int oracle_dgeqrf_v03_mt(int *lila_param, int m, int n, int i, int mt, double *A, int lda,
                         double *T, int ldt, double *work, int lwork)
{
    switch (lila_param[1]) {
    case 0: return oracle_dgeqrf_v03_mt_l(m, n, i, mt, A, lda, T, ldt, work, lwork);
    case 1: return oracle_dgeqrf_v03_mt_hh(lila_param, m, n, i, mt, A, lda, T, ldt, work, lwork);
    default: return 0;
    }
}

/* lila-c/lila_dgeqrf_v03_recursive.c:3-26 */
int oracle_dgeqrf_v03_recursive(int *lila_param, int m, int n, int i, int mt, double *A, int lda,
                                double *T, int ldt, double *work, int lwork)
{
    if (n < lila_param[3] || n <= 1)
        return oracle_dgeqrf_v03_mt(lila_param, m, n, i, mt, A, lda, T, ldt, work, lwork);
    int nb1 = n / 2, nb2 = n - nb1;
    oracle_dgeqrf_v03_recursive(lila_param, m, nb1, i, mt, A, lda, T, ldt, work, lwork);
    oracle_dormqrf_w03(m, nb2, nb1, i, i + nb1, mt, A, lda, T, ldt, work, lwork);
    oracle_dgeqrf_v03_recursive(lila_param, m, nb2, i + nb1, mt, A, lda, T, ldt, work, lwork);
    oracle_dlarft_connect_w03(m, nb2, i + nb1, i, mt, A, lda, T, ldt);
    return 0;
}

/* lila-c/lila_dgeqrf_v03_levelx.c:3-47 */
int oracle_dgeqrf_v03_levelx(int *lila_param, int n_lvl, int i_lvl, int *nb_lvl, int m, int n,
                             int i, int mt, double *A, int lda, double *T, int ldt, double *work,
                             int lwork)
{
    int nb = nb_lvl[i_lvl];
    int last = (i_lvl == n_lvl - 1);
    int k = 0, j = i;
    while (j < i + n) {
        int vb = imin(nb, i + n - j);
        if (k > 0) oracle_dormqrf_w03(m, vb, k, i, j, mt, A, lda, T, ldt, work, lwork);
        if (last)
            oracle_dgeqrf_v03_mt(lila_param, m, vb, j, mt, A, lda, T, ldt, work, lwork);
        else
            oracle_dgeqrf_v03_levelx(lila_param, n_lvl, i_lvl + 1, nb_lvl, m, vb, j, mt, A, lda, T,
                                     ldt, work, lwork);
        if (k > 0) oracle_dlarft_connect_w03(m, vb, j, i, mt, A, lda, T, ldt);
        k += vb;
        j += vb;
    }
    return 0;
}

/* Q(i:m, i:i+n) = [I; 0] - V (T V1^T) of one tile's reflectors.
 * Restates lila-c/lila_dgeqr2_q03_3.c:3-43; work holds the n x n product. */
int oracle_dgeqr2_q03_3(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                        double *Q, int ldq, double *work, int lwork)
{
    (void)lwork;
    int ml = m - i;
    double *Aii = &EL(A, i, i, lda), *Qii = &EL(Q, i, i, ldq), *Tki = &EL(T, i % mt, i, ldt);
    ob_dlacpy(ml, n, Aii, lda, Qii, ldq);
    for (int c = 0; c < n; c++)
        for (int r = 0; r <= c && r < ml; r++) EL(Qii, r, c, ldq) = (r == c) ? 1.0 : 0.0;
    for (int c = 0; c < n; c++)
        for (int r = 0; r < n; r++) EL(work, r, c, n) = (r <= c) ? EL(Tki, r, c, ldt) : 0.0;
    ob_dtrmm(OB_RIGHT, OB_LOWER, OB_T, OB_UNIT, n, n, 1.0, Aii, lda, work, n);
    ob_dtrmm(OB_RIGHT, OB_UPPER, OB_N, OB_NONUNIT, ml, n, -1.0, work, n, Qii, ldq);
    for (int c = 0; c < n; c++) EL(Qii, c, c, ldq) += 1.0;
    return 0;
}

/* dorgqr with tau = diag of the tile's T, tau in work[0:n].
 * Restates lila-c/lila_dgeqr2_q03_l.c:3-30. */
int oracle_dgeqr2_q03_l(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                        double *Q, int ldq, double *work, int lwork)
{
    (void)lwork;
    int ml = m - i;
    double *Qii = &EL(Q, i, i, ldq), *Tki = &EL(T, i % mt, i, ldt);
    for (int c = 0; c < n; c++) work[c] = EL(Tki, c, c, ldt);
    ob_dlacpy(ml, n, &EL(A, i, i, lda), lda, Qii, ldq);
    ob_dorg2r(ml, n, n, Qii, ldq, work);
    return 0;
}

/* lila-c/lila_dgeqr2_q03.c:3-19 */
int oracle_dgeqr2_q03(int *lila_param, int m, int n, int i, int mt, double *A, int lda, double *T,
                      int ldt, double *Q, int ldq, double *work, int lwork)
{
    switch (lila_param[2]) {
    case 0: return oracle_dgeqr2_q03_l(m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork);
    case 1: return oracle_dgeqr2_q03_3(m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork);
    default: return 0;
    }
}

/* Tiles: Q of each tile's reflectors, extended by the leaf's earlier ones.
 * Restates lila-c/lila_dgeqrf_q03_mt_hh.c:3-32. */
int oracle_dgeqrf_q03_mt_hh(int *lila_param, int m, int n, int i, int mt, double *A, int lda,
                            double *T, int ldt, double *Q, int ldq, double *work, int lwork)
{
    int vb = imin(mt - i % mt, n);
    oracle_dgeqr2_q03(lila_param, m, vb, i, mt, A, lda, T, ldt, Q, ldq, work, lwork);
    for (int j = i + vb; j < i + n; j += vb) {
        vb = imin(mt, i + n - j);
        oracle_dgeqr2_q03(lila_param, m, vb, j, mt, A, lda, T, ldt, Q, ldq, work, lwork);
        oracle_dormqrbz_w03(m, vb, j - i, i, j, mt, A, lda, Q, ldq, T, ldt, work, lwork);
    }
    return 0;
}

/* dorgqr of the whole leaf with tau from the T tiles, tau in work[0:n].
 * Restates lila-c/lila_dgeqrf_q03_mt_l.c:3-23. */
int oracle_dgeqrf_q03_mt_l(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                           double *Q, int ldq, double *work, int lwork)
{
    (void)lwork;
    int ml = m - i;
    double *Qii = &EL(Q, i, i, ldq);
    oracle_dT2tau_w03(m, n, i, mt, T, ldt, work);
    ob_dlacpy(ml, n, &EL(A, i, i, lda), lda, Qii, ldq);
    ob_dorg2r(ml, n, n, Qii, ldq, work);
    return 0;
}

/* lila-c/lila_dgeqrf_q03_mt.c:3-19 */
int oracle_dgeqrf_q03_mt(int *lila_param, int m, int n, int i, int mt, double *A, int lda,
                         double *T, int ldt, double *Q, int ldq, double *work, int lwork)
{
    switch (lila_param[1]) {
    case 0: return oracle_dgeqrf_q03_mt_l(m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork);
    case 1: return oracle_dgeqrf_q03_mt_hh(lila_param, m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork);
    default: return 0;
    }
}

/* lila-c/lila_dgeqrf_q03_recursive.c:3-25 */
int oracle_dgeqrf_q03_recursive(int *lila_param, int m, int n, int i, int mt, double *A, int lda,
                                double *T, int ldt, double *Q, int ldq, double *work, int lwork)
{
    if (n < lila_param[3] || n <= 1)
        return oracle_dgeqrf_q03_mt(lila_param, m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork);
    int nb1 = n / 2, nb2 = n - nb1;
    oracle_dgeqrf_q03_recursive(lila_param, m, nb1, i, mt, A, lda, T, ldt, Q, ldq, work, lwork);
    oracle_dgeqrf_q03_recursive(lila_param, m, nb2, i + nb1, mt, A, lda, T, ldt, Q, ldq, work, lwork);
    oracle_dormqrbz_w03(m, nb2, nb1, i, i + nb1, mt, A, lda, Q, ldq, T, ldt, work, lwork);
    return 0;
}

/* lila-c/lila_dgeqrf_q03_levelx.c:3-48 */
int oracle_dgeqrf_q03_levelx(int *lila_param, int n_lvl, int i_lvl, int *nb_lvl, int m, int n,
                             int i, int mt, double *A, int lda, double *T, int ldt, double *Q,
                             int ldq, double *work, int lwork)
{
    int nb = nb_lvl[i_lvl];
    int last = (i_lvl == n_lvl - 1);
    int k = 0, j = i;
    while (j < i + n) {
        int vb = imin(nb, i + n - j);
        if (last)
            oracle_dgeqrf_q03_mt(lila_param, m, vb, j, mt, A, lda, T, ldt, Q, ldq, work, lwork);
        else
            oracle_dgeqrf_q03_levelx(lila_param, n_lvl, i_lvl + 1, nb_lvl, m, vb, j, mt, A, lda, T,
                                     ldt, Q, ldq, work, lwork);
        if (k > 0) oracle_dormqrbz_w03(m, vb, k, i, j, mt, A, lda, Q, ldq, T, ldt, work, lwork);
        k += vb;
        j += vb;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Workspace queries (counts of doubles); restate lila-c/lila_query_*.c      */
/* ------------------------------------------------------------------------ */

/* lila-c/lila_query_dormqrf_w03.c:3-32 */
int oracle_query_dormqrf_w03(int m, int n, int k, int i, int j, int mt)
{
    (void)j;
    int need = n * mt, ml = m - i;
    for (int a = i; a < i + k || a == i;) {
        int b = tile_end(a, i + k, mt);
        need = imax(need, (ml - (b - a)) * n);
        ml -= b - a;
        if (b >= i + k) break;
        a = b;
    }
    return need;
}

/* lila-c/lila_query_dormqrbz_w03.c:3-32 */
int oracle_query_dormqrbz_w03(int m, int n, int k, int i, int j, int mt)
{
    (void)j;
    int vb = (i + k) % mt;
    if (vb == 0) vb = mt;
    if (vb > k) vb = k;
    int need = n * k, ml = m - (i + k - vb), jj = 1;
    while (jj + vb - 1 != k) {
        need = imax(need, n * vb);
        need = imax(need, (ml - vb) * k);
        jj += vb;
        vb = (jj + mt - 1 <= k) ? mt : k - jj + 1;
        ml += vb;
    }
    return need;
}

static int query_panel(int panel, int n)
{
    /* lila-c/lila_query_dgeqr2_w03_{l,3,hr}.c: n*n, n*n, n */
    if (panel == 2) return n;
    return n * n;
}

/* mt_hr: n*(j-i)+n per tile (lila-c/lila_query_ormhr2_w03_hr.c:8) plus S (i+n). */
int oracle_query_dgeqrf_w03_mt_hr(int m, int n, int i, int mt)
{
    (void)m;
    int need = 0;
    for (int j = i; j < i + n;) {
        int vb = imin(tile_end(j, i + n, mt) - j, n);
        need = imax(need, vb * (j - i) + vb);
        j += vb;
    }
    return need + i + n;
}

/* lila-c/lila_query_dgeqrf_w03_mt_hh.c:3-52 */
int oracle_query_dgeqrf_w03_mt_hh(int *lila_param, int m, int n, int i, int mt)
{
    int vb = imin(mt - i % mt, n);
    int need = query_panel(lila_param[2], vb);
    for (int j = i + vb; j < i + n; j += vb) {
        vb = imin(mt, i + n - j);
        need = imax(need, oracle_query_dormqrf_w03(m, vb, j - i, i, j, mt));
        need = imax(need, query_panel(lila_param[2], vb));
        need = imax(need, oracle_query_dormqrbz_w03(m, vb, j - i, i, j, mt));
    }
    return need;
}

/* lila-c/lila_query_dgeqrf_w03_mt.c:3-18 (mt_l: n*n, lila_query_dgeqrf_w03_mt_l.c:5;
 * the leaf also stores tau at work + n, so 2n is added to cover it). */
int oracle_query_dgeqrf_w03_mt(int *lila_param, int m, int n, int i, int mt)
{
    switch (lila_param[1]) {
    case 0: return imax(n * n, 2 * n);
    case 1: return oracle_query_dgeqrf_w03_mt_hh(lila_param, m, n, i, mt);
    case 2: return oracle_query_dgeqrf_w03_mt_hr(m, n, i, mt);
    default: return 0;
    }
}

/* lila-c/lila_query_dgeqrf_w03_recursive.c:3-26 */
int oracle_query_dgeqrf_w03_recursive(int *lila_param, int m, int n, int i, int mt)
{
    if (n <= lila_param[3]) return oracle_query_dgeqrf_w03_mt(lila_param, m, n, i, mt);
    int nb1 = n / 2, nb2 = n - nb1, need = 0;
    need = imax(need, oracle_query_dgeqrf_w03_recursive(lila_param, m, nb1, i, mt));
    need = imax(need, oracle_query_dormqrf_w03(m, nb2, nb1, i, i + nb1, mt));
    need = imax(need, oracle_query_dgeqrf_w03_recursive(lila_param, m, nb2, i + nb1, mt));
    need = imax(need, oracle_query_dormqrbz_w03(m, nb2, nb1, i, i + nb1, mt));
    return need;
}

/* lila-c/lila_query_dgeqrf_w03_levelx.c:3-55 */
int oracle_query_dgeqrf_w03_levelx(int *lila_param, int n_lvl, int i_lvl, int *nb_lvl, int m,
                                   int n, int i, int mt)
{
    int nb = nb_lvl[i_lvl], need = 0, k = 0, j = i;
    int last = (i_lvl == n_lvl - 1);
    while (j < i + n) {
        int vb = imin(nb, i + n - j);
        if (k > 0) need = imax(need, oracle_query_dormqrf_w03(m, vb, k, i, j, mt));
        if (last)
            need = imax(need, oracle_query_dgeqrf_w03_mt(lila_param, m, vb, j, mt));
        else
            need = imax(need, oracle_query_dgeqrf_w03_levelx(lila_param, n_lvl, i_lvl + 1, nb_lvl, m, vb, j, mt));
        if (k > 0) need = imax(need, oracle_query_dormqrbz_w03(m, vb, k, i, j, mt));
        k += vb;
        j += vb;
    }
    return need;
}

/* ------------------------------------------------------------------------ */
/* Least squares and checks                                                 */
/* ------------------------------------------------------------------------ */

/*
 * min ||A x - B||: QR with T by the recursive panel, B := Q^T B through V and
 * T, then R X = B(0:n).  A (m x n) and B (m x nrhs) are overwritten; X is
 * B(0:n, :); T is n x n.  Restates least-squares/main_ls_qr3.c:94-119.
 */
int oracle_ls_solve(int m, int n, int nrhs, double *A, int lda, double *T, int ldt, double *B,
                    int ldb, double *work)
{
    oracle_dgeqr3(m, n, A, lda, T, ldt);
    ob_dlacpy(n, nrhs, B, ldb, work, n);
    ob_dtrmm(OB_LEFT, OB_LOWER, OB_T, OB_UNIT, n, nrhs, 1.0, A, lda, work, n);
    ob_dgemm(OB_T, OB_N, n, nrhs, m - n, 1.0, A + n, lda, B + n, ldb, 1.0, work, n);
    ob_dtrmm(OB_LEFT, OB_UPPER, OB_T, OB_NONUNIT, n, nrhs, 1.0, T, ldt, work, n);
    ob_dgemm(OB_N, OB_N, m - n, nrhs, n, -1.0, A + n, lda, work, n, 1.0, B + n, ldb);
    ob_dtrmm(OB_LEFT, OB_LOWER, OB_N, OB_UNIT, n, nrhs, 1.0, A, lda, work, n);
    for (int c = 0; c < nrhs; c++)
        for (int r = 0; r < n; r++) EL(B, r, c, ldb) -= EL(work, r, c, n);
    ob_dtrsm(OB_LEFT, OB_UPPER, OB_N, OB_NONUNIT, n, nrhs, 1.0, A, lda, B, ldb);
    return 0;
}

/* ||I - Q^T Q||_F over Q(i:m, i:i+n).  Restates
 * lila-c-lila_param/lila/src/lila_test_qq_orth_1.c:3-19. */
double oracle_test_qq_orth_1(int m, int n, int i, double *Q, int ldq)
{
    int ml = m - i;
    double *Qii = &EL(Q, i, i, ldq);
    double *G = (double *)calloc((size_t)n * n, sizeof(double));
    for (int c = 0; c < n; c++) EL(G, c, c, n) = 1.0;
    ob_dgemm(OB_T, OB_N, n, n, ml, -1.0, Qii, ldq, Qii, ldq, 1.0, G, n);
    double r = ob_dlange_fro(n, n, G, n);
    free(G);
    return r;
}

/* ||A - Q R||_F / ||A||_F over the block at (i, i), R upper n x n.  Restates
 * lila-c-lila_param/lila/src/lila_test_qr_repres_1.c:3-27. */
double oracle_test_qr_repres_1(int m, int n, int i, double *A, int lda, double *Q, int ldq,
                               double *R, int ldr)
{
    int ml = m - i;
    double *Aii = &EL(A, i, i, lda), *Qii = &EL(Q, i, i, ldq), *Rii = &EL(R, i, i, ldr);
    double *W = (double *)malloc(sizeof(double) * (size_t)ml * n);
    ob_dlacpy(ml, n, Qii, ldq, W, ml);
    ob_dtrmm(OB_RIGHT, OB_UPPER, OB_N, OB_NONUNIT, ml, n, 1.0, Rii, ldr, W, ml);
    for (int c = 0; c < n; c++)
        for (int r = 0; r < ml; r++) EL(W, r, c, ml) -= EL(Aii, r, c, lda);
    double num = ob_dlange_fro(ml, n, W, ml);
    double den = ob_dlange_fro(ml, n, Aii, lda);
    free(W);
    return den > 0 ? num / den : num;
}

/* Reference products for the split-precision kernels: C = op(A) B with each
 * entry accumulated in double-double (error ~2^-100 relative to |A||B|). */
int oracle_gemm_dd(int ta, int m, int n, int k, double *A, int lda, double *B, int ldb, double *C,
                   int ldc)
{
    ob_dgemm_dd(ta, m, n, k, A, lda, B, ldb, C, ldc);
    return 0;
}
