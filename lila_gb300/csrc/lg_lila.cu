// lg_lila.cu -- the lila.h w03 routines on GB300: host-side drivers that
// enqueue FP64 kernels on the library stream.
//
// Each routine follows the algorithm of the reference routine cited in its
// comment (same tile walk over the global-index T layout), but is built from
// this library's fused device operations: a block-reflector tile is one
// split-K reduction GEMM (W = V^T C, unit-lower mask applied on the fly, so
// the reference's trmm/gemm pair is one launch), one small GEMM with the
// triangular T, and one rank-vb update GEMM.  Workspace comes from the
// caller's `work` (device memory); lila_query_* report what is needed.
#include <algorithm>

#include "lg_common.cuh"
#include "../../include/lila.h"

namespace lg {

static inline int imin(int a, int b) { return a < b ? a : b; }
static inline int imax(int a, int b) { return a > b ? a : b; }
static inline long long lmax(long long a, long long b) { return a > b ? a : b; }

// End of the reflector tile that starts at a, clipped to `end`.
static inline int tile_end(int a, int end, int mt)
{
    int b = (a / mt + 1) * mt;
    return b < end ? b : end;
}

// Partial-product storage the split-K GEMM may use for an M x N output.
static long long splitk_budget(int M, int N)
{
    if (M <= 0 || N <= 0) return 0;
    long long tiles = (long long)((M + 31) / 32) * ((N + 31) / 32);
    long long s = (4 * 152 + tiles - 1) / tiles;
    if (s > 64) s = 64;
    if (s < 2) return 0;
    return s * (long long)M * N;
}

struct Work {
    double *p;
    long long len;
    double *take(long long n)
    {
        double *r = p;
        p += n;
        len -= n;
        return r;
    }
};

static GemmEpi epi(double alpha, double beta)
{
    GemmEpi e;
    e.alpha = alpha;
    e.beta = beta;
    return e;
}

// ---------------------------------------------------------------------------
// workspace needs (doubles); the minimum is what the routine cannot run
// without, the query value adds split-K room
// ---------------------------------------------------------------------------
static long long need_apply(int n, int k, int mt, bool full)
{
    if (n <= 0 || k <= 0) return 0;
    int vb = imin(mt, k);
    long long base = 2LL * vb * n;
    return full ? base + splitk_budget(vb, n) : base;
}

static long long need_dgeqr3(int n, bool full)
{
    if (n <= 1) return 0;
    int n1 = n / 2, n2 = n - n1;
    long long base = 2LL * n1 * n2;
    if (!full) return base;
    // the query adds room for the one-launch panel of widths up to 64
    return lmax(base + splitk_budget(n1, n2), panel_coop_work(imin(n, 64)));
}

static long long need_connect(int n, int mt, bool full)
{
    int vb = imin(mt, n), wb = mt;
    long long base = 2LL * wb * vb;
    return full ? base + splitk_budget(wb, vb) : base;
}

static long long need_panel(int panel, int n, bool full)
{
    if (panel == 2) return n + (full ? splitk_budget(n, n) : 0);
    return (long long)n * n + need_dgeqr3(n, full);
}

static long long need_ormhr2(int n, int i, int j, bool full)
{
    (void)full;
    return (long long)(j - i) * n;
}

static long long need_mt_hr(int n, int i, int mt, bool full)
{
    long long inner = full ? splitk_budget(n, n) : 0;
    for (int j = i; j < i + n;) {
        int vb = imin(tile_end(j, i + n, mt) - j, n);
        inner = lmax(inner, need_ormhr2(vb, i, j, full));
        j += vb;
    }
    return (long long)(i + n) + inner;
}

static long long need_mt_l(int n, bool full) { return 2LL * n * n + need_dgeqr3(n, full); }

static long long need_mt_hh(int panel, int n, int i, int mt, bool full)
{
    int vb = imin(mt - i % mt, n);
    long long need = need_panel(panel, vb, full);
    for (int j = i + vb; j < i + n; j += vb) {
        vb = imin(mt, i + n - j);
        need = lmax(need, need_apply(vb, j - i, mt, full));
        need = lmax(need, need_panel(panel, vb, full));
    }
    return need;
}

static long long need_mt(const int *lp, int n, int i, int mt, bool full)
{
    switch (lp[1]) {
    case 0: return need_mt_l(n, full);
    case 1: return need_mt_hh(lp[2], n, i, mt, full);
    case 2: return need_mt_hr(n, i, mt, full);
    case 3: return need_mixed_leaf(n);
    }
    return 0;
}

static long long need_recursive(const int *lp, int n, int i, int mt, bool full)
{
    if (n <= lp[3]) return need_mt(lp, n, i, mt, full);
    int nb1 = n / 2, nb2 = n - nb1;
    long long need = need_recursive(lp, nb1, i, mt, full);
    need = lmax(need, need_apply(nb2, nb1, mt, full));
    need = lmax(need, need_recursive(lp, nb2, i + nb1, mt, full));
    need = lmax(need, need_connect(nb2, mt, full));
    return need;
}

static long long need_levelx(const int *lp, int n_lvl, int i_lvl, const int *nb_lvl, int n, int i,
                             int mt, bool full)
{
    int nb = nb_lvl[i_lvl];
    long long need = 0;
    int k = 0, j = i;
    while (j < i + n) {
        int vb = imin(nb, i + n - j);
        if (k > 0) {
            need = lmax(need, need_apply(vb, k, mt, full));
            need = lmax(need, need_connect(vb, mt, full));
        }
        if (i_lvl == n_lvl - 1)
            need = lmax(need, need_mt(lp, vb, j, mt, full));
        else
            need = lmax(need, need_levelx(lp, n_lvl, i_lvl + 1, nb_lvl, vb, j, mt, full));
        k += vb;
        j += vb;
    }
    return need;
}

static int clamp_query(long long v)
{
    if (v < 1) v = 1;
    if (v > 0x7fffffffLL) v = 0x7fffffffLL;
    return (int)v;
}

// ---------------------------------------------------------------------------
// block reflector applications
// ---------------------------------------------------------------------------

// C := H^T C, C addressed by global row (row r of the block is C + r).
// lila-c/lila_dormqrf_w03.c:15-76 / lila_dormqrf_z03.c:11-67.
static void apply_qt(int m, int n, int k, int i, int mt, const double *A, int lda, const double *T,
                     int ldt, double *C, int ldc, Work w)
{
    if (n <= 0 || k <= 0) return;
    int vbmax = imin(mt, k);
    double *W1 = w.take((long long)vbmax * n);
    double *W2 = w.take((long long)vbmax * n);
    for (int a = i; a < i + k;) {
        int b = tile_end(a, i + k, mt), vb = b - a;
        const double *V = A + a + (size_t)a * lda;
        const double *Tt = T + a % mt + (size_t)a * ldt;
        double *Ct = C + a;
        gemm(vb, n, m - a, opnd(V, lda, TR, M_UNIT_LOWER), opnd(Ct, ldc), W1, vb, epi(1, 0), w.p, w.len);
        gemm(vb, n, vb, opnd(Tt, ldt, TR, M_UPPER), opnd(W1, vb), W2, vb, epi(1, 0));
        gemm(m - a, n, vb, opnd(V, lda, NT, M_UNIT_LOWER), opnd(W2, vb), Ct, ldc, epi(-1, 1));
        a = b;
    }
}

// apply_qt on a caller-supplied scratch region (used by the entry point whose
// scratch is a fixed device array, lg_noalloc.cu).
void apply_qt_scratch(int m, int n, int k, int i, int mt, const double *A, int lda, const double *T, int ldt,
                      double *C, int ldc, double *scratch, long long scratch_len)
{
    apply_qt(m, n, k, i, mt, A, lda, T, ldt, C, ldc, Work{scratch, scratch_len});
}

// Q(i:m, j:j+n) := H [0; Q(i+k:m, j:j+n)], tiles backward.
// lila-c/lila_dormqrbz_w03.c:12-62.
static void apply_q_bz(int m, int n, int k, int i, int j, int mt, const double *A, int lda,
                       double *Q, int ldq, const double *T, int ldt, Work w)
{
    if (n <= 0 || k <= 0) return;
    int vbmax = imin(mt, k);
    double *W1 = w.take((long long)vbmax * n);
    double *W2 = w.take((long long)vbmax * n);
    double *X = Q + (size_t)j * ldq;
    // tile starts, walked backward
    int b = i + k;
    while (b > i) {
        int a = ((b - 1) / mt) * mt;
        if (a < i) a = i;
        int vb = b - a;
        const double *V = A + a + (size_t)a * lda;
        const double *Vbot = A + b + (size_t)a * lda;
        const double *Tt = T + a % mt + (size_t)a * ldt;
        gemm(vb, n, m - b, opnd(Vbot, lda, TR), opnd(X + b, ldq), W1, vb, epi(1, 0), w.p, w.len);
        gemm(vb, n, vb, opnd(Tt, ldt, NT, M_UPPER), opnd(W1, vb), W2, vb, epi(1, 0));
        GemmEpi e = epi(-1, 1);
        e.zero_rows = vb;
        gemm(m - a, n, vb, opnd(V, lda, NT, M_UNIT_LOWER), opnd(W2, vb), X + a, ldq, e);
        b = a;
    }
}

// T12 = -T11 (V1^T V2) T22 within one tile.  lila-c/lila_dlarft_connect_w03.c:3-32.
static void connect(int m, int n, int i, int j, int mt, const double *A, int lda, double *T,
                    int ldt, Work w)
{
    int vb = imin(mt - i % mt, n);
    int wb = (j / mt == i / mt) ? i - j : i % mt;
    if (wb == mt) wb = 1;
    if (wb <= 0 || vb <= 0) return;
    double *G = w.take((long long)wb * vb);
    double *Y = w.take((long long)wb * vb);
    const double *V1 = A + i + (size_t)(i - wb) * lda;
    const double *V2 = A + i + (size_t)i * lda;
    double *Tki = T + i % mt + (size_t)i * ldt;
    double *Tji = T + (i % mt - wb) + (size_t)i * ldt;
    double *Tjj = T + (i % mt - wb) + (size_t)(i - wb) * ldt;
    gemm(wb, vb, m - i, opnd(V1, lda, TR), opnd(V2, lda, NT, M_UNIT_LOWER), G, wb, epi(1, 0), w.p, w.len);
    gemm(wb, vb, wb, opnd(Tjj, ldt, NT, M_UPPER), opnd(G, wb), Y, wb, epi(1, 0));
    gemm(wb, vb, vb, opnd(Y, wb), opnd(Tki, ldt, NT, M_UPPER), Tji, ldt, epi(-1, 0));
}

// ---------------------------------------------------------------------------
// panels
// ---------------------------------------------------------------------------

// Elmroth-Gustavson recursive QR, lila-c/dgeqr3.c:3-114.  W lives in `w`
// instead of T's strictly upper part; the final T is the same.
static void dgeqr3_dev(int m, int n, double *A, int lda, double *T, int ldt, Work w)
{
    if (n <= 0) return;
    // the same V, R, T in one cooperative launch when the panel fits
    if (n >= 2 && w.len >= panel_coop_work(n) && panel_coop(m, n, A, lda, T, ldt, w.p)) return;
    if (n == 1) {
        larfg(m, A, T);
        return;
    }
    int n1 = n / 2, n2 = n - n1;
    dgeqr3_dev(m, n1, A, lda, T, ldt, w);
    Work w2 = w;
    double *W1 = w2.take((long long)n1 * n2);
    double *W2 = w2.take((long long)n1 * n2);
    double *A12 = A + (size_t)n1 * lda;
    gemm(n1, n2, m, opnd(A, lda, TR, M_UNIT_LOWER), opnd(A12, lda), W1, n1, epi(1, 0), w2.p, w2.len);
    gemm(n1, n2, n1, opnd(T, ldt, TR, M_UPPER), opnd(W1, n1), W2, n1, epi(1, 0));
    gemm(m, n2, n1, opnd(A, lda, NT, M_UNIT_LOWER), opnd(W2, n1), A12, lda, epi(-1, 1));
    double *A22 = A + n1 + (size_t)n1 * lda;
    double *T22 = T + n1 + (size_t)n1 * ldt;
    dgeqr3_dev(m - n1, n2, A22, lda, T22, ldt, w);
    // T12 = -T11 (Y1(n1:m)^T Y2) T22
    gemm(n1, n2, m - n1, opnd(A + n1, lda, TR), opnd(A22, lda, NT, M_UNIT_LOWER), W1, n1, epi(1, 0), w2.p, w2.len);
    gemm(n1, n2, n1, opnd(T, ldt, NT, M_UPPER), opnd(W1, n1), W2, n1, epi(1, 0));
    gemm(n1, n2, n2, opnd(W2, n1), opnd(T22, ldt, NT, M_UPPER), T + (size_t)n1 * ldt, ldt, epi(-1, 0));
}

// Q(0:ml, 0:n) = [I; 0] - V (T V1^T), T upper n x n with leading dim ldt.
static void explicit_q(int ml, int n, const double *V, int ldv, const double *T, int ldt, double *Q,
                       int ldq, Work w)
{
    double *Y = w.take((long long)n * n);
    gemm(n, n, n, opnd(T, ldt, NT, M_UPPER), opnd(V, ldv, TR, M_UNIT_LOWER), Y, n, epi(1, 0));
    GemmEpi e = epi(-1, 0);
    e.add_diag = 1;
    gemm(ml, n, n, opnd(V, ldv, NT, M_UNIT_LOWER), opnd(Y, n), Q, ldq, e);
}

// lila-c/lila_dgeqr2_w03_3.c:3-34 (and the LAPACK panel lila_dgeqr2_w03_l.c,
// whose V, R, T and Q are the same Householder quantities).
static void panel_hh(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt, double *Q,
                     int ldq, Work w)
{
    int ml = m - i;
    double *Aii = A + i + (size_t)i * lda;
    double *Qii = Q + i + (size_t)i * ldq;
    double *Tki = T + i % mt + (size_t)i * ldt;
    Work wq = w;
    wq.take((long long)n * n);  // keep the explicit-Q product apart from dgeqr3's scratch
    dgeqr3_dev(ml, n, Aii, lda, Tki, ldt, wq);
    explicit_q(ml, n, Aii, lda, Tki, ldt, Qii, ldq, w);
}

__global__ void k_move_strict_lower(int n, double *T, int ldt, double *A, int lda)
{
    int total = n * n;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
        int r = idx % n, c = idx / n;
        if (r > c) {
            A[(size_t)r + (size_t)c * lda] = T[(size_t)r + (size_t)c * ldt];
            T[(size_t)r + (size_t)c * ldt] = 0.0;
        }
    }
}

static void move_strict_lower(int n, double *T, int ldt, double *A, int lda)
{
    if (n <= 1) return;
    int blocks = (n * n + 255) / 256;
    k_move_strict_lower<<<blocks, 256, 0, stream()>>>(n, T, ldt, A, lda);
    note_launch("move_strict_lower");
}

void move_strict_lower_dev(int n, double *T, int ldt, double *A, int lda) { move_strict_lower(n, T, ldt, A, lda); }

// LU-with-sign reconstruction finishing steps shared by lila_dorgh2_3 and the
// tile routine: T holds the (reduced) top block, A(n:rows) the reduced rest.
// lila-c/lila_dorgh2_3.c:8-51.
static void reconstruct(int rows_v, int n, double *Ajj, int lda, double *Tjj, int ldt, double *Qc,
                        int q_rows, int ldq, double *S)
{
    lu_sign(n, Tjj, ldt, S);
    flip_rows(n, n, S, Ajj, lda, 1);
    flip_cols(q_rows, n, S, Qc, ldq);
    move_strict_lower(n, Tjj, ldt, Ajj, lda);
    trsm_right_upper(rows_v, n, 1.0, Tjj, ldt, Ajj + n, lda, S, "hr_trsm_v");
    trsm_right_lower_unit_trans(n, n, -1.0, Ajj, lda, Tjj, ldt);
}

// Cholesky QR of A(i:m, i:i+n) into Q, R into A's top block.
static void cholqr(int ml, int n, double *Aii, int lda, double *Qii, int ldq, Work w)
{
    copy2d(ml, n, Aii, lda, Qii, ldq);
    GemmEpi e = epi(1, 0);
    e.upper_only = 1;
    gemm(n, n, ml, opnd(Qii, ldq, TR), opnd(Qii, ldq), Aii, lda, e, w.p, w.len, "cholqr_gram");
    potrf_upper(n, Aii, lda);
    trsm_right_upper(ml, n, 1.0, Aii, lda, Qii, ldq, nullptr, "cholqr_trsm");
}

// lila-c/lila_dgeqr2_w03_hr.c:3-29.
static void panel_hr(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt, double *Q,
                     int ldq, Work w)
{
    int ml = m - i;
    double *S = w.take(n);
    double *Aii = A + i + (size_t)i * lda;
    double *Qii = Q + i + (size_t)i * ldq;
    double *Tki = T + i % mt + (size_t)i * ldt;
    cholqr(ml, n, Aii, lda, Qii, ldq, w);
    copy2d(ml - n, n, Qii + n, ldq, Aii + n, lda);
    copy2d(n, n, Qii, ldq, Tki, ldt);
    reconstruct(ml - n, n, Aii, lda, Tki, ldt, Qii, ml, ldq, S);
}

static void panel(const int *lp, int m, int n, int i, int mt, double *A, int lda, double *T,
                  int ldt, double *Q, int ldq, Work w)
{
    if (lp[2] == 2)
        panel_hr(m, n, i, mt, A, lda, T, ldt, Q, ldq, w);
    else
        panel_hh(m, n, i, mt, A, lda, T, ldt, Q, ldq, w);
}

// Tile j of a CholQR leaf starting at i.  lila-c/lila_ormhr2_w03_hr.c:3-84;
// scratch is w, S is separate (global index).
static void ormhr2(int m, int n, int i, int j, int mt, double *A, int lda, double *T, int ldt,
                   double *Q, int ldq, double *S, Work w)
{
    int jw = j - i;
    double *Qij = Q + i + (size_t)j * ldq;
    double *Qjj = Q + j + (size_t)j * ldq;
    double *Tjj = T + j % mt + (size_t)j * ldt;
    double *Aii = A + i + (size_t)i * lda;
    double *Ajj = A + j + (size_t)j * lda;
    double *Aji = A + j + (size_t)i * lda;
    flip_rows(jw, n, S + i, A + i + (size_t)j * lda, lda, 0);
    double *W2 = w.take((long long)jw * n);
    int ldw = jw > 0 ? jw : 1;
    copy2d(jw, n, Qij, ldq, W2, ldw);
    copy2d(n, n, Qjj, ldq, Tjj, ldt);
    copy2d(m - j - n, n, Qjj + n, ldq, Ajj + n, lda);
    if (jw > 0) {
        trsm_left_lower_unit(jw, n, Aii, lda, W2, ldw);
        gemm(n, n, jw, opnd(Aji, lda), opnd(W2, ldw), Tjj, ldt, epi(-1, 1));
        gemm(m - j - n, n, jw, opnd(Aji + n, lda), opnd(W2, ldw), Ajj + n, lda, epi(-1, 1), nullptr, 0,
             "hr_couple");
    }
    reconstruct(m - j - n, n, Ajj, lda, Tjj, ldt, Qij, m - i, ldq, S + j);
}

// ---------------------------------------------------------------------------
// leaves and drivers
// ---------------------------------------------------------------------------
// The tile loop of the Cholesky QR leaf, on an orthonormal Q and its R (upper
// part of A's leaf block) computed elsewhere (used by the TSQR leaf).
void hr_tiles(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt, double *Q, int ldq,
              double *S, double *work, long long lwork)
{
    Work w{work, lwork};
    for (int j = i; j < i + n;) {
        int vb = imin(tile_end(j, i + n, mt) - j, n);
        ormhr2(m, vb, i, j, mt, A, lda, T, ldt, Q, ldq, S, w);
        j += vb;
    }
}

static void mt_hh(const int *lp, int m, int n, int i, int mt, double *A, int lda, double *T,
                  int ldt, double *Q, int ldq, Work w)
{
    int vb = imin(mt - i % mt, n);
    panel(lp, m, vb, i, mt, A, lda, T, ldt, Q, ldq, w);
    for (int j = i + vb; j < i + n; j += vb) {
        vb = imin(mt, i + n - j);
        int l = j - i;
        apply_qt(m, vb, l, i, mt, A, lda, T, ldt, A + (size_t)j * lda, lda, w);
        panel(lp, m, vb, j, mt, A, lda, T, ldt, Q, ldq, w);
        apply_q_bz(m, vb, l, i, j, mt, A, lda, Q, ldq, T, ldt, w);
    }
}

// LAPACK leaf lila-c/lila_dgeqrf_w03_mt_l.c:3-22: one Householder QR of the
// whole leaf with its full n x n T, whose diagonal tile blocks are the
// per-tile dlarft factors; explicit Q from the full T.
__global__ void k_copy_upper(int n, const double *src, int lds, double *dst, int ldd)
{
    int total = n * n;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
        int r = idx % n, c = idx / n;
        if (r <= c) dst[(size_t)r + (size_t)c * ldd] = src[(size_t)r + (size_t)c * lds];
    }
}

// The per-tile T factors (diagonal blocks of the leaf's full n x n T, Tf)
// into the global tile layout.
static void tiles_from_full_t(int n, int i, int mt, const double *Tf, double *T, int ldt)
{
    for (int a = i; a < i + n;) {
        int b = tile_end(a, i + n, mt), vb = b - a;
        const double *src = Tf + (a - i) + (size_t)(a - i) * n;
        k_copy_upper<<<(vb * vb + 255) / 256, 256, 0, stream()>>>(vb, src, n, T + a % mt + (size_t)a * ldt, ldt);
        note_launch("copy_upper");
        a = b;
    }
}

static void mt_l(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt, double *Q,
                 int ldq, Work w)
{
    int ml = m - i;
    double *Aii = A + i + (size_t)i * lda;
    double *Qii = Q + i + (size_t)i * ldq;
    double *Tf = w.take((long long)n * n);
    Work wq = w;
    wq.take((long long)n * n);
    dgeqr3_dev(ml, n, Aii, lda, Tf, n, wq);
    tiles_from_full_t(n, i, mt, Tf, T, ldt);
    explicit_q(ml, n, Aii, lda, Tf, n, Qii, ldq, w);
}

// CholQR + Householder reconstruction leaf, lila-c/lila_dgeqrf_w03_mt_hr.c:3-33.
static void mt_hr(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt, double *Q,
                  int ldq, Work w)
{
    double *S = w.take(i + n);
    int ml = m - i;
    double *Aii = A + i + (size_t)i * lda;
    double *Qii = Q + i + (size_t)i * ldq;
    cholqr(ml, n, Aii, lda, Qii, ldq, w);
    for (int j = i; j < i + n;) {
        int vb = imin(tile_end(j, i + n, mt) - j, n);
        ormhr2(m, vb, i, j, mt, A, lda, T, ldt, Q, ldq, S, w);
        j += vb;
    }
}

static void leaf(const int *lp, int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                 double *Q, int ldq, Work w)
{
    switch (lp[1]) {
    case 0: mt_l(m, n, i, mt, A, lda, T, ldt, Q, ldq, w); break;
    case 1: mt_hh(lp, m, n, i, mt, A, lda, T, ldt, Q, ldq, w); break;
    case 2: mt_hr(m, n, i, mt, A, lda, T, ldt, Q, ldq, w); break;
    case 3: mixed_leaf_entry(m, n, i, mt, A, lda, T, ldt, Q, ldq, w.p, w.len, 0); break;
    }
}

// lila-c/lila_dgeqrf_w03_recursive.c:3-29.
static void recursive(const int *lp, int m, int n, int i, int mt, double *A, int lda, double *T,
                      int ldt, double *Q, int ldq, Work w)
{
    if (n <= lp[3]) {
        leaf(lp, m, n, i, mt, A, lda, T, ldt, Q, ldq, w);
        return;
    }
    int nb1 = n / 2, nb2 = n - nb1;
    recursive(lp, m, nb1, i, mt, A, lda, T, ldt, Q, ldq, w);
    apply_qt(m, nb2, nb1, i, mt, A, lda, T, ldt, A + (size_t)(i + nb1) * lda, lda, w);
    recursive(lp, m, nb2, i + nb1, mt, A, lda, T, ldt, Q, ldq, w);
    connect(m, nb2, i + nb1, i, mt, A, lda, T, ldt, w);
    apply_q_bz(m, nb2, nb1, i, i + nb1, mt, A, lda, Q, ldq, T, ldt, w);
}

// lila-c/lila_dgeqrf_w03_levelx.c:3-52.
static void levelx(const int *lp, int n_lvl, int i_lvl, const int *nb_lvl, int m, int n, int i,
                   int mt, double *A, int lda, double *T, int ldt, double *Q, int ldq, Work w)
{
    int nb = nb_lvl[i_lvl];
    int k = 0, j = i;
    while (j < i + n) {
        int vb = imin(nb, i + n - j);
        if (k > 0) apply_qt(m, vb, k, i, mt, A, lda, T, ldt, A + (size_t)j * lda, lda, w);
        if (i_lvl == n_lvl - 1)
            leaf(lp, m, vb, j, mt, A, lda, T, ldt, Q, ldq, w);
        else
            levelx(lp, n_lvl, i_lvl + 1, nb_lvl, m, vb, j, mt, A, lda, T, ldt, Q, ldq, w);
        if (k > 0) {
            connect(m, vb, j, i, mt, A, lda, T, ldt, w);
            apply_q_bz(m, vb, k, i, j, mt, A, lda, Q, ldq, T, ldt, w);
        }
        k += vb;
        j += vb;
    }
}

// ---------------------------------------------------------------------------
// V, R, T without Q (v03) and Q from V, T (q03)
// ---------------------------------------------------------------------------
// Both recursions stop at n < nx (w03 at n <= nx); a single column is always
// a leaf (the reference's recursion on one column with nx = 1 never ends).
// Leaf 2 and panel 2 are not implemented in the reference
// (lila-c/lila_dgeqrf_v03_mt.c:14-16, lila_dgeqr2_v03.c:13-15 and the q03
// twins): leaf 2 does nothing, panel 2 factors nothing while the tile loop
// around it still applies the earlier tiles, here as there.

// lila-c/lila_dgeqr2_v03_3.c:3-34 (its product T V1^T into the workspace is
// never read and is not formed) and lila_dgeqr2_v03_l.c:3-27 (dgeqrf +
// dlarft: the same V, R and T).
static void v03_panel(int panel, int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                      Work w)
{
    if (panel == 2) return;
    dgeqr3_dev(m - i, n, A + i + (size_t)i * lda, lda, T + i % mt + (size_t)i * ldt, ldt, w);
}

// lila-c/lila_dgeqrf_v03_mt_hh.c:3-35.
static void v03_mt_hh(int panel, int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                      Work w)
{
    int vb = imin(mt - i % mt, n);
    v03_panel(panel, m, vb, i, mt, A, lda, T, ldt, w);
    for (int j = i + vb; j < i + n; j += vb) {
        vb = imin(mt, i + n - j);
        apply_qt(m, vb, j - i, i, mt, A, lda, T, ldt, A + (size_t)j * lda, lda, w);
        v03_panel(panel, m, vb, j, mt, A, lda, T, ldt, w);
    }
}

// lila-c/lila_dgeqrf_v03_mt_l.c:3-19: one Householder QR of the leaf, the
// per-tile T factors (lila_dlarft_w03) from its full T.
static void v03_mt_l(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt, Work w)
{
    double *Tf = w.take((long long)n * n);
    dgeqr3_dev(m - i, n, A + i + (size_t)i * lda, lda, Tf, n, w);
    tiles_from_full_t(n, i, mt, Tf, T, ldt);
}

// lila-c/lila_dgeqrf_v03_mt.c:3-19.
static void v03_leaf(const int *lp, int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                     Work w)
{
    if (lp[1] == 0) v03_mt_l(m, n, i, mt, A, lda, T, ldt, w);
    if (lp[1] == 1) v03_mt_hh(lp[2], m, n, i, mt, A, lda, T, ldt, w);
}

// lila-c/lila_dgeqrf_v03_recursive.c:3-26.
static void v03_recursive(const int *lp, int m, int n, int i, int mt, double *A, int lda, double *T,
                          int ldt, Work w)
{
    if (n < lp[3] || n <= 1) {
        v03_leaf(lp, m, n, i, mt, A, lda, T, ldt, w);
        return;
    }
    int nb1 = n / 2, nb2 = n - nb1;
    v03_recursive(lp, m, nb1, i, mt, A, lda, T, ldt, w);
    apply_qt(m, nb2, nb1, i, mt, A, lda, T, ldt, A + (size_t)(i + nb1) * lda, lda, w);
    v03_recursive(lp, m, nb2, i + nb1, mt, A, lda, T, ldt, w);
    connect(m, nb2, i + nb1, i, mt, A, lda, T, ldt, w);
}

// lila-c/lila_dgeqrf_v03_levelx.c:3-47.
static void v03_levelx(const int *lp, int n_lvl, int i_lvl, const int *nb_lvl, int m, int n, int i,
                       int mt, double *A, int lda, double *T, int ldt, Work w)
{
    int nb = nb_lvl[i_lvl];
    int k = 0, j = i;
    while (j < i + n) {
        int vb = imin(nb, i + n - j);
        if (k > 0) apply_qt(m, vb, k, i, mt, A, lda, T, ldt, A + (size_t)j * lda, lda, w);
        if (i_lvl == n_lvl - 1)
            v03_leaf(lp, m, vb, j, mt, A, lda, T, ldt, w);
        else
            v03_levelx(lp, n_lvl, i_lvl + 1, nb_lvl, m, vb, j, mt, A, lda, T, ldt, w);
        if (k > 0) connect(m, vb, j, i, mt, A, lda, T, ldt, w);
        k += vb;
        j += vb;
    }
}

// Q(i:m, i:i+n) of one tile's reflectors: lila-c/lila_dgeqr2_q03_3.c:3-43
// ([I; 0] - V (T V1^T)) and lila_dgeqr2_q03_l.c:3-30 (dorgqr with tau =
// diag(T), the same Q).
static void q03_panel(int panel, int m, int n, int i, int mt, const double *A, int lda, const double *T,
                      int ldt, double *Q, int ldq, Work w)
{
    if (panel == 2) return;
    explicit_q(m - i, n, A + i + (size_t)i * lda, lda, T + i % mt + (size_t)i * ldt, ldt,
               Q + i + (size_t)i * ldq, ldq, w);
}

// lila-c/lila_dgeqrf_q03_mt_hh.c:3-32.
static void q03_mt_hh(int panel, int m, int n, int i, int mt, const double *A, int lda, const double *T,
                      int ldt, double *Q, int ldq, Work w)
{
    int vb = imin(mt - i % mt, n);
    q03_panel(panel, m, vb, i, mt, A, lda, T, ldt, Q, ldq, w);
    for (int j = i + vb; j < i + n; j += vb) {
        vb = imin(mt, i + n - j);
        q03_panel(panel, m, vb, j, mt, A, lda, T, ldt, Q, ldq, w);
        apply_q_bz(m, vb, j - i, i, j, mt, A, lda, Q, ldq, T, ldt, w);
    }
}

// lila-c/lila_dgeqrf_q03_mt_l.c:3-23 runs dorgqr over the whole leaf with tau
// from the T tiles, i.e. Q = H_i .. H_{i+n-1} [I; 0].  Only the per-tile T
// factors are stored, so the same product is formed tile by tile.
static void q03_mt_l(int m, int n, int i, int mt, const double *A, int lda, const double *T, int ldt,
                     double *Q, int ldq, Work w)
{
    q03_mt_hh(1, m, n, i, mt, A, lda, T, ldt, Q, ldq, w);
}

// lila-c/lila_dgeqrf_q03_mt.c:3-19.
static void q03_leaf(const int *lp, int m, int n, int i, int mt, const double *A, int lda, const double *T,
                     int ldt, double *Q, int ldq, Work w)
{
    if (lp[1] == 0) q03_mt_l(m, n, i, mt, A, lda, T, ldt, Q, ldq, w);
    if (lp[1] == 1) q03_mt_hh(lp[2], m, n, i, mt, A, lda, T, ldt, Q, ldq, w);
}

// lila-c/lila_dgeqrf_q03_recursive.c:3-25.
static void q03_recursive(const int *lp, int m, int n, int i, int mt, const double *A, int lda,
                          const double *T, int ldt, double *Q, int ldq, Work w)
{
    if (n < lp[3] || n <= 1) {
        q03_leaf(lp, m, n, i, mt, A, lda, T, ldt, Q, ldq, w);
        return;
    }
    int nb1 = n / 2, nb2 = n - nb1;
    q03_recursive(lp, m, nb1, i, mt, A, lda, T, ldt, Q, ldq, w);
    q03_recursive(lp, m, nb2, i + nb1, mt, A, lda, T, ldt, Q, ldq, w);
    apply_q_bz(m, nb2, nb1, i, i + nb1, mt, A, lda, Q, ldq, T, ldt, w);
}

// lila-c/lila_dgeqrf_q03_levelx.c:3-48.
static void q03_levelx(const int *lp, int n_lvl, int i_lvl, const int *nb_lvl, int m, int n, int i,
                       int mt, const double *A, int lda, const double *T, int ldt, double *Q, int ldq,
                       Work w)
{
    int nb = nb_lvl[i_lvl];
    int k = 0, j = i;
    while (j < i + n) {
        int vb = imin(nb, i + n - j);
        if (i_lvl == n_lvl - 1)
            q03_leaf(lp, m, vb, j, mt, A, lda, T, ldt, Q, ldq, w);
        else
            q03_levelx(lp, n_lvl, i_lvl + 1, nb_lvl, m, vb, j, mt, A, lda, T, ldt, Q, ldq, w);
        if (k > 0) apply_q_bz(m, vb, k, i, j, mt, A, lda, Q, ldq, T, ldt, w);
        k += vb;
        j += vb;
    }
}

// Workspace minima of the v03 / q03 routines (doubles); each is at most the
// w03 query of the same arguments.
static long long need_v03_mt(const int *lp, int n, int i, int mt)
{
    if (lp[1] == 0) return (long long)n * n + need_dgeqr3(n, false);
    if (lp[1] != 1) return 0;
    int vb = imin(mt - i % mt, n);
    long long need = lp[2] == 2 ? 0 : need_dgeqr3(vb, false);
    for (int j = i + vb; j < i + n; j += vb) {
        vb = imin(mt, i + n - j);
        need = lmax(need, need_apply(vb, j - i, mt, false));
        if (lp[2] != 2) need = lmax(need, need_dgeqr3(vb, false));
    }
    return need;
}

static long long need_q03_mt(const int *lp, int n, int i, int mt)
{
    if (lp[1] != 0 && lp[1] != 1) return 0;
    const int panel = lp[1] == 0 ? 1 : lp[2];
    int vb = imin(mt - i % mt, n);
    long long need = panel == 2 ? 0 : (long long)vb * vb;
    for (int j = i + vb; j < i + n; j += vb) {
        vb = imin(mt, i + n - j);
        need = lmax(need, need_apply(vb, j - i, mt, false));
        if (panel != 2) need = lmax(need, (long long)vb * vb);
    }
    return need;
}

static long long need_vq_recursive(bool v, const int *lp, int n, int i, int mt)
{
    if (n < lp[3] || n <= 1) return v ? need_v03_mt(lp, n, i, mt) : need_q03_mt(lp, n, i, mt);
    int nb1 = n / 2, nb2 = n - nb1;
    long long need = lmax(need_vq_recursive(v, lp, nb1, i, mt), need_vq_recursive(v, lp, nb2, i + nb1, mt));
    need = lmax(need, need_apply(nb2, nb1, mt, false));
    if (v) need = lmax(need, need_connect(nb2, mt, false));
    return need;
}

static long long need_vq_levelx(bool v, const int *lp, int n_lvl, int i_lvl, const int *nb_lvl, int n, int i,
                                int mt)
{
    int nb = nb_lvl[i_lvl];
    long long need = 0;
    int k = 0, j = i;
    while (j < i + n) {
        int vb = imin(nb, i + n - j);
        if (k > 0) {
            need = lmax(need, need_apply(vb, k, mt, false));
            if (v) need = lmax(need, need_connect(vb, mt, false));
        }
        if (i_lvl == n_lvl - 1)
            need = lmax(need, v ? need_v03_mt(lp, vb, j, mt) : need_q03_mt(lp, vb, j, mt));
        else
            need = lmax(need, need_vq_levelx(v, lp, n_lvl, i_lvl + 1, nb_lvl, vb, j, mt));
        k += vb;
        j += vb;
    }
    return need;
}

__global__ void k_tile_diag(int n, int i, int mt, const double *T, int ldt, double *tau)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < n) tau[c] = T[(size_t)((i + c) % mt) + (size_t)(i + c) * ldt];
}

// tau_c = 2 / (1 + ||A(c+1:m, c)||^2), one warp per column.
__global__ void k_v2tau(int m, int n, int i, const double *A, int lda, double *tau)
{
    int c = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    int lane = threadIdx.x % 32;
    if (c >= n) return;
    int gc = i + c;
    const double *v = A + (size_t)(gc + 1) + (size_t)gc * lda;
    double s = 0.0;
    for (int r = lane; r < m - gc - 1; r += 32) s = fma(v[r], v[r], s);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) tau[c] = 2.0 / (1.0 + s);
}

}  // namespace lg

// ===========================================================================
// C ABI
// ===========================================================================
using namespace lg;

// lila_param[1] (leaf): 0 LAPACK-style, 1 Householder tiles, 2 Cholesky QR +
// reconstruction (the reference's three), 3 the same leaf with split-precision
// tensor-core products (Cholesky QR 2 / shifted 3; leaves of at most 64 columns).
static bool bad_lp(const int *lp)
{
    return !lp || lp[1] < 0 || lp[1] > 3 || lp[2] < 0 || lp[2] > 2 || lp[3] < 1;
}

extern "C" {

int dgeqr3(int m, int n, double *A, int lda, double *T, int ldt)
{
    if (m < 0) return -1;
    if (n < 0 || n > m) return -2;
    if (!A && m * n) return -3;
    if (lda < imax(1, m)) return -4;
    if (!T && n) return -5;
    if (ldt < imax(1, n)) return -6;
    if (n == 0) return 0;
    // dgeqr3's lila.h signature carries no workspace: the scratch for the
    // off-diagonal products lives in a library-owned buffer cached per device
    // and size, reused across calls on the same stream order.
    static thread_local double *buf = nullptr;
    static thread_local long long buf_len = 0;
    long long need = need_dgeqr3(n, true);
    if (need > buf_len) {
        if (buf) {
            cudaStreamSynchronize(stream());
            cudaFree(buf);
        }
        buf = nullptr;
        buf_len = 0;
        if (cudaMalloc(&buf, (size_t)need * sizeof(double)) != cudaSuccess) return -100;
        buf_len = need;
    }
    Work w{buf, buf_len};
    dgeqr3_dev(m, n, A, lda, T, ldt, w);
    return 0;
}

int lila_query_dormqrf_w03(int m, int n, int k, int i, int j, int mt, double *A, int lda, double *T,
                           int ldt, double *work, int lwork)
{
    return clamp_query(need_apply(n, k, mt, true));
}

static int check_apply(int m, int n, int k, int i, int j, int mt, int lda, int ldt, long long lwork,
                       bool inplace)
{
    if (m < 0) return -1;
    if (n < 0) return -2;
    if (k < 0 || i + k > m) return -3;
    if (i < 0) return -4;
    if (j < 0 || (inplace && j < i + k && n > 0 && k > 0)) return -5;
    if (mt <= 0) return -6;
    if (lda < imax(1, m)) return -8;
    if (ldt < mt) return -10;
    if (lwork < need_apply(n, k, mt, false)) return -12;
    return 0;
}

int lila_dormqrf_w03(int m, int n, int k, int i, int j, int mt, double *A, int lda, double *T,
                     int ldt, double *work, int lwork)
{
    int e = check_apply(m, n, k, i, j, mt, lda, ldt, lwork, true);
    if (e) return e;
    return graph_call("dormqrf_w03", {(long long)m, (long long)n, (long long)k, (long long)i, (long long)j, (long long)mt, (long long)(uintptr_t)A, (long long)lda, (long long)(uintptr_t)T, (long long)ldt, (long long)(uintptr_t)work, (long long)lwork}, [&] {
        apply_qt(m, n, k, i, mt, A, lda, T, ldt, A + (size_t)j * lda, lda, Work{work, lwork});
        return 0;
    });
}

int lila_dormqrf_z03(int m, int n, int k, int i, int j, int mt, double *A, int lda, double *T,
                     int ldt, double *B, int ldb, double *work, int lwork)
{
    int e = check_apply(m, n, k, i, j, mt, lda, ldt, lwork, false);
    if (e) return e == -12 ? -14 : e;
    if (ldb < imax(1, m)) return -12;
    return graph_call("dormqrf_z03", {(long long)m, (long long)n, (long long)k, (long long)i, (long long)j, (long long)mt, (long long)(uintptr_t)A, (long long)lda, (long long)(uintptr_t)T, (long long)ldt, (long long)(uintptr_t)B, (long long)ldb, (long long)(uintptr_t)work, (long long)lwork}, [&] {
        apply_qt(m, n, k, i, mt, A, lda, T, ldt, B + (size_t)j * ldb, ldb, Work{work, lwork});
        return 0;
    });
}

int lila_query_dormqrbz_w03(int m, int n, int k, int i, int j, int mt, double *A, int lda,
                            double *Q, int ldq, double *T, int ldt, double *work, int lwork)
{
    return clamp_query(need_apply(n, k, mt, true));
}

int lila_dormqrbz_w03(int m, int n, int k, int i, int j, int mt, double *A, int lda, double *Q,
                      int ldq, double *T, int ldt, double *work, int lwork)
{
    if (m < 0) return -1;
    if (n < 0) return -2;
    if (k < 0 || i + k > m) return -3;
    if (i < 0) return -4;
    if (j < 0) return -5;
    if (mt <= 0) return -6;
    if (lda < imax(1, m)) return -8;
    if (ldq < imax(1, m)) return -10;
    if (ldt < mt) return -12;
    if (lwork < need_apply(n, k, mt, false)) return -14;
    return graph_call("dormqrbz_w03", {(long long)m, (long long)n, (long long)k, (long long)i, (long long)j, (long long)mt, (long long)(uintptr_t)A, (long long)lda, (long long)(uintptr_t)Q, (long long)ldq, (long long)(uintptr_t)T, (long long)ldt, (long long)(uintptr_t)work, (long long)lwork}, [&] {
        apply_q_bz(m, n, k, i, j, mt, A, lda, Q, ldq, T, ldt, Work{work, lwork});
        return 0;
    });
}

int lila_dlarft_connect_w03(int m, int n, int i, int j, int mt, double *A, int lda, double *T,
                            int ldt)
{
    if (m < 0) return -1;
    if (n < 0) return -2;
    if (i < 0 || i + n > m) return -3;
    if (j < 0 || j > i) return -4;
    if (mt <= 0) return -5;
    if (lda < imax(1, m)) return -7;
    if (ldt < mt) return -9;
    // the connect signature carries no workspace: use a per-thread cached buffer
    static thread_local double *buf = nullptr;
    static thread_local long long buf_len = 0;
    long long need = need_connect(n, mt, true);
    if (need > buf_len) {
        if (buf) {
            cudaStreamSynchronize(stream());
            cudaFree(buf);
        }
        buf = nullptr;
        buf_len = 0;
        if (cudaMalloc(&buf, (size_t)need * sizeof(double)) != cudaSuccess) return -100;
        buf_len = need;
    }
    connect(m, n, i, j, mt, A, lda, T, ldt, Work{buf, buf_len});
    return 0;
}

int lila_dlarft_w03(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                    double *tau)
{
    if (m < 0) return -1;
    if (n < 0 || i + n > m) return -2;
    if (i < 0) return -3;
    if (mt <= 0) return -4;
    if (lda < imax(1, m)) return -6;
    if (ldt < mt) return -8;
    if (n == 0) return 0;
    static thread_local double *buf = nullptr;
    static thread_local long long buf_len = 0;
    int vbmax = imin(mt, n);
    long long need = (long long)vbmax * vbmax + splitk_budget(vbmax, vbmax);
    if (need > buf_len) {
        if (buf) {
            cudaStreamSynchronize(stream());
            cudaFree(buf);
        }
        buf = nullptr;
        buf_len = 0;
        if (cudaMalloc(&buf, (size_t)need * sizeof(double)) != cudaSuccess) return -100;
        buf_len = need;
    }
    for (int a = i; a < i + n;) {
        int b = tile_end(a, i + n, mt), vb = b - a;
        const double *V = A + a + (size_t)a * lda;
        double *G = buf;
        gemm(vb, vb, m - a, opnd(V, lda, TR, M_UNIT_LOWER), opnd(V, lda, NT, M_UNIT_LOWER), G, vb,
             epi(1, 0), buf + (long long)vb * vb, buf_len - (long long)vb * vb);
        larft_from_gram(vb, G, vb, tau + (a - i), T + a % mt + (size_t)a * ldt, ldt);
        a = b;
    }
    return 0;
}

int lila_dT2tau_w03(int m, int n, int i, int mt, double *T, int ldt, double *tau)
{
    if (n < 0) return -2;
    if (mt <= 0) return -4;
    if (n == 0) return 0;
    k_tile_diag<<<(n + 255) / 256, 256, 0, stream()>>>(n, i, mt, T, ldt, tau);
    note_launch("tile_diag");
    return 0;
}

int lila_dV2tau_w03(int m, int n, int i, int mt, double *A, int lda, double *tau)
{
    if (n < 0 || i + n > m) return -2;
    if (lda < imax(1, m)) return -6;
    if (n == 0) return 0;
    k_v2tau<<<(n + 7) / 8, 256, 0, stream()>>>(m, n, i, A, lda, tau);
    note_launch("v2tau");
    return 0;
}

int lila_query_dorgh2_3(int m, int n, double *A, int lda, double *T, int ldt, double *Q, int ldq,
                        double *work, int lwork, double *S)
{
    return 0;
}

int lila_dorgh2_3(int m, int n, double *A, int lda, double *T, int ldt, double *Q, int ldq,
                  double *work, int lwork, double *S)
{
    if (m < 0) return -1;
    if (n < 0 || n > m) return -2;
    if (lda < imax(1, m)) return -4;
    if (ldt < imax(1, n)) return -6;
    if (ldq < imax(1, m)) return -8;
    if (!S && n) return -11;
    return graph_call("dorgh2_3", {(long long)m, (long long)n, (long long)(uintptr_t)A, (long long)lda, (long long)(uintptr_t)T, (long long)ldt, (long long)(uintptr_t)Q, (long long)ldq, (long long)(uintptr_t)S}, [&] {
        reconstruct(m - n, n, A, lda, T, ldt, Q, m, ldq, S);
        return 0;
    });
}

int lila_query_ormhr2_w03_hr(int m, int n, int i, int j, int l, int mt, double *A, int lda,
                             double *T, int ldt, double *Q, int ldq, double *work, int lwork,
                             double *S)
{
    return clamp_query(need_ormhr2(n, i, j, true));
}

int lila_ormhr2_w03_hr(int m, int n, int i, int j, int l, int mt, double *A, int lda, double *T,
                       int ldt, double *Q, int ldq, double *work, int lwork, double *S)
{
    if (m < 0) return -1;
    if (n < 0 || j + n > m) return -2;
    if (i < 0) return -3;
    if (j < i) return -4;
    if (mt <= 0 || (j % mt) + n > mt) return -6;
    if (lda < imax(1, m)) return -8;
    if (ldt < mt) return -10;
    if (ldq < imax(1, m)) return -12;
    if (lwork < need_ormhr2(n, i, j, false)) return -14;
    if (!S) return -15;
    return graph_call("ormhr2_w03_hr", {(long long)m, (long long)n, (long long)i, (long long)j, (long long)mt, (long long)(uintptr_t)A, (long long)lda, (long long)(uintptr_t)T, (long long)ldt, (long long)(uintptr_t)Q, (long long)ldq, (long long)(uintptr_t)S, (long long)(uintptr_t)work, (long long)lwork}, [&] {
        ormhr2(m, n, i, j, mt, A, lda, T, ldt, Q, ldq, S, Work{work, lwork});
        return 0;
    });
}

int lila_dorgh2(int m, int n, int i, int j, int mt, double *A, int lda, double *T, int ldt,
                double *Q, int ldq, double *work, int lwork, double *S)
{
    int e = lila_ormhr2_w03_hr(m, n, i, j, -1, mt, A, lda, T, ldt, Q, ldq, work, lwork, S);
    if (e < -5) e += 1;  // no `l` argument in this signature
    return e;
}

static int check_fact(int m, int n, int i, int mt, int lda, int ldt, int ldq, int base)
{
    // base = position of m in the argument list
    if (m < 0) return -(base);
    if (n < 0 || i + n > m) return -(base + 1);
    if (i < 0) return -(base + 2);
    if (mt <= 0) return -(base + 3);
    if (lda < imax(1, m)) return -(base + 5);
    if (ldt < mt) return -(base + 7);
    if (ldq < imax(1, m)) return -(base + 9);
    return 0;
}

int lila_query_dgeqr2_w03_3(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                            double *Q, int ldq, double *work, int lwork)
{
    return clamp_query(need_panel(1, n, true));
}
int lila_query_dgeqr2_w03_l(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                            double *Q, int ldq, double *work, int lwork)
{
    return clamp_query(need_panel(0, n, true));
}
int lila_query_dgeqr2_w03_hr(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                             double *Q, int ldq, double *work, int lwork)
{
    return clamp_query(need_panel(2, n, true));
}

static int panel_entry(int which, int m, int n, int i, int mt, double *A, int lda, double *T,
                       int ldt, double *Q, int ldq, double *work, int lwork)
{
    int e = check_fact(m, n, i, mt, lda, ldt, ldq, 1);
    if (e) return e;
    if ((i % mt) + n > mt) return -2;
    if (lwork < need_panel(which, n, false)) return -12;
    return graph_call("dgeqr2_w03", {(long long)which, (long long)m, (long long)n, (long long)i, (long long)mt, (long long)(uintptr_t)A, (long long)lda, (long long)(uintptr_t)T, (long long)ldt, (long long)(uintptr_t)Q, (long long)ldq, (long long)(uintptr_t)work, (long long)lwork}, [&] {
        int lp[4] = {0, 1, which, 0};
        panel(lp, m, n, i, mt, A, lda, T, ldt, Q, ldq, Work{work, lwork});
        return 0;
    });
}

int lila_dgeqr2_w03_l(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                      double *Q, int ldq, double *work, int lwork)
{
    return panel_entry(0, m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork);
}
int lila_dgeqr2_w03_3(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                      double *Q, int ldq, double *work, int lwork)
{
    return panel_entry(1, m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork);
}
int lila_dgeqr2_w03_hr(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                       double *Q, int ldq, double *work, int lwork)
{
    return panel_entry(2, m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork);
}

int lila_dgeqr2_w03(int *lila_param, int m, int n, int i, int mt, double *A, int lda, double *T,
                    int ldt, double *Q, int ldq, double *work, int lwork)
{
    if (bad_lp(lila_param)) return -1;
    int e = panel_entry(lila_param[2], m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork);
    return e ? e - 1 : 0;
}

int lila_query_dgeqrf_w03_mt_l(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                               double *Q, int ldq, double *work, int lwork)
{
    return clamp_query(need_mt_l(n, true));
}
int lila_query_dgeqrf_w03_mt_hr(int m, int n, int i, int mt, double *A, int lda, double *T,
                                int ldt, double *Q, int ldq, double *work, int lwork)
{
    return clamp_query(need_mt_hr(n, i, mt, true));
}
int lila_query_dgeqrf_w03_mt_hh(int *lila_param, int m, int n, int i, int mt, double *A, int lda,
                                double *T, int ldt, double *Q, int ldq, double *work, int lwork)
{
    if (bad_lp(lila_param) || mt <= 0) return 0;
    return clamp_query(need_mt_hh(lila_param[2], n, i, mt, true));
}
int lila_query_dgeqrf_w03_mt(int *lila_param, int m, int n, int i, int mt, double *A, int lda,
                             double *T, int ldt, double *Q, int ldq, double *work, int lwork)
{
    if (bad_lp(lila_param) || mt <= 0) return 0;
    return clamp_query(need_mt(lila_param, n, i, mt, true));
}
int lila_query_dgeqrf_w03_recursive(int *lila_param, int m, int n, int i, int mt, double *A,
                                    int lda, double *T, int ldt, double *Q, int ldq, double *work,
                                    int lwork)
{
    if (bad_lp(lila_param) || mt <= 0) return 0;
    return clamp_query(need_recursive(lila_param, n, i, mt, true));
}
int lila_query_dgeqrf_w03_levelx(int *lila_param, int n_lvl, int i_lvl, int *nb_lvl, int m, int n,
                                 int i, int mt, double *A, int lda, double *T, int ldt, double *Q,
                                 int ldq, double *work, int lwork)
{
    if (bad_lp(lila_param) || mt <= 0 || !nb_lvl || n_lvl <= 0 || i_lvl < 0 || i_lvl >= n_lvl) return 0;
    for (int l = i_lvl; l < n_lvl; l++)
        if (nb_lvl[l] <= 0) return 0;
    return clamp_query(need_levelx(lila_param, n_lvl, i_lvl, nb_lvl, n, i, mt, true));
}

int lila_dgeqrf_w03_mt_l(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                         double *Q, int ldq, double *work, int lwork)
{
    int e = check_fact(m, n, i, mt, lda, ldt, ldq, 1);
    if (e) return e;
    if (lwork < need_mt_l(n, false)) return -12;
    return graph_call("mt_l", {(long long)m, (long long)n, (long long)i, (long long)mt, (long long)(uintptr_t)A, (long long)lda, (long long)(uintptr_t)T, (long long)ldt, (long long)(uintptr_t)Q, (long long)ldq, (long long)(uintptr_t)work, (long long)lwork}, [&] {
        mt_l(m, n, i, mt, A, lda, T, ldt, Q, ldq, Work{work, lwork});
        return 0;
    });
}

int lila_dgeqrf_w03_mt_hr(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                          double *Q, int ldq, double *work, int lwork)
{
    int e = check_fact(m, n, i, mt, lda, ldt, ldq, 1);
    if (e) return e;
    if (lwork < need_mt_hr(n, i, mt, false)) return -12;
    return graph_call("mt_hr", {(long long)m, (long long)n, (long long)i, (long long)mt, (long long)(uintptr_t)A, (long long)lda, (long long)(uintptr_t)T, (long long)ldt, (long long)(uintptr_t)Q, (long long)ldq, (long long)(uintptr_t)work, (long long)lwork}, [&] {
        mt_hr(m, n, i, mt, A, lda, T, ldt, Q, ldq, Work{work, lwork});
        return 0;
    });
}

int lila_dgeqrf_w03_mt_hh(int *lila_param, int m, int n, int i, int mt, double *A, int lda,
                          double *T, int ldt, double *Q, int ldq, double *work, int lwork)
{
    if (bad_lp(lila_param)) return -1;
    int e = check_fact(m, n, i, mt, lda, ldt, ldq, 2);
    if (e) return e;
    if (lwork < need_mt_hh(lila_param[2], n, i, mt, false)) return -13;
    return graph_call("mt_hh", {lila_param[0], lila_param[1], lila_param[2], lila_param[3], (long long)m, (long long)n, (long long)i, (long long)mt, (long long)(uintptr_t)A, (long long)lda, (long long)(uintptr_t)T, (long long)ldt, (long long)(uintptr_t)Q, (long long)ldq, (long long)(uintptr_t)work, (long long)lwork}, [&] {
        mt_hh(lila_param, m, n, i, mt, A, lda, T, ldt, Q, ldq, Work{work, lwork});
        return 0;
    });
}

int lila_dgeqrf_w03_mt(int *lila_param, int m, int n, int i, int mt, double *A, int lda, double *T,
                       int ldt, double *Q, int ldq, double *work, int lwork)
{
    if (bad_lp(lila_param)) return -1;
    int e = check_fact(m, n, i, mt, lda, ldt, ldq, 2);
    if (e) return e;
    if (lila_param[1] == 3 && n > 64) return -3;
    if (lwork < need_mt(lila_param, n, i, mt, false)) return -13;
    return graph_call("mt", {lila_param[0], lila_param[1], lila_param[2], lila_param[3], (long long)m, (long long)n, (long long)i, (long long)mt, (long long)(uintptr_t)A, (long long)lda, (long long)(uintptr_t)T, (long long)ldt, (long long)(uintptr_t)Q, (long long)ldq, (long long)(uintptr_t)work, (long long)lwork}, [&] {
        leaf(lila_param, m, n, i, mt, A, lda, T, ldt, Q, ldq, Work{work, lwork});
        return 0;
    });
}

int lila_dgeqrf_w03_recursive(int *lila_param, int m, int n, int i, int mt, double *A, int lda,
                              double *T, int ldt, double *Q, int ldq, double *work, int lwork)
{
    if (bad_lp(lila_param)) return -1;
    int e = check_fact(m, n, i, mt, lda, ldt, ldq, 2);
    if (e) return e;
    if (lila_param[1] == 3 && lila_param[3] > 64 && n > 64) return -1;
    if (lwork < need_recursive(lila_param, n, i, mt, false)) return -13;
    return graph_call("recursive", {lila_param[0], lila_param[1], lila_param[2], lila_param[3], (long long)m, (long long)n, (long long)i, (long long)mt, (long long)(uintptr_t)A, (long long)lda, (long long)(uintptr_t)T, (long long)ldt, (long long)(uintptr_t)Q, (long long)ldq, (long long)(uintptr_t)work, (long long)lwork}, [&] {
        recursive(lila_param, m, n, i, mt, A, lda, T, ldt, Q, ldq, Work{work, lwork});
        return 0;
    });
}

int lila_dgeqrf_w03_levelx(int *lila_param, int n_lvl, int i_lvl, int *nb_lvl, int m, int n,
                           int i, int mt, double *A, int lda, double *T, int ldt, double *Q,
                           int ldq, double *work, int lwork)
{
    if (bad_lp(lila_param)) return -1;
    if (n_lvl <= 0) return -2;
    if (i_lvl < 0 || i_lvl >= n_lvl) return -3;
    if (!nb_lvl) return -4;
    for (int l = i_lvl; l < n_lvl; l++)
        if (nb_lvl[l] <= 0) return -4;
    int e = check_fact(m, n, i, mt, lda, ldt, ldq, 5);
    if (e) return e;
    if (lila_param[1] == 3 && nb_lvl[n_lvl - 1] > 64 && n > 64) return -4;
    if (lwork < need_levelx(lila_param, n_lvl, i_lvl, nb_lvl, n, i, mt, false)) return -16;
    if (n_lvl - i_lvl > 8) {
        levelx(lila_param, n_lvl, i_lvl, nb_lvl, m, n, i, mt, A, lda, T, ldt, Q, ldq, Work{work, lwork});
        return 0;
    }
    long long nb[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int l = i_lvl; l < n_lvl; l++) nb[l - i_lvl] = nb_lvl[l];
    return graph_call("levelx", {lila_param[0], lila_param[1], lila_param[2], lila_param[3], (long long)n_lvl,
                                 (long long)i_lvl, nb[0], nb[1], nb[2], nb[3], nb[4], nb[5], nb[6], nb[7], (long long)m, (long long)n, (long long)i, (long long)mt, (long long)(uintptr_t)A, (long long)lda, (long long)(uintptr_t)T, (long long)ldt, (long long)(uintptr_t)Q, (long long)ldq, (long long)(uintptr_t)work, (long long)lwork},
                      [&] {
                          levelx(lila_param, n_lvl, i_lvl, nb_lvl, m, n, i, mt, A, lda, T, ldt, Q, ldq,
                                 Work{work, lwork});
                          return 0;
                      });
}

int lila_dgeqrf_w03_appendcols(int *lila_param, int m, int k, int n, int mt, double *A, int lda,
                               double *Q, int ldq, double *T, int ldt, double *work, int lwork)
{
    if (bad_lp(lila_param)) return -1;
    if (m < 0) return -2;
    if (k < 0) return -3;
    if (n < 0 || k + n > m) return -4;
    if (mt <= 0) return -5;
    if (lda < imax(1, m)) return -7;
    if (ldq < imax(1, m)) return -9;
    if (ldt < mt) return -11;
    long long need = need_recursive(lila_param, n, k, mt, false);
    if (k) need = lmax(need, lmax(need_apply(n, k, mt, false), need_connect(n, mt, false)));
    if (lwork < need) return -13;
    Work w{work, lwork};
    if (k) apply_qt(m, n, k, 0, mt, A, lda, T, ldt, A + (size_t)k * lda, lda, w);
    recursive(lila_param, m, n, k, mt, A, lda, T, ldt, Q, ldq, w);
    if (k) {
        connect(m, n, k, 0, mt, A, lda, T, ldt, w);
        apply_q_bz(m, n, k, 0, k, mt, A, lda, Q, ldq, T, ldt, w);
    }
    return 0;
}

// Autotuner of the recursive driver's panel width mt and recursion cutoff
// nx (lila_param[3]) for one shape: every candidate factors a fresh copy of
// A (copied on the device outside the timed region) once to warm up and once
// timed with CUDA events on the library stream; the fastest is written back.
int lila_gpu_recursive_autotune(int *lila_param, int m, int n, const double *A, int lda, double *Ascratch,
                                double *T, int ldt, double *Q, int ldq, double *work, int lwork, int *mt_out)
{
    if (bad_lp(lila_param)) return -1;
    if (m < 1 || n < 1 || n > m) return -2;
    if (!A || !Ascratch || !T || !Q || !work || !mt_out) return -4;
    if (lda < m || ldq < m) return -5;
    const int cand_mt[4] = {32, 64, 128, 256};
    const int cand_nx[5] = {32, 64, 128, 256, 512};
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 3.0e38f;
    int bmt = 0, bnx = 0;
    for (int a = 0; a < 4; a++)
        for (int b = 0; b < 5; b++) {
            const int mt = cand_mt[a], nx = cand_nx[b];
            int lp[4] = {lila_param[0], lila_param[1], lila_param[2], nx};
            if (mt > ldt) continue;
            if (lp[1] == 3 && nx > 64) continue;  // the split-precision leaf takes at most 64 columns
            if (lwork < need_recursive(lp, n, 0, mt, false)) continue;
            float ms = 0.f;
            for (int rep = 0; rep < 2; rep++) {
                copy2d(m, n, A, lda, Ascratch, lda);
                cudaEventRecord(e0, stream());
                recursive(lp, m, n, 0, mt, Ascratch, lda, T, ldt, Q, ldq, Work{work, lwork});
                cudaEventRecord(e1, stream());
                cudaEventSynchronize(e1);
                cudaEventElapsedTime(&ms, e0, e1);
            }
            if (ms < best) {
                best = ms;
                bmt = mt;
                bnx = nx;
            }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!bmt) return -12;
    lila_param[3] = bnx;
    *mt_out = bmt;
    return (int)(best * 1000.0f);
}

// ---------------------------------------------------------------------------
// V, R, T without Q (v03) and Q from V, T (q03): lila.h:74-90 of the
// reference.  The reference has no workspace queries for them; the w03 query
// of the same arguments is always enough.  Leaf 3 (the split-precision leaf
// of this library) has no v03 / q03 form: lila_param[1] == 3 is rejected.
// ---------------------------------------------------------------------------
#define LL(x) ((long long)(x))
#define LP(x) ((long long)(uintptr_t)(x))

static bool bad_vq_lp(const int *lp) { return bad_lp(lp) || lp[1] == 3; }

int lila_dgeqr2_v03_3(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt, double *work,
                      int lwork)
{
    int e = check_fact(m, n, i, mt, lda, ldt, imax(1, m), 1);
    if (e) return e;
    if ((i % mt) + n > mt) return -2;
    if (lwork < need_dgeqr3(n, false)) return -10;
    return graph_call("dgeqr2_v03", {1, LL(m), LL(n), LL(i), LL(mt), LP(A), LL(lda), LP(T), LL(ldt), LP(work), LL(lwork)}, [&] {
        v03_panel(1, m, n, i, mt, A, lda, T, ldt, Work{work, lwork});
        return 0;
    });
}

int lila_dgeqr2_v03_l(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt, double *work,
                      int lwork)
{
    return lila_dgeqr2_v03_3(m, n, i, mt, A, lda, T, ldt, work, lwork);
}

int lila_dgeqr2_v03(int *lila_param, int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                    double *work, int lwork)
{
    if (bad_vq_lp(lila_param)) return -1;
    if (lila_param[2] == 2) return 0;
    int e = lila_dgeqr2_v03_3(m, n, i, mt, A, lda, T, ldt, work, lwork);
    return e ? e - 1 : 0;
}

int lila_dgeqrf_v03_mt_l(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt, double *work,
                         int lwork)
{
    int e = check_fact(m, n, i, mt, lda, ldt, imax(1, m), 1);
    if (e) return e;
    const int lp[4] = {0, 0, 0, 1};
    if (lwork < need_v03_mt(lp, n, i, mt)) return -10;
    return graph_call("v03_mt_l", {LL(m), LL(n), LL(i), LL(mt), LP(A), LL(lda), LP(T), LL(ldt), LP(work), LL(lwork)}, [&] {
        v03_mt_l(m, n, i, mt, A, lda, T, ldt, Work{work, lwork});
        return 0;
    });
}

static int v03_entry(const char *name, int *lp, int m, int n, int i, int mt, double *A, int lda, double *T,
                     int ldt, double *work, int lwork, bool recursive)
{
    if (bad_vq_lp(lp)) return -1;
    int e = check_fact(m, n, i, mt, lda, ldt, imax(1, m), 2);
    if (e) return e;
    if (lwork < (recursive ? need_vq_recursive(true, lp, n, i, mt) : need_v03_mt(lp, n, i, mt))) return -11;
    return graph_call(name, {LL(lp[0]), LL(lp[1]), LL(lp[2]), LL(lp[3]), LL(m), LL(n), LL(i), LL(mt), LP(A), LL(lda), LP(T), LL(ldt), LP(work), LL(lwork)}, [&] {
        Work w{work, lwork};
        if (recursive)
            v03_recursive(lp, m, n, i, mt, A, lda, T, ldt, w);
        else
            v03_leaf(lp, m, n, i, mt, A, lda, T, ldt, w);
        return 0;
    });
}

int lila_dgeqrf_v03_mt_hh(int *lila_param, int m, int n, int i, int mt, double *A, int lda, double *T,
                          int ldt, double *work, int lwork)
{
    if (bad_vq_lp(lila_param)) return -1;
    int lp[4] = {lila_param[0], 1, lila_param[2], lila_param[3]};
    return v03_entry("v03_mt_hh", lp, m, n, i, mt, A, lda, T, ldt, work, lwork, false);
}

int lila_dgeqrf_v03_mt(int *lila_param, int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                       double *work, int lwork)
{
    return v03_entry("v03_mt", lila_param, m, n, i, mt, A, lda, T, ldt, work, lwork, false);
}

int lila_dgeqrf_v03_recursive(int *lila_param, int m, int n, int i, int mt, double *A, int lda, double *T,
                              int ldt, double *work, int lwork)
{
    return v03_entry("v03_recursive", lila_param, m, n, i, mt, A, lda, T, ldt, work, lwork, true);
}

static int levelx_args(int *lp, int n_lvl, int i_lvl, const int *nb_lvl)
{
    if (bad_vq_lp(lp)) return -1;
    if (n_lvl <= 0) return -2;
    if (i_lvl < 0 || i_lvl >= n_lvl) return -3;
    if (!nb_lvl) return -4;
    for (int l = i_lvl; l < n_lvl; l++)
        if (nb_lvl[l] <= 0) return -4;
    return 0;
}

int lila_dgeqrf_v03_levelx(int *lila_param, int n_lvl, int i_lvl, int *nb_lvl, int m, int n, int i, int mt,
                           double *A, int lda, double *T, int ldt, double *work, int lwork)
{
    int e = levelx_args(lila_param, n_lvl, i_lvl, nb_lvl);
    if (e) return e;
    e = check_fact(m, n, i, mt, lda, ldt, imax(1, m), 5);
    if (e) return e;
    if (lwork < need_vq_levelx(true, lila_param, n_lvl, i_lvl, nb_lvl, n, i, mt)) return -14;
    v03_levelx(lila_param, n_lvl, i_lvl, nb_lvl, m, n, i, mt, A, lda, T, ldt, Work{work, lwork});
    return 0;
}

int lila_dgeqr2_q03_3(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt, double *Q, int ldq,
                      double *work, int lwork)
{
    int e = check_fact(m, n, i, mt, lda, ldt, ldq, 1);
    if (e) return e;
    if ((i % mt) + n > mt) return -2;
    if (lwork < (long long)n * n) return -12;
    return graph_call("dgeqr2_q03", {1, LL(m), LL(n), LL(i), LL(mt), LP(A), LL(lda), LP(T), LL(ldt), LP(Q), LL(ldq), LP(work), LL(lwork)}, [&] {
        q03_panel(1, m, n, i, mt, A, lda, T, ldt, Q, ldq, Work{work, lwork});
        return 0;
    });
}

int lila_dgeqr2_q03_l(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt, double *Q, int ldq,
                      double *work, int lwork)
{
    return lila_dgeqr2_q03_3(m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork);
}

int lila_dgeqr2_q03(int *lila_param, int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                    double *Q, int ldq, double *work, int lwork)
{
    if (bad_vq_lp(lila_param)) return -1;
    if (lila_param[2] == 2) return 0;
    int e = lila_dgeqr2_q03_3(m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork);
    return e ? e - 1 : 0;
}

int lila_dgeqrf_q03_mt_l(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt, double *Q,
                         int ldq, double *work, int lwork)
{
    int e = check_fact(m, n, i, mt, lda, ldt, ldq, 1);
    if (e) return e;
    const int lp[4] = {0, 0, 0, 1};
    if (lwork < need_q03_mt(lp, n, i, mt)) return -12;
    return graph_call("q03_mt_l", {LL(m), LL(n), LL(i), LL(mt), LP(A), LL(lda), LP(T), LL(ldt), LP(Q), LL(ldq), LP(work), LL(lwork)}, [&] {
        q03_mt_l(m, n, i, mt, A, lda, T, ldt, Q, ldq, Work{work, lwork});
        return 0;
    });
}

static int q03_entry(const char *name, int *lp, int m, int n, int i, int mt, double *A, int lda, double *T,
                     int ldt, double *Q, int ldq, double *work, int lwork, bool recursive)
{
    if (bad_vq_lp(lp)) return -1;
    int e = check_fact(m, n, i, mt, lda, ldt, ldq, 2);
    if (e) return e;
    if (lwork < (recursive ? need_vq_recursive(false, lp, n, i, mt) : need_q03_mt(lp, n, i, mt))) return -13;
    return graph_call(name, {LL(lp[0]), LL(lp[1]), LL(lp[2]), LL(lp[3]), LL(m), LL(n), LL(i), LL(mt), LP(A), LL(lda), LP(T), LL(ldt), LP(Q), LL(ldq), LP(work), LL(lwork)}, [&] {
        Work w{work, lwork};
        if (recursive)
            q03_recursive(lp, m, n, i, mt, A, lda, T, ldt, Q, ldq, w);
        else
            q03_leaf(lp, m, n, i, mt, A, lda, T, ldt, Q, ldq, w);
        return 0;
    });
}

int lila_dgeqrf_q03_mt_hh(int *lila_param, int m, int n, int i, int mt, double *A, int lda, double *T,
                          int ldt, double *Q, int ldq, double *work, int lwork)
{
    if (bad_vq_lp(lila_param)) return -1;
    int lp[4] = {lila_param[0], 1, lila_param[2], lila_param[3]};
    return q03_entry("q03_mt_hh", lp, m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork, false);
}

int lila_dgeqrf_q03_mt(int *lila_param, int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                       double *Q, int ldq, double *work, int lwork)
{
    return q03_entry("q03_mt", lila_param, m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork, false);
}

int lila_dgeqrf_q03_recursive(int *lila_param, int m, int n, int i, int mt, double *A, int lda, double *T,
                              int ldt, double *Q, int ldq, double *work, int lwork)
{
    return q03_entry("q03_recursive", lila_param, m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork, true);
}

int lila_dgeqrf_q03_levelx(int *lila_param, int n_lvl, int i_lvl, int *nb_lvl, int m, int n, int i, int mt,
                           double *A, int lda, double *T, int ldt, double *Q, int ldq, double *work, int lwork)
{
    int e = levelx_args(lila_param, n_lvl, i_lvl, nb_lvl);
    if (e) return e;
    e = check_fact(m, n, i, mt, lda, ldt, ldq, 5);
    if (e) return e;
    if (lwork < need_vq_levelx(false, lila_param, n_lvl, i_lvl, nb_lvl, n, i, mt)) return -16;
    q03_levelx(lila_param, n_lvl, i_lvl, nb_lvl, m, n, i, mt, A, lda, T, ldt, Q, ldq, Work{work, lwork});
    return 0;
}

#undef LL
#undef LP

}  // extern "C"
