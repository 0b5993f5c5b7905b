// lg_common.cuh -- shared declarations of the GB300 (sm_103a) LILA library.
//
// Conventions used everywhere in this library:
//   * column-major FP64 matrices, LP64 int dimensions, leading dimensions in
//     elements; element (r, c) of X lives at X[r + c*ld];
//   * every matrix pointer handed to a kernel is a device pointer;
//   * all work is enqueued on the calling thread's library stream
//     (lila_gpu_set_stream), asynchronously, in stream order;
//   * the reflector tile [a, b) of a block of Householder vectors has its
//     compact-WY factor at T + (a % mt) + a*ldt (global-index T layout of
//     the lila w03 interface).
#pragma once

#include <functional>
#include <initializer_list>

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

namespace lg {

// ---- error / status -------------------------------------------------------
// Status bits written by kernels (atomicOr) into a per-device word; read with
// lila_gpu_status().  Kernels never trap: they record and carry on.
enum StatusBits : int {
    ST_CHOL_BREAKDOWN = 1,   // non-positive pivot in a Cholesky factorization
    ST_LU_ZERO_PIVOT = 2,    // zero pivot in the reconstruction LU
    ST_NONFINITE = 4,        // a non-finite value reached a checked output
    ST_CHECK_FAILED = 8,     // an on-device accuracy check exceeded its bound
    ST_WAIT_TIMEOUT = 16,    // a bounded device-side wait gave up
    ST_LAUNCH_ERROR = 32,    // a kernel launch returned an error (host side)
};

int *status_ptr();            // device address of this device's status word
long long wait_limit();       // clock-cycle limit of the grid-barrier waits (lila_gpu_set_wait_limit)
double *noalloc_scratch_addr();  // device address of the no-allocation scratch array (lg_noalloc.cu)
cudaStream_t stream();        // current library stream of this host thread
void note_launch(const char *what);   // count, check cudaGetLastError, close a trace
void trace_begin();                   // open a CUDA-event trace of the next launch
void trace_cancel();                  // drop the open trace (the launch did not happen)
void trace_break();                   // untraced stream work follows: the next trace starts its own event
// Run body, or replay the CUDA graph captured from an earlier call with the
// same arguments when graph mode is on (lila_gpu_graph_mode).
int graph_call(const char *fn, std::initializer_list<long long> args, const std::function<int()> &body);

// ---- operand descriptors for the masked GEMM ------------------------------
enum Trans : int { NT = 0, TR = 1 };
// Structural masks applied to the STORED operand (before op()):
enum Mask : int {
    M_FULL = 0,        // plain matrix
    M_UNIT_LOWER = 1,  // unit lower trapezoid: (r<c) -> 0, (r==c) -> 1
    M_UPPER = 2,       // upper triangle incl. diagonal: (r>c) -> 0
    M_LOWER = 3,       // lower triangle incl. diagonal: (r<c) -> 0
    M_UNIT_UPPER = 4,  // unit upper: (r>c) -> 0, (r==c) -> 1
};

struct Operand {
    const double *p;
    int ld;
    int trans;  // Trans
    int mask;   // Mask
};

static inline Operand opnd(const double *p, int ld, int trans = NT, int mask = M_FULL)
{
    Operand o;
    o.p = p;
    o.ld = ld;
    o.trans = trans;
    o.mask = mask;
    return o;
}

// ---- primitive launchers (lg_kernels.cu) -----------------------------------
// C(MxN) = alpha*op(A)*op(B) + beta*C.  Rows r < zero_rows of C take beta = 0
// (C is not read there); add_diag adds 1 to C(r,r); upper_only stores only
// r <= c.  When `part` is non-null and splits > 1, the K range is split over
// `splits` CTA slices whose partial products go to part[s*M*N ...] (ld M)
// and a reduction kernel finishes the epilogue.  K may be 0.
struct GemmEpi {
    double alpha = 1.0;
    double beta = 0.0;
    int zero_rows = 0;
    int add_diag = 0;
    int upper_only = 0;
};
void gemm(int M, int N, int K, Operand A, Operand B, double *C, int ldc, const GemmEpi &e,
          double *part = nullptr, long long part_len = 0, const char *tag = "gemm");

// Number of split-K slices gemm() would use for this shape given `part_len`
// doubles of partial storage (1 = no split).
int gemm_splits(int M, int N, int K, long long part_len);
// Adds `splits` partial products part[z*M*N + r + c*M] and applies the epilogue.
void splitk_reduce(int M, int N, int splits, const double *part, double *C, int ldc, const GemmEpi &e);
// The same product at FP64 grade on the BF16 tensor cores (lg_ozgemm.cu).
void ozgemm(int M, int N, int K, Operand A, Operand B, double *C, int ldc, const GemmEpi &e,
            double *part = nullptr, long long part_len = 0, const char *tag = "ozgemm");
int ozgemm_splits(int M, int N, int K, long long part_len);
// Many independent split-precision GEMMs in one launch: C = alpha op(A) op(B)
// + beta C per group; d_prefix[g] = tiles of groups 0..g-1 (ozgemm_group_tiles
// each), total_tiles = all of them; d_tilemap (total_tiles entries) is
// scratch for the tile -> (group, tile) table.  Device arrays.
struct OzGroup {
    Operand A, B;
    double *C;
    int ldc, M, N, K;
    GemmEpi e;
    // optional precomputed scales over the whole K range: the largest biased
    // exponent of every row of op(A) (M ints) and column of op(B) (N ints)
    const int *rexp, *cexp;
};
// Row scales (largest biased exponent over n columns) of many column-major
// m x n matrices: job j writes rexp[0:m].  Device arrays.
struct RowExpJob {
    const double *A;
    int lda, m, n;
    int *rexp;
};
void row_exponents(const RowExpJob *d_jobs, int njobs);
int ozgemm_group_tiles(int M, int N);
// Many FP64-grade Grams in one launch: G(0:nm, 0:n) = A(:, 0:nm)^T A(:, 0:n)
// (nm = min(n, 128), n <= 192), one job per instance and 64-column block
// `half` of G's columns; the half-0 job's colexp (n ints) receives the column
// scales.  Device arrays.
struct GramW {
    const double *A;
    int lda, m, n;
    int *colexp;
    double *G;
    int ldg, half;
};
// The first nstacked jobs are diagonal blocks computed from their own 64
// columns (n <= 64, or the 64..127 block of a wider matrix); the others are
// first blocks of wider matrices (which also fill G(0:64, 64:128)) or the
// block of columns 128.. .
void ozaki_grams(const GramW *d_jobs, int njobs, int nstacked);
void ozgemm_groups(const OzGroup *d_groups, const int *d_prefix, int ngroups, int total_tiles, int2 *d_tilemap);
// Batched row maps out(:, col0 : col0 + ncols) = A X(:, col0 : col0 + ncols)
// at FP64 grade, X upper triangular (rows >= kend are zero, kend <= 128),
// A m x K column-major; rexp (m ints) and cexp (column scales of X) are the
// largest biased exponents of A's rows and X's columns.  One work item per
// instance and 64-column block; d_counter is one device int of scratch.
struct MapItem {
    const double *A;
    int lda, m;
    const double *X;
    int ldx, col0, ncols, kend;
    double *out;
    int ldo;
    const int *rexp, *cexp;
};
void map_items(const MapItem *d_items, int nitems, int *d_counter);
// Library precision of the large products: 0 FP64 CUDA cores, 1 FP64-grade
// split products on the tensor cores (lila_gpu_set_precision).
int precision();
// Householder QR of an m x nb panel (nb <= 64) in one cooperative launch
// (lg_panel.cu): V, R in A and the nb x nb T, as dgeqr3 returns them.
bool panel_coop_fits(int m, int nb);
long long panel_coop_work(int nb);
bool panel_coop(int m, int nb, double *A, int lda, double *T, int ldt, double *work);

// Copies / element-wise helpers.
void copy2d(int m, int n, const double *src, int lds, double *dst, int ldd);
void copy2d_trans(int m, int n, const double *src, int lds, double *dst, int ldd);  // dst = src^T (n x m)
void set2d(int m, int n, double offdiag, double diag, double *dst, int ldd, int uplo);  // uplo: 0 all, 1 strict upper+diag, 2 strict lower
void sub2d(int m, int n, const double *src, int lds, double *dst, int ldd);  // dst -= src
void flip_rows(int nrows, int n, const double *S, double *X, int ldx, int row_from_col);  // X(k, k*row_from_col + c) *= S(k) for c >= 0
void flip_cols(int m, int n, const double *S, double *X, int ldx);   // X(:, k) *= S(k)

// Triangular solves.
// Left, lower, unit, no-trans, small M (column per thread): B = L^-1 B.
void trsm_left_lower_unit(int M, int N, const double *L, int ldl, double *B, int ldb);
// Right, upper, non-unit, no-trans, row per thread: B = alpha * B * U^-1, with
// the optional column sign vector applied first (B(:,k) *= S(k)).
void trsm_right_upper(int M, int N, double alpha, const double *U, int ldu, double *B, int ldb,
                      const double *S = nullptr, const char *tag = "trsm_right_upper");
// Right, lower, unit, transposed (small n x n): B = alpha * B * L^-T.
void trsm_right_lower_unit_trans(int M, int N, double alpha, const double *L, int ldl, double *B,
                                 int ldb);

// Factorizations on one CTA.
void potrf_upper(int n, double *A, int lda, bool record_breakdown = true);
// LU without pivoting of (T*S - I) with the sign choice of lila_dorgh2_3.
void lu_sign(int n, double *T, int ldt, double *S);
// Householder vector of a column: LAPACK dlarfg on x(0:m) (alpha = x(0)),
// tau written to *tau.
void larfg(int m, double *x, double *tau);
// T(k x k) of forward columnwise reflectors from G = V^T V (k x k, upper part
// used) and tau (LAPACK dlarft recurrence).
void larft_from_gram(int k, const double *G, int ldg, const double *tau, double *T, int ldt);
// out(k) = T(k, k) for k < n.
void diag_to_vec(int n, const double *T, int ldt, double *out);
// Move the strict lower part of T (n x n) into A and zero it in T.
void move_strict_lower_dev(int n, double *T, int ldt, double *A, int lda);

// Split-precision FP64-grade products on the BF16 tensor cores (lg_ozaki.cu).
int sm_count();
long long ozaki_gram_work(int parts);
// colexp_ready: the first 64 ints of `work` already hold A's column scales
// (the largest biased exponent of every column), written by the ozaki_map
// that produced A; the scale pre-pass over A is skipped.
// pred (device int, may be null): the Gram's kernels do nothing when *pred
// is 0 at the time they run (a pass the device-side pass control skipped).
// rexp_out (m ints, may be null): the scale pre-pass (colexp not ready)
// also writes A's row scales there, for a following ozaki_map of A.
int ozaki_gram(int m, int n, const double *A, int lda, double *G, int ldg, double *work, long long lwork,
               int rows_per_override = 0, bool colexp_ready = false, const int *pred = nullptr,
               int *rexp_out = nullptr);
// colexp_out (64 ints, may be null): receives the column scales of `out`,
// for a following ozaki_gram of `out` with colexp_ready; pred as for
// ozaki_gram.  rexp_in (m ints, may be null): A's row scales (the largest
// biased exponent of each row), which let the register-fed map run one K
// half ahead; rexp_out (m ints, may be null, only with rexp_in): receives
// out's row scales.  rexp_out may be rexp_in (each row's scale is read
// before it is written).
int ozaki_map(int m, int n, const double *A, int lda, const double *X, int ldx, int nout, double *out, int ldo,
              int *colexp_out = nullptr, const int *pred = nullptr, const int *rexp_in = nullptr,
              int *rexp_out = nullptr);
// One row map of the tall-skinny split-precision kernel.
struct MapJob {
    const double *A;
    int lda, m, n;
    const double *X;
    int ldx, nout;
    double *out;
    int ldo;
};
// Mixed-precision Cholesky QR 2/3 + Householder reconstruction leaf (lg_tsmixed.cu).
long long need_mixed_leaf(int n);
int mixed_leaf_entry(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt, double *Q, int ldq,
                     double *work, long long lwork, int variant);

#ifdef __CUDACC__
// 1 / sqrt(d) for a positive finite d: Newton–Raphson on f(y) = y^-2 - d,
// y <- y + y (1 - d y^2) / 2, two steps from the single-precision estimate
// rsqrtf of d scaled into [1, 4) by an even power of two (the seed's relative
// error below 2^-21 becomes ~2^-42, then rounding level; the result is
// within about 1.5 ulp).  The scalings and conversions are exact exponent
// and bit moves, so the pivot chain holds six FP64 operations.
__device__ __forceinline__ double rsqrt_nr(double d)
{
    int hi = __double2hiint(d);
    int lo = __double2loint(d);
    int adj = 0;
    if (((hi >> 20) & 0x7FF) == 0) {  // subnormal: scale by 2^64 first
        const double s = d * 0x1p64;
        hi = __double2hiint(s);
        lo = __double2loint(s);
        adj = 32;
    }
    const int e = ((hi >> 20) & 0x7FF) - 1023;
    const int k = e >> 1;  // floor(e / 2)
    const int hm = hi - 2 * k * 1048576;  // dm = d 2^-2k in [1, 4)
    const double dm = __hiloint2double(hm, lo);
    // dm as a float (mantissa truncated to 23 bits), its rsqrtf, and that as a double
    const float fm = __int_as_float((((hm >> 20) - 1023 + 127) << 23) | ((hm & 0xFFFFF) << 3) |
                                    (int)((unsigned)lo >> 29));
    const unsigned yb = __float_as_uint(rsqrtf(fm));
    double y = __hiloint2double((int)((((yb >> 23) - 127 + 1023) << 20) | ((yb & 0x7FFFFFu) >> 3)),
                                (int)((yb & 7u) << 29));
#pragma unroll
    for (int it = 0; it < 2; it++) {
        const double t = dm * y;
        const double r = fma(-t, y, 1.0);
        y = fma(0.5 * y, r, y);
    }
    // 1 / sqrt(d) = y 2^(adj - k)
    return __hiloint2double(__double2hiint(y) + (adj - k) * 1048576, __double2loint(y));
}
#endif

}  // namespace lg
