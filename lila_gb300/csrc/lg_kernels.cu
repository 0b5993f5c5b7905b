// lg_kernels.cu -- FP64 building blocks of the GB300 LILA library.
//
// These are the general, shape-agnostic kernels every lila routine can be
// expressed with (masked GEMM with split-K, small triangular solves, one-CTA
// Cholesky / sign-choice LU / Householder generation).  FP64 on GB300 runs
// at roughly 2 DFMA per clock per SM, so one resident warp already keeps an
// SM's FP64 pipe busy: the kernels below are sized to put work on all 152
// SMs (split-K for the tall reductions) rather than for register reuse.
#include <math.h>

#include "lg_common.cuh"

namespace lg {

// ---------------------------------------------------------------------------
// masked GEMM
// ---------------------------------------------------------------------------
__device__ __forceinline__ double op_elem(const Operand &X, int r, int k)
{
    int sr = X.trans == NT ? r : k;
    int sc = X.trans == NT ? k : r;
    switch (X.mask) {
    case M_UNIT_LOWER:
        if (sr < sc) return 0.0;
        if (sr == sc) return 1.0;
        break;
    case M_UPPER:
        if (sr > sc) return 0.0;
        break;
    case M_LOWER:
        if (sr < sc) return 0.0;
        break;
    case M_UNIT_UPPER:
        if (sr > sc) return 0.0;
        if (sr == sc) return 1.0;
        break;
    default:
        break;
    }
    return X.p[(size_t)sr + (size_t)sc * (size_t)X.ld];
}

__device__ __forceinline__ void epilogue_store(double v, int r, int c, double *C, int ldc,
                                               const GemmEpi &e)
{
    if (e.upper_only && r > c) return;
    double out = e.alpha * v;
    if (e.add_diag && r == c) out += 1.0;
    size_t off = (size_t)r + (size_t)c * (size_t)ldc;
    if (e.beta != 0.0 && r >= e.zero_rows) out += e.beta * C[off];
    C[off] = out;
}

template <int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
    k_gemm(int M, int N, int K, int kchunk, Operand A, Operand B, double *C, int ldc, GemmEpi e,
           double *part)
{
    constexpr int RT = BM / TM;  // threads along rows
    constexpr int NTH = (BM / TM) * (BN / TN);
    __shared__ double As[BK][BM];
    __shared__ double Bs[BK][BN];
    const int tid = threadIdx.x;
    const int tr = tid % RT, tc = tid / RT;
    const int row0 = blockIdx.x * BM, col0 = blockIdx.y * BN;
    const int kbeg = blockIdx.z * kchunk;
    const int kend = min(K, kbeg + kchunk);
    double acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; i++)
#pragma unroll
        for (int j = 0; j < TN; j++) acc[i][j] = 0.0;

    for (int k0 = kbeg; k0 < kend; k0 += BK) {
        for (int idx = tid; idx < BM * BK; idx += NTH) {
            int r, k;
            if (A.trans == NT) {
                r = idx % BM;
                k = idx / BM;
            } else {
                k = idx % BK;
                r = idx / BK;
            }
            int gr = row0 + r, gk = k0 + k;
            As[k][r] = (gr < M && gk < kend) ? op_elem(A, gr, gk) : 0.0;
        }
        for (int idx = tid; idx < BN * BK; idx += NTH) {
            int c, k;
            if (B.trans == NT) {
                k = idx % BK;
                c = idx / BK;
            } else {
                c = idx % BN;
                k = idx / BN;
            }
            int gc = col0 + c, gk = k0 + k;
            Bs[k][c] = (gc < N && gk < kend) ? op_elem(B, gk, gc) : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < BK; k++) {
            double a[TM], b[TN];
#pragma unroll
            for (int i = 0; i < TM; i++) a[i] = As[k][tr + i * RT];
#pragma unroll
            for (int j = 0; j < TN; j++) b[j] = Bs[k][tc + j * (BN / TN)];
#pragma unroll
            for (int i = 0; i < TM; i++)
#pragma unroll
                for (int j = 0; j < TN; j++) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < TM; i++)
#pragma unroll
        for (int j = 0; j < TN; j++) {
            int r = row0 + tr + i * RT, c = col0 + tc + j * (BN / TN);
            if (r < M && c < N) {
                if (part)
                    part[(size_t)blockIdx.z * M * N + (size_t)r + (size_t)c * M] = acc[i][j];
                else
                    epilogue_store(acc[i][j], r, c, C, ldc, e);
            }
        }
}

__global__ void k_splitk_reduce(int M, int N, int splits, const double *part, double *C, int ldc,
                                GemmEpi e)
{
    size_t total = (size_t)M * N;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int z = 0; z < splits; z++) s += part[(size_t)z * total + idx];
        int r = (int)(idx % M), c = (int)(idx / M);
        epilogue_store(s, r, c, C, ldc, e);
    }
}

// SM count of the current device (queried once), for the grid heuristics
static int num_sm() { return sm_count(); }

static inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

int gemm_splits(int M, int N, int K, long long part_len)
{
    if (M <= 0 || N <= 0 || K <= 512) return 1;
    const int BM = (M * (long long)N >= 64LL * 64 * 2 * num_sm()) ? 64 : 32;
    long long tiles = (long long)ceil_div(M, BM) * ceil_div(N, BM);
    if (tiles >= 2 * num_sm()) return 1;
    int s = ceil_div(K, 256);
    s = s < ceil_div(4 * num_sm(), tiles) ? s : ceil_div(4 * num_sm(), tiles);
    if (s > 128) s = 128;
    long long fit = part_len / ((long long)M * N);
    if (s > fit) s = (int)fit;
    return s < 2 ? 1 : s;
}

void gemm(int M, int N, int K, Operand A, Operand B, double *C, int ldc, const GemmEpi &e,
          double *part, long long part_len, const char *tag)
{
    if (M <= 0 || N <= 0) return;
    // large products go to the tensor cores in split-precision mode
    if (precision() == 1 && M >= 64 && N >= 64 && K >= 64 && (double)M * N * K >= 134217728.0) {
        ozgemm(M, N, K, A, B, C, ldc, e, part, part_len, "ozgemm");
        return;
    }
    cudaStream_t st = stream();
    int splits = part ? gemm_splits(M, N, K, part_len) : 1;
    const bool big = (M * (long long)N >= 64LL * 64 * 2 * num_sm());
    int kchunk = K > 0 ? K : 1;
    if (splits > 1) {
        kchunk = ceil_div(ceil_div(K, splits), 16) * 16;
        splits = ceil_div(K, kchunk);
    }
    double *p = splits > 1 ? part : nullptr;
    trace_begin();
    if (big) {
        dim3 grid(ceil_div(M, 64), ceil_div(N, 64), splits);
        k_gemm<64, 64, 16, 4, 4><<<grid, 256, 0, st>>>(M, N, K, kchunk, A, B, C, ldc, e, p);
    } else {
        dim3 grid(ceil_div(M, 32), ceil_div(N, 32), splits);
        k_gemm<32, 32, 16, 2, 2><<<grid, 256, 0, st>>>(M, N, K, kchunk, A, B, C, ldc, e, p);
    }
    note_launch(tag);
    if (splits > 1) splitk_reduce(M, N, splits, part, C, ldc, e);
}

void splitk_reduce(int M, int N, int splits, const double *part, double *C, int ldc, const GemmEpi &e)
{
    long long total = (long long)M * N;
    int blocks = ceil_div(total, 256);
    if (blocks > 4 * num_sm()) blocks = 4 * num_sm();
    trace_begin();
    k_splitk_reduce<<<blocks, 256, 0, stream()>>>(M, N, splits, part, C, ldc, e);
    note_launch("splitk_reduce");
}

// ---------------------------------------------------------------------------
// element-wise helpers
// ---------------------------------------------------------------------------
__global__ void k_copy2d(int m, int n, const double *src, int lds, double *dst, int ldd)
{
    size_t total = (size_t)m * n;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        size_t r = idx % m, c = idx / m;
        dst[r + c * ldd] = src[r + c * lds];
    }
}

__global__ void k_copy2d_trans(int m, int n, const double *src, int lds, double *dst, int ldd)
{
    size_t total = (size_t)m * n;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        size_t r = idx % m, c = idx / m;
        dst[c + r * ldd] = src[r + c * lds];
    }
}

__global__ void k_set2d(int m, int n, double off, double diag, double *dst, int ldd, int uplo)
{
    size_t total = (size_t)m * n;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        int r = (int)(idx % m), c = (int)(idx / m);
        if (uplo == 1 && r > c) continue;
        if (uplo == 2 && r <= c) continue;
        dst[(size_t)r + (size_t)c * ldd] = (r == c) ? diag : off;
    }
}

__global__ void k_sub2d(int m, int n, const double *src, int lds, double *dst, int ldd)
{
    size_t total = (size_t)m * n;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        size_t r = idx % m, c = idx / m;
        dst[r + c * ldd] -= src[r + c * lds];
    }
}

__global__ void k_flip_rows(int nrows, int n, const double *S, double *X, int ldx, int upper)
{
    size_t total = (size_t)nrows * n;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        int k = (int)(idx % nrows), c = (int)(idx / nrows);
        if (upper && c < k) continue;
        if (S[k] == -1.0) X[(size_t)k + (size_t)c * ldx] = -X[(size_t)k + (size_t)c * ldx];
    }
}

__global__ void k_flip_cols(int m, int n, const double *S, double *X, int ldx)
{
    size_t total = (size_t)m * n;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        size_t r = idx % m, c = idx / m;
        if (S[c] == -1.0) X[r + c * ldx] = -X[r + c * ldx];
    }
}

static inline int ew_blocks(long long total)
{
    int b = ceil_div(total > 0 ? total : 1, 256);
    return b > 8 * num_sm() ? 8 * num_sm() : b;
}

void copy2d(int m, int n, const double *src, int lds, double *dst, int ldd)
{
    if (m <= 0 || n <= 0) return;
    trace_begin();
    k_copy2d<<<ew_blocks((long long)m * n), 256, 0, stream()>>>(m, n, src, lds, dst, ldd);
    note_launch("copy2d");
}
void copy2d_trans(int m, int n, const double *src, int lds, double *dst, int ldd)
{
    if (m <= 0 || n <= 0) return;
    k_copy2d_trans<<<ew_blocks((long long)m * n), 256, 0, stream()>>>(m, n, src, lds, dst, ldd);
    note_launch("copy2d_trans");
}
void set2d(int m, int n, double off, double diag, double *dst, int ldd, int uplo)
{
    if (m <= 0 || n <= 0) return;
    k_set2d<<<ew_blocks((long long)m * n), 256, 0, stream()>>>(m, n, off, diag, dst, ldd, uplo);
    note_launch("set2d");
}
void sub2d(int m, int n, const double *src, int lds, double *dst, int ldd)
{
    if (m <= 0 || n <= 0) return;
    k_sub2d<<<ew_blocks((long long)m * n), 256, 0, stream()>>>(m, n, src, lds, dst, ldd);
    note_launch("sub2d");
}
void flip_rows(int nrows, int n, const double *S, double *X, int ldx, int upper)
{
    if (nrows <= 0 || n <= 0) return;
    k_flip_rows<<<ew_blocks((long long)nrows * n), 256, 0, stream()>>>(nrows, n, S, X, ldx, upper);
    note_launch("flip_rows");
}
void flip_cols(int m, int n, const double *S, double *X, int ldx)
{
    if (m <= 0 || n <= 0) return;
    trace_begin();
    k_flip_cols<<<ew_blocks((long long)m * n), 256, 0, stream()>>>(m, n, S, X, ldx);
    note_launch("flip_cols");
}

// ---------------------------------------------------------------------------
// triangular solves
// ---------------------------------------------------------------------------
__global__ void k_trsm_left_lower_unit(int M, int N, const double *L, int ldl, double *B, int ldb)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    double *b = B + (size_t)c * ldb;
    for (int r = 1; r < M; r++) {
        double s = b[r];
        for (int p = 0; p < r; p++) s -= L[(size_t)r + (size_t)p * ldl] * b[p];
        b[r] = s;
    }
}

void trsm_left_lower_unit(int M, int N, const double *L, int ldl, double *B, int ldb)
{
    if (M <= 1 || N <= 0) return;
    k_trsm_left_lower_unit<<<ceil_div(N, 64), 64, 0, stream()>>>(M, N, L, ldl, B, ldb);
    note_launch("trsm_left_lower_unit");
}

// Row r of B solves x * U = alpha * S.*b.  U (N x N) is staged in shared
// memory when it fits; the row's solved prefix is re-read from global memory
// (coalesced across the threads of a warp, which own consecutive rows).
template <bool SMEM>
__global__ void k_trsm_right_upper(int M, int N, double alpha, const double *U, int ldu, double *B,
                                   int ldb, const double *S)
{
    extern __shared__ double Us[];
    if (SMEM) {
        for (int idx = threadIdx.x; idx < N * N; idx += blockDim.x) {
            int r = idx % N, c = idx / N;
            Us[idx] = (r <= c) ? U[(size_t)r + (size_t)c * ldu] : 0.0;
        }
        __syncthreads();
    }
    for (size_t r = blockIdx.x * (size_t)blockDim.x + threadIdx.x; r < (size_t)M;
         r += (size_t)gridDim.x * blockDim.x) {
        for (int c = 0; c < N; c++) {
            double s = alpha * B[r + (size_t)c * ldb];
            if (S && S[c] == -1.0) s = -s;
            for (int p = 0; p < c; p++) {
                double u = SMEM ? Us[p + c * N] : U[(size_t)p + (size_t)c * ldu];
                s -= B[r + (size_t)p * ldb] * u;
            }
            double d = SMEM ? Us[c + c * N] : U[(size_t)c + (size_t)c * ldu];
            B[r + (size_t)c * ldb] = s / d;
        }
    }
}

// The same solve for few rows (N <= 64): one warp per row, row r's 64
// values held two per lane; column c's dot product with the solved columns
// is split over the lanes and reduced by shuffles, so a row costs N
// reduction steps instead of N^2 / 2 dependent FMAs on one thread.
__global__ void __launch_bounds__(128) k_trsm_right_upper_warp(int M, int N, double alpha, const double *U, int ldu,
                                                                double *B, int ldb, const double *S)
{
    __shared__ double Us[64 * 64];
    for (int idx = threadIdx.x; idx < N * N; idx += blockDim.x) {
        const int r = idx % N, c = idx / N;
        Us[r + 64 * c] = (r <= c) ? U[(size_t)r + (size_t)c * ldu] : 0.0;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (row >= M) return;
    double b0 = lane < N ? B[(size_t)row + (size_t)lane * ldb] : 0.0;
    double b1 = lane + 32 < N ? B[(size_t)row + (size_t)(lane + 32) * ldb] : 0.0;
    double x0 = 0.0, x1 = 0.0;
    for (int c = 0; c < N; c++) {
        double s = alpha * __shfl_sync(0xffffffffu, c < 32 ? b0 : b1, c & 31);
        if (S && S[c] == -1.0) s = -s;
        double d = (lane < c ? x0 * Us[lane + 64 * c] : 0.0) + (lane + 32 < c ? x1 * Us[lane + 32 + 64 * c] : 0.0);
        for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
        const double x = (s - d) / Us[c + 64 * c];
        if (c < 32) {
            if (lane == c) x0 = x;
        } else if (lane == c - 32) {
            x1 = x;
        }
    }
    if (lane < N) B[(size_t)row + (size_t)lane * ldb] = x0;
    if (lane + 32 < N) B[(size_t)row + (size_t)(lane + 32) * ldb] = x1;
}

void trsm_right_upper(int M, int N, double alpha, const double *U, int ldu, double *B, int ldb,
                      const double *S, const char *tag)
{
    if (M <= 0 || N <= 0) return;
    if (N <= 64 && M <= 2048) {
        trace_begin();
        k_trsm_right_upper_warp<<<ceil_div(M, 4), 128, 0, stream()>>>(M, N, alpha, U, ldu, B, ldb, S);
        note_launch(tag);
        return;
    }
    int blocks = ceil_div(M, 128);
    if (blocks > 16 * num_sm()) blocks = 16 * num_sm();
    size_t sm = (size_t)N * N * sizeof(double);
    trace_begin();
    if (N <= 64) {
        k_trsm_right_upper<true><<<blocks, 128, sm, stream()>>>(M, N, alpha, U, ldu, B, ldb, S);
    } else {
        k_trsm_right_upper<false><<<blocks, 128, 0, stream()>>>(M, N, alpha, U, ldu, B, ldb, S);
    }
    note_launch(tag);
}

// Row r: x * L^T = alpha * b with L unit lower (so L^T unit upper).
__global__ void k_trsm_right_lower_unit_trans(int M, int N, double alpha, const double *L, int ldl,
                                              double *B, int ldb)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= M) return;
    for (int c = 0; c < N; c++) {
        double s = alpha * B[(size_t)r + (size_t)c * ldb];
        for (int p = 0; p < c; p++) s -= B[(size_t)r + (size_t)p * ldb] * L[(size_t)c + (size_t)p * ldl];
        B[(size_t)r + (size_t)c * ldb] = s;
    }
}

void trsm_right_lower_unit_trans(int M, int N, double alpha, const double *L, int ldl, double *B,
                                 int ldb)
{
    if (M <= 0 || N <= 0) return;
    k_trsm_right_lower_unit_trans<<<ceil_div(M, 64), 64, 0, stream()>>>(M, N, alpha, L, ldl, B, ldb);
    note_launch("trsm_right_lower_unit_trans");
}

// ---------------------------------------------------------------------------
// one-CTA factorizations
// ---------------------------------------------------------------------------
// Block-wide reduction; `ident` is the identity of `op` (0 for sums, 0 for
// maxima of absolute values), used for the lanes beyond the block's warps.
template <typename Op>
__device__ double block_reduce(double v, Op op, double *red, double ident = 0.0)
{
    for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
    int w = threadIdx.x / 32, l = threadIdx.x % 32;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    int nw = (blockDim.x + 31) / 32;
    if (w == 0) {
        v = (l < nw) ? red[l] : ident;
        for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (l == 0) red[32] = v;
    }
    __syncthreads();
    return red[32];
}

struct OpSum {
    __device__ double operator()(double a, double b) const { return a + b; }
};
struct OpMax {
    __device__ double operator()(double a, double b) const { return a > b ? a : b; }
};

// Cholesky G = U^T U (upper, in place), left-looking by rows.  On a
// non-positive pivot the status bit is set and the factorization stops
// (LAPACK dpotrf leaves the matrix partially factored the same way).
__global__ void k_potrf_upper(int n, double *A, int lda, int *status)
{
    __shared__ double red[33];
    __shared__ int bad;
    if (threadIdx.x == 0) bad = 0;
    for (int j = 0; j < n; j++) {
        double part = 0.0;
        for (int p = threadIdx.x; p < j; p += blockDim.x) {
            double a = A[(size_t)p + (size_t)j * lda];
            part += a * a;
        }
        double s = block_reduce(part, OpSum(), red);
        if (threadIdx.x == 0) {
            double d = A[(size_t)j + (size_t)j * lda] - s;
            if (!(d > 0.0)) {
                A[(size_t)j + (size_t)j * lda] = d;
                bad = 1;
                atomicOr(status, ST_CHOL_BREAKDOWN);
            } else {
                A[(size_t)j + (size_t)j * lda] = sqrt(d);
            }
        }
        __syncthreads();
        if (bad) return;
        double d = A[(size_t)j + (size_t)j * lda];
        for (int c = j + 1 + threadIdx.x; c < n; c += blockDim.x) {
            double t = A[(size_t)j + (size_t)c * lda];
            for (int p = 0; p < j; p++)
                t -= A[(size_t)p + (size_t)j * lda] * A[(size_t)p + (size_t)c * lda];
            A[(size_t)j + (size_t)c * lda] = t / d;
        }
        __syncthreads();
    }
}

__device__ int d_potrf_sink;

void potrf_upper(int n, double *A, int lda, bool record_breakdown)
{
    if (n <= 0) return;
    int *st = status_ptr();
    if (!record_breakdown) {
        void *p = nullptr;
        cudaGetSymbolAddress(&p, d_potrf_sink);
        st = (int *)p;
    }
    k_potrf_upper<<<1, 256, 0, stream()>>>(n, A, lda, st);
    note_launch("potrf_upper");
}

// LU without pivoting of (T S - I), S(k) = -1 when |1 - t_kk| < |1 + t_kk|
// (t_kk the partially eliminated diagonal), as in lila_dorgh2_3: column k is
// negated for S(k) = -1, the pivot is t_kk - 1, L below, U on/above.
__global__ void k_lu_sign(int n, double *T, int ldt, double *S, int *status)
{
    __shared__ double sgn, piv;
    for (int k = 0; k < n; k++) {
        if (threadIdx.x == 0) {
            double t = T[(size_t)k + (size_t)k * ldt];
            sgn = (fabs(1.0 - t) < fabs(1.0 + t)) ? -1.0 : 1.0;
            S[k] = sgn;
        }
        __syncthreads();
        if (sgn == -1.0)
            for (int r = threadIdx.x; r < n; r += blockDim.x)
                T[(size_t)r + (size_t)k * ldt] = -T[(size_t)r + (size_t)k * ldt];
        __syncthreads();
        if (threadIdx.x == 0) {
            double p = T[(size_t)k + (size_t)k * ldt] - 1.0;
            T[(size_t)k + (size_t)k * ldt] = p;
            piv = p;
            if (p == 0.0) atomicOr(status, ST_LU_ZERO_PIVOT);
        }
        __syncthreads();
        for (int r = k + 1 + threadIdx.x; r < n; r += blockDim.x)
            T[(size_t)r + (size_t)k * ldt] /= piv;
        __syncthreads();
        int w = n - k - 1;
        for (int idx = threadIdx.x; idx < w * w; idx += blockDim.x) {
            int r = k + 1 + idx % w, c = k + 1 + idx / w;
            T[(size_t)r + (size_t)c * ldt] -= T[(size_t)r + (size_t)k * ldt] * T[(size_t)k + (size_t)c * ldt];
        }
        __syncthreads();
    }
}

void lu_sign(int n, double *T, int ldt, double *S)
{
    if (n <= 0) return;
    k_lu_sign<<<1, 256, 0, stream()>>>(n, T, ldt, S, status_ptr());
    note_launch("lu_sign");
}

// LAPACK dlarfg on x(0:m): beta = -sign(alpha)*||x||, tau = (beta-alpha)/beta,
// v = x(1:m)/(alpha-beta); norm by max-scaled sum of squares.
__global__ void k_larfg(int m, double *x, double *tau)
{
    __shared__ double red[33];
    __shared__ double s_scale_inv;
    const double safmin = 2.2250738585072014e-308 / 1.1102230246251565e-16;
    int len = m - 1;
    double alpha = x[0];
    double *xs = x + 1;
    double mx = 0.0;
    for (int i = threadIdx.x; i < len; i += blockDim.x) mx = fmax(mx, fabs(xs[i]));
    double scale = block_reduce(mx, OpMax(), red);
    if (len <= 0 || scale == 0.0) {
        if (threadIdx.x == 0) *tau = 0.0;
        return;
    }
    double part = 0.0;
    for (int i = threadIdx.x; i < len; i += blockDim.x) {
        double t = xs[i] / scale;
        part += t * t;
    }
    double ssq = block_reduce(part, OpSum(), red);
    double xnorm = scale * sqrt(ssq);
    double beta = -copysign(hypot(alpha, xnorm), alpha);
    int knt = 0;
    if (fabs(beta) < safmin) {
        const double rsafmn = 1.0 / safmin;
        while (fabs(beta) < safmin && knt < 20) {
            knt++;
            for (int i = threadIdx.x; i < len; i += blockDim.x) xs[i] *= rsafmn;
            beta *= rsafmn;
            alpha *= rsafmn;
            __syncthreads();
        }
        mx = 0.0;
        for (int i = threadIdx.x; i < len; i += blockDim.x) mx = fmax(mx, fabs(xs[i]));
        scale = block_reduce(mx, OpMax(), red);
        part = 0.0;
        for (int i = threadIdx.x; i < len; i += blockDim.x) {
            double t = xs[i] / scale;
            part += t * t;
        }
        ssq = block_reduce(part, OpSum(), red);
        xnorm = scale * sqrt(ssq);
        beta = -copysign(hypot(alpha, xnorm), alpha);
    }
    if (threadIdx.x == 0) s_scale_inv = 1.0 / (alpha - beta);
    __syncthreads();
    double sc = s_scale_inv;
    for (int i = threadIdx.x; i < len; i += blockDim.x) xs[i] *= sc;
    if (threadIdx.x == 0) {
        *tau = (beta - alpha) / beta;
        for (int j = 0; j < knt; j++) beta *= safmin;
        x[0] = beta;
    }
}

void larfg(int m, double *x, double *tau)
{
    if (m <= 0) return;
    int th = m > 4096 ? 1024 : 256;
    k_larfg<<<1, th, 0, stream()>>>(m, x, tau);
    note_launch("larfg");
}

// dlarft recurrence from the Gram G = V^T V (only G(r, j), r < j used):
// T(j,j) = tau_j ; T(0:j, j) = T(0:j,0:j) * (-tau_j * G(0:j, j)).
__global__ void k_larft_from_gram(int k, const double *G, int ldg, const double *tau, double *T,
                                  int ldt)
{
    extern __shared__ double tmp[];
    for (int j = 0; j < k; j++) {
        double tj = tau[j];
        for (int r = threadIdx.x; r < j; r += blockDim.x)
            tmp[r] = (tj == 0.0) ? 0.0 : -tj * G[(size_t)r + (size_t)j * ldg];
        __syncthreads();
        for (int r = threadIdx.x; r < j; r += blockDim.x) {
            double s = 0.0;
            for (int c = r; c < j; c++) s += T[(size_t)r + (size_t)c * ldt] * tmp[c];
            T[(size_t)r + (size_t)j * ldt] = s;
        }
        if (threadIdx.x == 0) T[(size_t)j + (size_t)j * ldt] = tj;
        __syncthreads();
    }
}

void larft_from_gram(int k, const double *G, int ldg, const double *tau, double *T, int ldt)
{
    if (k <= 0) return;
    k_larft_from_gram<<<1, 256, (size_t)k * sizeof(double), stream()>>>(k, G, ldg, tau, T, ldt);
    note_launch("larft_from_gram");
}

__global__ void k_diag_to_vec(int n, const double *T, int ldt, double *out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = T[(size_t)i + (size_t)i * ldt];
}

void diag_to_vec(int n, const double *T, int ldt, double *out)
{
    if (n <= 0) return;
    k_diag_to_vec<<<ceil_div(n, 256), 256, 0, stream()>>>(n, T, ldt, out);
    note_launch("diag_to_vec");
}

}  // namespace lg
