// lg_tsmixed.cu -- tall-skinny QR leaf with FP64-grade split-precision
// products: Cholesky QR 2 (shifted Cholesky QR 3 when the matrix is too
// ill-conditioned for the plain Gram) followed by Householder reconstruction,
// returning the same V, R, T and Q as lila_dgeqrf_w03_mt_hr
// (lila-c/lila_dgeqrf_w03_mt_hr.c:3-33, lila_ormhr2_w03_hr.c:3-84).
//
// Data flow for the leaf block A(i:m, i:i+n), ml = m - i, n <= 64:
//   G1 = A^T A                 (split-precision Gram, tensor cores)
//   R1 = chol(G1 [+ sigma I])  (FP64, one CTA; sigma only for the shifted form)
//   Q  = A R1^-1               (split-precision row map into the Q buffer)
//   repeat 1 or 2 times: G = Q^T Q, Rk = chol(G), R = Rk R, and, except for
//   the last pass, Q = Q Rk^-1 (in place)
//   with Xl = Rk^-1 of the last pass the final orthonormal factor is Q Xl; the
//   sign-choice LU of its top n x n block and the tile coupling of the
//   reconstruction are done on n x n FP64 matrices, yielding two n x n maps:
//   M_V (rows below the leaf's top block -> V) and M_Q = Xl S (-> Q S).
//   V(i+n:m) = Q M_V and Q = Q M_Q are two more split-precision row maps.
#include <math.h>

#include <algorithm>

#include "lg_common.cuh"
#include "../../include/lila.h"
#include "../../include/lila_gpu.h"

namespace lg {

static inline int imin2(int a, int b) { return a < b ? a : b; }
static inline int tile_end2(int a, int end, int mt)
{
    int b = (a / mt + 1) * mt;
    return b < end ? b : end;
}

// sigma = c * trace(G) added to the diagonal (shifted Cholesky QR), and the
// Cholesky-diagonal ratio used to pick the variant.
__global__ void k_shift_diag(int n, double *G, int ldg, double factor)
{
    __shared__ double tr;
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < n; k++) t += G[(size_t)k + (size_t)k * ldg];
        tr = t;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < n; k += blockDim.x) G[(size_t)k + (size_t)k * ldg] += factor * tr;
}

// flag[0] = 1 when the trial Cholesky factor R (n x n) broke down or its
// 1-norm condition estimate ||R||_1 ||R^-1||_1 (X = R^-1) exceeds `limit`.
__global__ void k_chol_check(int n, const double *R, int ldr, const double *X, int ldx, double limit, int *flag)
{
    __shared__ double nr[64], nx[64];
    __shared__ int bad;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
        double sr = 0.0, sx = 0.0;
        for (int r = 0; r <= c; r++) {
            sr += fabs(R[(size_t)r + (size_t)c * ldr]);
            sx += fabs(X[(size_t)r + (size_t)c * ldx]);
        }
        double d = R[(size_t)c + (size_t)c * ldr];
        if (!(d > 0.0) || !isfinite(sr) || !isfinite(sx)) bad = 1;
        nr[c] = sr;
        nx[c] = sx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int c = 0; c < n; c++) {
            a = fmax(a, nr[c]);
            b = fmax(b, nx[c]);
        }
        *flag = (bad || !(a * b <= limit)) ? 1 : 0;
    }
}

struct MixedWs {
    double *G, *R, *Rk, *X, *Tmp, *Qt, *Atop, *MV, *MQ, *W, *S;
    int *flag;
    double *oz;
    long long ozlen;
};

static long long mixed_ws_len(int n)
{
    // 10 n x n blocks (64 x 64), S, flag, Gram workspace
    return 10LL * 64 * 64 + 64 + 64 + ozaki_gram_work(sm_count());
}

static MixedWs carve(double *w, long long len)
{
    MixedWs s;
    const long long B = 64 * 64;
    s.G = w;
    s.R = w + B;
    s.Rk = w + 2 * B;
    s.X = w + 3 * B;
    s.Tmp = w + 4 * B;
    s.Qt = w + 5 * B;
    s.Atop = w + 6 * B;
    s.MV = w + 7 * B;
    s.MQ = w + 8 * B;
    s.W = w + 9 * B;
    s.S = w + 10 * B;
    s.flag = (int *)(w + 10 * B + 64);
    s.oz = w + 10 * B + 128;
    s.ozlen = len - (10 * B + 128);
    return s;
}

static GemmEpi ep(double a, double b)
{
    GemmEpi e;
    e.alpha = a;
    e.beta = b;
    return e;
}

// X = R^-1 for upper triangular R (n x n, ld n).
// X = R^-1 for the upper n x n R (n <= 64): CTA j (one warp) forms column j
// by back substitution, X(j, j) = 1 / R(j, j) and, for r = j - 1 .. 0,
// X(r, j) = -(sum_{p = r+1}^{j} R(r, p) X(p, j)) / R(r, r), the lanes
// splitting each row's dot product; the columns run on separate SMs.
__global__ void k_tri_inv_cols(int n, const double *R, int ldr, double *X, int ldx)
{
    __shared__ double xs[64];
    const int j = blockIdx.x, lane = threadIdx.x;
    for (int r = lane; r < n; r += 32) xs[r] = r == j ? 1.0 / R[j + (size_t)j * ldr] : 0.0;
    __syncwarp();
    for (int r = j - 1; r >= 0; r--) {
        double s = 0.0;
        for (int p = r + 1 + lane; p <= j; p += 32) s += R[r + (size_t)p * ldr] * xs[p];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) xs[r] = -s / R[r + (size_t)r * ldr];
        __syncwarp();
    }
    for (int r = lane; r < n; r += 32) X[r + (size_t)j * ldx] = xs[r];
}

static void tri_inverse(int n, const double *R, double *X)
{
    trace_begin();
    k_tri_inv_cols<<<n, 32, 0, stream()>>>(n, R, n, X, n);
    note_launch("tri_inverse");
}

static int g_last_variant = 0;

// The reconstruction on n x n data (lila-c/lila_ormhr2_w03_hr.c:23-80 per tile,
// with the tall rows deferred to the row maps): inputs Qt = top n rows of the
// final orthonormal factor, R (upper, final), Xl; outputs Atop (leaf top block
// of A: S R above the diagonal, L and V rows below), T tiles, S, MQ, MV.
static void reconstruct_small(int n, int i0, int mt, MixedWs &w, double *T, int ldt)
{
    // Atop = upper(R), strictly lower zero
    set2d(n, n, 0.0, 0.0, w.Atop, n, 0);
    GemmEpi e = ep(1, 0);
    copy2d(n, n, w.R, n, w.Tmp, n);
    set2d(n, n, 0.0, 0.0, w.Tmp, n, 2);
    copy2d(n, n, w.Tmp, n, w.Atop, n);
    for (int j = i0; j < i0 + n;) {
        const int nt = imin2(tile_end2(j, i0 + n, mt) - j, n);
        const int lj = j - i0;
        double *Tj = T + (j % mt) + (size_t)j * ldt;
        if (lj > 0) {
            flip_rows(lj, nt, w.S, w.Atop + (size_t)lj * n, n, 0);
            // W = L_prev^-1 Qt(0:lj, tile)
            copy2d(lj, nt, w.Qt + (size_t)lj * n, n, w.W, lj);
            trsm_left_lower_unit(lj, nt, w.Atop, n, w.W, lj);
            // Qt(lj:n, tile) -= Atop(lj:n, 0:lj) W
            gemm(n - lj, nt, lj, opnd(w.Atop + lj, n), opnd(w.W, lj), w.Qt + lj + (size_t)lj * n, n, ep(-1, 1));
            // MV(:, tile) = Xl(:, tile) - MV(:, 0:lj) W
            copy2d(n, nt, w.X + (size_t)lj * n, n, w.MV + (size_t)lj * n, n);
            gemm(n, nt, lj, opnd(w.MV, n), opnd(w.W, lj), w.MV + (size_t)lj * n, n, ep(-1, 1));
        } else {
            copy2d(n, nt, w.X, n, w.MV, n);
        }
        copy2d(nt, nt, w.Qt + lj + (size_t)lj * n, n, Tj, ldt);
        lu_sign(nt, Tj, ldt, w.S + lj);
        flip_rows(nt, nt, w.S + lj, w.Atop + lj + (size_t)lj * n, n, 1);
        move_strict_lower_dev(nt, Tj, ldt, w.Atop + lj + (size_t)lj * n, n);
        const int below = n - lj - nt;
        if (below > 0) {
            copy2d(below, nt, w.Qt + lj + nt + (size_t)lj * n, n, w.Atop + lj + nt + (size_t)lj * n, n);
            trsm_right_upper(below, nt, 1.0, Tj, ldt, w.Atop + lj + nt + (size_t)lj * n, n, w.S + lj, "hr_small");
        }
        trsm_right_upper(n, nt, 1.0, Tj, ldt, w.MV + (size_t)lj * n, n, w.S + lj, "hr_small");
        trsm_right_lower_unit_trans(nt, nt, -1.0, w.Atop + lj + (size_t)lj * n, n, Tj, ldt);
        j += nt;
    }
    (void)e;
    copy2d(n, n, w.X, n, w.MQ, n);
    flip_cols(n, n, w.S, w.MQ, n);
}

static int g_last_passes = 0;

// variant: 0 adaptive, 1 Cholesky QR 2 (never shifted), 2 first pass shifted.
// Each pass factors the Gram of the current orthonormal candidate (A for the
// first pass).  A pass whose trial Cholesky breaks down or whose factor has a
// 1-norm condition estimate above 1e7 is redone with the shift
// sigma = 11 (ml n + n (n + 1)) u ||Q||_F^2 (shifted Cholesky QR); the leaf
// stops after two consecutive unshifted passes (Cholesky QR 2), so a matrix
// of condition number kappa takes about log(kappa) / log(1/sqrt(sigma))
// shifted passes before the final two.
struct PassState {
    int plain_run = 0, shifted_passes = 0, passes = 0;
    static constexpr int max_passes = 8;
    bool more() const { return plain_run < 2 && passes < max_passes; }
};

// The factor of one pass from its Gram w.G: Rk (trial, else shifted), X =
// Rk^-1, R = Rk R.
static void factor_pass(int n, MixedWs &w, int variant, double shift_factor, PassState &ps)
{
    const double cond_limit = 1e7;
    bool shift = (variant == 2 && ps.passes == 0);
    if (!shift && variant != 1) {
        // trial factorization: its breakdown only selects the shift, so it
        // is not recorded in the status word
        copy2d(n, n, w.G, n, w.Rk, n);
        potrf_upper(n, w.Rk, n, false);
        tri_inverse(n, w.Rk, w.X);
        k_chol_check<<<1, 64, 0, stream()>>>(n, w.Rk, n, w.X, n, cond_limit, w.flag);
        note_launch("chol_check");
        int flag = 0;
        cudaMemcpyAsync(&flag, w.flag, sizeof(int), cudaMemcpyDeviceToHost, stream());
        cudaStreamSynchronize(stream());
        shift = flag != 0;
    } else if (!shift) {
        copy2d(n, n, w.G, n, w.Rk, n);
        potrf_upper(n, w.Rk, n);
        tri_inverse(n, w.Rk, w.X);
    }
    if (shift) {
        copy2d(n, n, w.G, n, w.Rk, n);
        k_shift_diag<<<1, 64, 0, stream()>>>(n, w.Rk, n, shift_factor);
        note_launch("shift_diag");
        potrf_upper(n, w.Rk, n);
        tri_inverse(n, w.Rk, w.X);
        ps.shifted_passes++;
        ps.plain_run = 0;
    } else {
        ps.plain_run++;
    }
    ps.passes++;
    // R = Rk R
    gemm(n, n, n, opnd(w.Rk, n, NT, M_UPPER), opnd(w.R, n, NT, M_UPPER), w.Tmp, n, ep(1, 0));
    copy2d(n, n, w.Tmp, n, w.R, n);
}

static int mixed_leaf(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt, double *Q, int ldq,
                      double *work, long long lwork, int variant)
{
    const int ml = m - i;
    double *Aii = A + i + (size_t)i * lda;
    double *Qii = Q + i + (size_t)i * ldq;
    MixedWs w = carve(work, lwork);
    const double u = 1.1102230246251565e-16;
    const double shift_factor = 11.0 * ((double)ml * n + (double)n * (n + 1)) * u;
    // R = I
    set2d(n, n, 0.0, 1.0, w.R, n, 0);
    const double *cur = Aii;  // current candidate (A, then the Q buffer)
    int cur_ld = lda;
    PassState ps;
    bool scales_ready = false;  // the map that produced cur left its column scales in the Gram workspace
    while (ps.more()) {
        ozaki_gram(ml, n, cur, cur_ld, w.G, n, w.oz, w.ozlen, 0, scales_ready);
        factor_pass(n, w, variant, shift_factor, ps);
        if (ps.more()) {
            ozaki_map(ml, n, cur, cur_ld, w.X, n, n, Qii, ldq, (int *)w.oz);
            cur = Qii;
            cur_ld = ldq;
            scales_ready = true;
        }
    }
    g_last_variant = ps.shifted_passes ? 2 : 1;
    g_last_passes = ps.passes;
    // the final orthonormal factor is cur * X; cur is the Q buffer unless the
    // matrix was already orthonormal enough after one pass (not reachable with
    // two required unshifted passes, kept for safety)
    if (cur != Qii) {
        copy2d(ml, n, cur, cur_ld, Qii, ldq);
        cur = Qii;
    }
    // top n rows of the final orthonormal factor, FP64 on n x n data
    gemm(n, n, n, opnd(Qii, ldq), opnd(w.X, n, NT, M_UPPER), w.Qt, n, ep(1, 0));
    reconstruct_small(n, i, mt, w, T, ldt);
    if (ml > n) ozaki_map(ml - n, n, Qii + n, ldq, w.MV, n, n, Aii + n, lda);
    ozaki_map(ml, n, Qii, ldq, w.MQ, n, n, Qii, ldq);
    copy2d(n, n, w.Atop, n, Aii, lda);
    return 0;
}

long long need_mixed_leaf(int n) { return mixed_ws_len(n); }

// ---------------------------------------------------------------------------
// Out-of-core form: the leaf above for an m x n matrix that stays in host
// memory.  The rows stream through the device in chunks of C rows on two
// copy streams (in, out) with two buffer slots, so the copies of chunk c + 1
// (and the write-back of chunk c - 1) overlap the work on chunk c.  Every
// pass reads A once: the factor candidate of pass p is A X_0 .. X_{p-1},
// recomputed per chunk by the same row maps the in-core leaf applies to the
// whole matrix (a row's map depends only on that row), instead of being
// stored.  The chunk Grams are summed in double-double (TwoSum), so the sum
// adds no rounding beyond the chunks' own.  The final pass writes V (rows
// n..m) into A and Q, as the in-core leaf does.
// ---------------------------------------------------------------------------

// hi + lo += g elementwise, exactly up to the final rounding of lo (TwoSum).
__global__ void k_twosum_acc(int len, const double *g, double *hi, double *lo)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < len; k += gridDim.x * blockDim.x) {
        const double a = hi[k], b = g[k];
        const double s = a + b;
        const double bb = s - a;
        const double e = (a - (s - bb)) + (b - bb);
        hi[k] = s;
        lo[k] += e;
    }
}

__global__ void k_twosum_fin(int len, const double *hi, const double *lo, double *out)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < len; k += gridDim.x * blockDim.x) out[k] = hi[k] + lo[k];
}

struct OocBufs {
    double *Xs;                     // the chain's factors inverses X_0 .. (8 blocks of 64 x 64)
    double *Ghi, *Glo, *Gc;         // the pass's Gram sum (double-double) and one chunk's Gram
    double *in[2], *mid[2], *vout[2];  // per slot: the chunk, the chain's other buffer, V rows
};

static int ooc_rows(int m, int n, int rows_per_chunk)
{
    long long c = rows_per_chunk > 0 ? rows_per_chunk : 1048576;
    c = c < n ? n : c;
    const long long mr = ((long long)m + 127) / 128 * 128;
    if (c > mr) c = mr;
    c = (c + 127) / 128 * 128;
    return (int)c;
}

// Doubles of the out-of-core workspace; carves it into w and b when base is set.
static long long ooc_layout(int n, int C, double *base, OocBufs *b)
{
    auto al = [](long long v) { return (v + 31) / 32 * 32; };
    const long long B = 64 * 64, CB = al((long long)C * n);
    long long off = al(mixed_ws_len(n));
    double **slots[3] = {b ? b->in : nullptr, b ? b->mid : nullptr, b ? b->vout : nullptr};
    if (b) {
        b->Xs = base + off;
        b->Ghi = base + off + 8 * B;
        b->Glo = base + off + 9 * B;
        b->Gc = base + off + 10 * B;
    }
    off += 11 * B;
    for (int k = 0; k < 3; k++)
        for (int s = 0; s < 2; s++) {
            if (b) slots[k][s] = base + off;
            off += CB;
        }
    return off;
}

static int ooc_leaf(int m, int n, int mt, double *Ah, int lda, double *T, int ldt, double *Qh, int ldq,
                    int rows_per_chunk, double *work, long long lwork)
{
    const int C = ooc_rows(m, n, rows_per_chunk);
    OocBufs b;
    ooc_layout(n, C, work, &b);
    MixedWs w = carve(work, mixed_ws_len(n));
    const long long B = 64 * 64;
    const int nch = (int)(((long long)m + C - 1) / C);
    const double u = 1.1102230246251565e-16;
    const double shift_factor = 11.0 * ((double)m * n + (double)n * (n + 1)) * u;
    cudaStream_t st = stream(), s_in = nullptr, s_out = nullptr;
    cudaEvent_t ev_in[2], ev_free[2], ev_done[2], ev_small;
    if (cudaStreamCreateWithFlags(&s_in, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s_out, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        if (s_in) cudaStreamDestroy(s_in);
        return -100;
    }
    for (int k = 0; k < 2; k++) {
        cudaEventCreateWithFlags(&ev_in[k], cudaEventDisableTiming);
        cudaEventCreateWithFlags(&ev_free[k], cudaEventDisableTiming);
        cudaEventCreateWithFlags(&ev_done[k], cudaEventDisableTiming);
        cudaEventRecord(ev_free[k], st);
    }
    cudaEventCreateWithFlags(&ev_small, cudaEventDisableTiming);
    auto rows_of = [&](int c) { return (int)std::min<long long>(C, (long long)m - (long long)c * C); };
    // a copy the runtime refuses (e.g. a host pointer it cannot reach) fails the call
    cudaError_t copy_err = cudaSuccess;
    auto chk = [&](cudaError_t e) {
        if (e != cudaSuccess && copy_err == cudaSuccess) copy_err = e;
    };
    // chunk c into slot s once the slot's previous chunk is done with
    auto load = [&](int c, int s) {
        cudaStreamWaitEvent(s_in, ev_free[s], 0);
        chk(cudaMemcpy2DAsync(b.in[s], (size_t)C * 8, Ah + (size_t)c * C, (size_t)lda * 8, (size_t)rows_of(c) * 8,
                              n, cudaMemcpyDefault, s_in));
        cudaEventRecord(ev_in[s], s_in);
    };
    // the candidate A X_0 .. X_{nx-1} of the chunk in slot s
    auto chain = [&](int s, int rows, int nx) {
        double *cur = b.in[s], *oth = b.mid[s];
        for (int p = 0; p < nx; p++) {
            ozaki_map(rows, n, cur, C, b.Xs + p * B, n, n, oth, C);
            std::swap(cur, oth);
        }
        return cur;
    };
    set2d(n, n, 0.0, 1.0, w.R, n, 0);
    PassState ps;
    int nx = 0;
    while (ps.more()) {
        set2d(n, n, 0.0, 0.0, b.Ghi, n, 0);
        set2d(n, n, 0.0, 0.0, b.Glo, n, 0);
        load(0, 0);
        for (int c = 0; c < nch; c++) {
            const int s = c & 1;
            if (c + 1 < nch) load(c + 1, s ^ 1);
            cudaStreamWaitEvent(st, ev_in[s], 0);
            double *cur = chain(s, rows_of(c), nx);
            ozaki_gram(rows_of(c), n, cur, C, b.Gc, n, w.oz, w.ozlen, 0, false);
            k_twosum_acc<<<(n * n + 255) / 256, 256, 0, st>>>(n * n, b.Gc, b.Ghi, b.Glo);
            note_launch("twosum_acc");
            cudaEventRecord(ev_free[s], st);
        }
        k_twosum_fin<<<(n * n + 255) / 256, 256, 0, st>>>(n * n, b.Ghi, b.Glo, w.G);
        note_launch("twosum_fin");
        factor_pass(n, w, 0, shift_factor, ps);
        if (ps.more()) copy2d(n, n, w.X, n, b.Xs + nx++ * B, n);
    }
    g_last_variant = ps.shifted_passes ? 2 : 1;
    g_last_passes = ps.passes;
    // top n rows of the final factor (chunk 0 holds them: C >= n), then the
    // reconstruction on n x n data
    load(0, 0);
    cudaStreamWaitEvent(st, ev_in[0], 0);
    double *cur0 = chain(0, rows_of(0), nx);
    gemm(n, n, n, opnd(cur0, C), opnd(w.X, n, NT, M_UPPER), w.Qt, n, ep(1, 0));
    cudaEventRecord(ev_free[0], st);
    reconstruct_small(n, 0, mt, w, T, ldt);
    // V rows into A (below the top n rows) and Q, chunk by chunk
    load(0, 0);
    for (int c = 0; c < nch; c++) {
        const int s = c & 1, rows = rows_of(c), skip = c == 0 ? n : 0;
        if (c + 1 < nch) load(c + 1, s ^ 1);
        cudaStreamWaitEvent(st, ev_in[s], 0);
        double *cur = chain(s, rows, nx);
        double *qout = cur == b.in[s] ? b.mid[s] : b.in[s];
        if (rows > skip) ozaki_map(rows - skip, n, cur + skip, C, w.MV, n, n, b.vout[s], C);
        ozaki_map(rows, n, cur, C, w.MQ, n, n, qout, C);
        cudaEventRecord(ev_done[s], st);
        cudaStreamWaitEvent(s_out, ev_done[s], 0);
        const size_t r0 = (size_t)c * C;
        if (rows > skip)
            chk(cudaMemcpy2DAsync(Ah + r0 + skip, (size_t)lda * 8, b.vout[s], (size_t)C * 8,
                                  (size_t)(rows - skip) * 8, n, cudaMemcpyDefault, s_out));
        chk(cudaMemcpy2DAsync(Qh + r0, (size_t)ldq * 8, qout, (size_t)C * 8, (size_t)rows * 8, n,
                              cudaMemcpyDefault, s_out));
        cudaEventRecord(ev_free[s], s_out);
    }
    // the top block of A (S R above the diagonal, L below)
    cudaEventRecord(ev_small, st);
    cudaStreamWaitEvent(s_out, ev_small, 0);
    chk(cudaMemcpy2DAsync(Ah, (size_t)lda * 8, w.Atop, (size_t)n * 8, (size_t)n * 8, n, cudaMemcpyDefault, s_out));
    cudaEventRecord(ev_small, s_out);
    cudaStreamWaitEvent(st, ev_small, 0);
    const cudaError_t e = cudaStreamSynchronize(st);
    for (int k = 0; k < 2; k++) {
        cudaEventDestroy(ev_in[k]);
        cudaEventDestroy(ev_free[k]);
        cudaEventDestroy(ev_done[k]);
    }
    cudaEventDestroy(ev_small);
    cudaStreamDestroy(s_in);
    cudaStreamDestroy(s_out);
    return (e == cudaSuccess && copy_err == cudaSuccess) ? 0 : -100;
}

int mixed_leaf_entry(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt, double *Q, int ldq,
                     double *work, long long lwork, int variant)
{
    return mixed_leaf(m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork, variant);
}

}  // namespace lg

using namespace lg;

extern "C" {

int lila_query_dgeqrf_w03_mt_hr_mixed(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt,
                                      double *Q, int ldq, double *work, int lwork)
{
    long long v = need_mixed_leaf(n);
    return v > 0x7fffffffLL ? 0x7fffffff : (int)v;
}

int lila_dgeqrf_w03_mt_hr_mixed_v(int variant, int m, int n, int i, int mt, double *A, int lda, double *T,
                                  int ldt, double *Q, int ldq, double *work, int lwork)
{
    if (variant < 0 || variant > 2) return -1;
    if (m < 0) return -2;
    if (n < 0 || n > 64 || i + n > m) return -3;
    if (i < 0) return -4;
    if (mt <= 0) return -5;
    if (lda < (m > 1 ? m : 1)) return -7;
    if (ldt < mt) return -9;
    if (ldq < (m > 1 ? m : 1)) return -11;
    if (lwork < need_mixed_leaf(n)) return -13;
    if (n == 0) return 0;
    return graph_call("mt_hr_mixed",
                      {(long long)variant, (long long)m, (long long)n, (long long)i, (long long)mt,
                       (long long)(uintptr_t)A, (long long)lda, (long long)(uintptr_t)T, (long long)ldt,
                       (long long)(uintptr_t)Q, (long long)ldq, (long long)(uintptr_t)work, (long long)lwork},
                      [&] { return mixed_leaf(m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork, variant); });
}

int lila_dgeqrf_w03_mt_hr_mixed(int m, int n, int i, int mt, double *A, int lda, double *T, int ldt, double *Q,
                                int ldq, double *work, int lwork)
{
    int e = lila_dgeqrf_w03_mt_hr_mixed_v(0, m, n, i, mt, A, lda, T, ldt, Q, ldq, work, lwork);
    return e < 0 ? e + 1 : e;
}

long long lila_gpu_query_dgeqrf_tall_host(int m, int n, int rows_per_chunk)
{
    if (m < 1 || n < 1 || n > 64 || m < n) return 0;
    return ooc_layout(n, ooc_rows(m, n, rows_per_chunk), nullptr, nullptr);
}

int lila_gpu_dgeqrf_tall_host(int m, int n, int mt, double *A, int lda, double *T, int ldt, double *Q, int ldq,
                              int rows_per_chunk, double *work, long long lwork)
{
    if (m < 0) return -1;
    if (n < 0 || n > 64 || n > m) return -2;
    if (mt <= 0) return -3;
    if (!A && m) return -4;
    if (lda < (m > 1 ? m : 1)) return -5;
    if (!T && n) return -6;
    if (ldt < mt) return -7;
    if (!Q && m) return -8;
    if (ldq < (m > 1 ? m : 1)) return -9;
    if (rows_per_chunk < 0) return -10;
    if (n == 0) return 0;
    if (!work || lwork < lila_gpu_query_dgeqrf_tall_host(m, n, rows_per_chunk)) return -12;
    return ooc_leaf(m, n, mt, A, lda, T, ldt, Q, ldq, rows_per_chunk, work, lwork);
}

int lila_gpu_last_variant(void) { return g_last_variant; }
int lila_gpu_last_passes(void) { return g_last_passes; }

}  // extern "C"
