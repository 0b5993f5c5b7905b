// lg_panel.cu -- Householder QR of an m x nb panel (nb <= 64) in one
// cooperative launch: the reflectors of dgeqr3 (lila-c/dgeqr3.c:3-114,
// LAPACK dlarfg conventions) computed column by column with every CTA holding
// a block of rows in shared memory for the whole panel, one grid barrier per
// column.
//
// Before the barrier of column j every CTA publishes, from its rows below
// the pivot (column j as updated by the reflectors before it): its sum of
// squares of column j, its dot products d_c = sum_r x_j(r) A(r, c) with the
// trailing columns c > j, and, from the CTA that owns row j, alpha = A(j, j)
// and the pivot row A(j, c).  After the barrier every CTA adds the partials
// in CTA order (so all CTAs get the same beta, tau bit for bit), forms
// sc = 1 / (alpha - beta), scales its part of the column into v, and
// updates its rows with w_c = v^T A(:, c) = A(j, c) + sc d_c:
// A(r, c) -= v_r tau w_c.  It then publishes the partials of column j + 1.
// The partials live in two alternating slot buffers, so a CTA can write
// column j + 1's while others still read column j's.
// T then follows from V^T V (dlarft recurrence, lg_kernels.cu).
//
// The grid barrier is a monotonic counter: arrival = fence + reduction, wait
// = acquire loads until the count reaches (barrier index + 1) x CTAs (the
// acquire load orders the CTA's later reads, so no fence follows it).
// All CTAs are co-resident (cudaLaunchCooperativeKernel).  Every wait is
// bounded (iteration and clock limits); a wait that gives up sets
// ST_WAIT_TIMEOUT and the CTA returns.
#include <math.h>

#include "lg_common.cuh"

namespace lg {
namespace pnl {

constexpr int NT = 256, MAXNB = 64;

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Returns false (and flags the status) when the wait gave up after `limit`
// clock cycles.
__device__ bool grid_barrier(unsigned *count, unsigned target, int *status, int *s_fail, long long limit)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        // the fence makes this CTA's slot writes (ordered before it by the
        // block barrier) visible before the arrival
        __threadfence();
        asm volatile("red.relaxed.gpu.global.add.u32 [%0], 1;\n" ::"l"(count) : "memory");
        const long long t0 = clock64();
        bool ok = false;
        for (unsigned it = 0; it < (1u << 26); ++it) {
            if (ld_acquire(count) >= target) {
                ok = true;
                break;
            }
            if (clock64() - t0 > limit) break;
        }
        if (!ok) {
            atomicOr(status, ST_WAIT_TIMEOUT);
            *s_fail = 1;
        }
    }
    __syncthreads();
    return *s_fail == 0;
}

__device__ double block_sum(double v, double *red)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < NT / 32; w++) s += red[w];
    __syncthreads();
    return s;  // valid in thread 0
}

// One slot buffer (doubles) for up to gmax CTAs: [0, G) the sums of squares,
// G + owner the pivot, (2 + c) G + q CTA q's dot product with column c, and
// (MAXNB + 2) gmax + c the pivot row.
__host__ __device__ inline long long slot_buffer(int gmax) { return (long long)(MAXNB + 2) * gmax + MAXNB; }

__global__ void __launch_bounds__(NT, 1)
    k_panel(int m, int nb, int rpb, double *A, int lda, double *tau, double *slots, long long bstride,
            unsigned *count, int *status, long long limit, int extra)
{
    extern __shared__ double X[];  // nb columns x nr rows, ld nr
    __shared__ double red[NT / 32];
    __shared__ double s_beta, s_tau, s_scal;
    __shared__ int s_fail;
    const int G = gridDim.x, b = blockIdx.x;
    const int r0 = b * rpb, r1 = min(m, r0 + rpb), nr = max(0, r1 - r0);
    const long long prow = bstride - MAXNB;  // offset of the pivot row in a buffer
    if (threadIdx.x == 0) s_fail = 0;
    for (int idx = threadIdx.x; idx < nr * nb; idx += NT) {
        const int r = idx % nr, c = idx / nr;
        X[idx] = A[(size_t)(r0 + r) + (size_t)c * lda];
    }
    __syncthreads();
    unsigned target = 0;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // this CTA's partials of column j (as updated so far) into buffer j & 1
    auto publish = [&](int j) {
        double *buf = slots + (size_t)(j & 1) * bstride;
        const int owner = j / rpb;
        const double *xj = X + (size_t)j * nr;
        double p = 0.0;
        for (int r = threadIdx.x; r < nr; r += NT)
            if (r0 + r > j) p += xj[r] * xj[r];
        p = block_sum(p, red);
        if (threadIdx.x == 0) {
            buf[b] = p;
            if (b == owner) buf[(size_t)G + owner] = xj[j - r0];
        }
        for (int c = j + 1 + warp; c < nb; c += NT / 32) {
            const double *xc = X + (size_t)c * nr;
            double s = 0.0;
            for (int r = lane; r < nr; r += 32)
                if (r0 + r > j) s += xj[r] * xc[r];
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) {
                buf[(size_t)(2 + c) * G + b] = s;
                if (b == owner) buf[prow + c] = xc[j - r0];
            }
        }
    };
    publish(0);
    target += G + extra;
    if (!grid_barrier(count, target, status, &s_fail, limit)) return;
    for (int j = 0; j < nb; j++) {
        const int owner = j / rpb;
        double *xj = X + (size_t)j * nr;
        const double *buf = slots + (size_t)(j & 1) * bstride;
        // the reflector (identical in every CTA: the same loads reduced in the
        // same tree)
        double ss = 0.0;
        for (int q = threadIdx.x; q < G; q += NT) ss += __ldcg(&buf[q]);
        ss = block_sum(ss, red);
        if (threadIdx.x == 0) {
            const double alpha = __ldcg(&buf[(size_t)G + owner]);
            const double xn = sqrt(ss);
            if (xn == 0.0) {
                s_tau = 0.0;
                s_beta = alpha;
                s_scal = 0.0;
            } else {
                const double beta = -copysign(sqrt(alpha * alpha + ss), alpha);
                s_tau = (beta - alpha) / beta;
                s_scal = 1.0 / (alpha - beta);
                s_beta = beta;
            }
            if (b == owner) tau[j] = s_tau;
        }
        __syncthreads();
        const double tj = s_tau, sc = s_scal;
        for (int r = threadIdx.x; r < nr; r += NT)
            if (r0 + r > j) xj[r] *= sc;
        if (b == owner && threadIdx.x == 0) xj[j - r0] = s_beta;
        __syncthreads();
        // the trailing columns of this CTA's rows, w_c = A(j, c) + sc d_c
        // (v_r = xj[r] for r0 + r > j, 1 at the pivot row, 0 above)
        if (tj != 0.0) {
            for (int c = j + 1 + warp; c < nb; c += NT / 32) {
                double d = 0.0;
                for (int q = lane; q < G; q += 32) d += __ldcg(&buf[(size_t)(2 + c) * G + q]);
                for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
                const double w = tj * fma(sc, d, __ldcg(&buf[prow + c]));
                double *xc = X + (size_t)c * nr;
                for (int r = lane; r < nr; r += 32) {
                    const int gr = r0 + r;
                    if (gr > j)
                        xc[r] -= xj[r] * w;
                    else if (gr == j)
                        xc[r] -= w;
                }
            }
        }
        __syncthreads();
        if (j + 1 < nb) {
            publish(j + 1);
            target += G + extra;
            if (!grid_barrier(count, target, status, &s_fail, limit)) return;
        }
    }
    for (int idx = threadIdx.x; idx < nr * nb; idx += NT) {
        const int r = idx % nr, c = idx / nr;
        A[(size_t)(r0 + r) + (size_t)c * lda] = X[idx];
    }
}

}  // namespace pnl

// Doubles of workspace panel_coop needs for an nb-column panel: tau, the
// Gram V^T V, the per-CTA reduction slots, the barrier counter and split-K
// room for the Gram.
long long panel_coop_work(int nb)
{
    return (long long)nb + (long long)nb * nb + 2 * pnl::slot_buffer(sm_count()) + 8 + 64LL * nb * nb;
}

// Whether the cooperative panel applies to an m x nb panel.
bool panel_coop_fits(int m, int nb)
{
    if (nb < 2 || nb > pnl::MAXNB || m < 2 * nb || m < 256) return false;
    const int G = sm_count();
    const int rpb = (m + G - 1) / G;
    return (size_t)rpb * nb * sizeof(double) <= 200 * 1024;
}

// V (unit lower, below the diagonal), R (on and above) in A and the nb x nb T
// of the panel's compact-WY form (forward, columnwise), as dgeqr3 gives them.
// Returns false when the cooperative launch was refused (nothing enqueued).
// extra: arrivals each grid barrier waits for beyond the CTAs' own (0; a
// test passes 1 so that every wait runs out, see lila_prim_panel_phantom).
static bool panel_coop_launch(int m, int nb, double *A, int lda, double *T, int ldt, double *work, int extra)
{
    if (!panel_coop_fits(m, nb)) return false;
    const int Gmax = sm_count();
    int G = (m + 15) / 16;
    if (G > Gmax) G = Gmax;
    const int rpb = (m + G - 1) / G;
    G = (m + rpb - 1) / rpb;
    double *tau = work;
    double *Gram = tau + nb;
    double *slots = Gram + (size_t)nb * nb;
    const long long bstride = pnl::slot_buffer(Gmax);
    unsigned *count = (unsigned *)(slots + 2 * bstride);
    double *part = slots + 2 * bstride + 8;
    const size_t smem = (size_t)rpb * nb * sizeof(double);
    cudaStream_t st = stream();
    cudaFuncSetAttribute(pnl::k_panel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaMemsetAsync(count, 0, sizeof(unsigned), st);
    int *status = status_ptr();
    long long limit = wait_limit();
    void *args[] = {(void *)&m,     (void *)&nb,      (void *)&rpb,    (void *)&A,      (void *)&lda,
                    (void *)&tau,   (void *)&slots,   (void *)&bstride, (void *)&count, (void *)&status,
                    (void *)&limit, (void *)&extra};
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pnl::k_panel, pnl::NT, smem) != cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        return false;
    }
    trace_begin();
    if (cudaLaunchCooperativeKernel((const void *)pnl::k_panel, dim3(G), dim3(pnl::NT), args, smem, st) != cudaSuccess) {
        cudaGetLastError();  // refused (e.g. not all CTAs can be resident): nothing ran
        trace_cancel();
        return false;
    }
    note_launch("panel_coop");
    // T from V^T V (only the strictly upper part of the Gram is used)
    GemmEpi e;
    gemm(nb, nb, m, opnd(A, lda, TR, M_UNIT_LOWER), opnd(A, lda, NT, M_UNIT_LOWER), Gram, nb, e, part,
         64LL * nb * nb, "panel_gram");
    larft_from_gram(nb, Gram, nb, tau, T, ldt);
    return true;
}

bool panel_coop(int m, int nb, double *A, int lda, double *T, int ldt, double *work)
{
    return panel_coop_launch(m, nb, A, lda, T, ldt, work, 0);
}

}  // namespace lg

extern "C" {
// Failure-path test of the grid-barrier wait: the panel of an m x nb matrix
// with every barrier waiting for `extra` arrivals that never come, so each
// CTA's wait runs out after the lila_gpu_set_wait_limit cycles, sets
// LILA_ST_WAIT_TIMEOUT and returns (A and T are then meaningless).  1 when
// the cooperative launch ran, 0 when the panel does not apply.
int lila_prim_panel_phantom(int m, int nb, double *A, int lda, double *T, int ldt, double *work, int extra)
{
    if (extra < 0) return -8;
    return lg::panel_coop_launch(m, nb, A, lda, T, ldt, work, extra) ? 1 : 0;
}
long long lila_prim_panel_work(int nb) { return lg::panel_coop_work(nb); }
}
