// lg_batched.cu -- thousands of independent least-squares problems
// min ||A_t x - b_t|| (A_t m_t x n_t, m_t >= n_t, nrhs right-hand sides) in
// one persistent launch.
//
// Per instance the algorithm is the reference's least-squares driver
// (least-squares/main_ls_qr3.c:94-119): Householder QR of A, Q^T applied to
// the right-hand sides, R x = (Q^T b)(0:n).  Here each reflector is applied to
// the right-hand sides as soon as it is formed, so no T factor is needed, and
// x overwrites B(0:n, :) (LAPACK dgels convention); A holds V and R on exit.
// CTAs take instances from a device counter (largest first, order prepared on
// the host), so uneven sizes balance without any inter-CTA waiting.
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "lg_common.cuh"
#include "../../include/lila_gpu.h"

namespace lg {
namespace bat {

struct Inst {
    int m, n, lda, ldb;
};

constexpr int CW = 8;  // columns updated per pass

template <int TH>
__device__ double bsum(double v, double *red)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
        v = l < TH / 32 ? red[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (l == 0) red[32] = v;
    }
    __syncthreads();
    return red[32];
}

template <int TH>
__device__ double bmax(double v, double *red)
{
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
        v = l < TH / 32 ? red[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (l == 0) red[32] = v;
    }
    __syncthreads();
    return red[32];
}

// column c of the combined [A | B] operand of an instance
__device__ __forceinline__ double *colp(double *A, int lda, double *B, int ldb, int n, int c)
{
    return c < n ? A + (size_t)c * lda : B + (size_t)(c - n) * ldb;
}

constexpr int NB = 8;   // panel width of the blocked factorization
constexpr int UW = 4;   // trailing columns per block-reflector pass

// Blocked Householder least squares per instance: panels of NB columns are
// factored column by column (each reflector applied to the rest of its
// panel), then the panel's block reflector I - V T V^T (T by the dlarft
// recurrence from V^T V) is applied to the trailing columns of A and to B,
// UW columns per pass: W = V^T C, W = T^T W, C -= V W.  The trailing matrix
// is read and written once per panel instead of once per column.
template <int TH>
__global__ void __launch_bounds__(TH)
    k_gels(int count, int nrhs, const Inst *inst, double *const *Aptr, double *const *Bptr, const int *order,
           int *counter, int *info)
{
    __shared__ double red[33 * CW];
    __shared__ double s_w[CW];
    __shared__ double s_tau, s_scale, s_beta;
    __shared__ double s_taus[NB], s_G[NB * NB], s_T[NB * NB], s_W[NB * UW];
    __shared__ double s_red[TH / 32][NB * (NB - 1) / 2 > NB * UW ? NB * (NB - 1) / 2 : NB * UW];
    __shared__ int s_idx;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (;;) {
        if (threadIdx.x == 0) s_idx = atomicAdd(counter, 1);
        __syncthreads();
        const int idx = s_idx;
        __syncthreads();
        if (idx >= count) break;
        const int t = order[idx];
        const Inst I = inst[t];
        double *A = Aptr[t], *B = Bptr[t];
        const int m = I.m, n = I.n;
        const int ncol = n + nrhs;
        int bad = 0;
        for (int j0 = 0; j0 < n; j0 += NB) {
            const int jb = min(NB, n - j0);
            // ---- panel: reflectors j0 .. j0 + jb - 1 on the panel's own columns
            for (int k = j0; k < j0 + jb; k++) {
                double *ck = A + (size_t)k * I.lda;
                // Householder vector of A(k:m, k) (LAPACK dlarfg convention)
                double mx = 0.0;
                for (int r = k + 1 + threadIdx.x; r < m; r += TH) mx = fmax(mx, fabs(ck[r]));
                const double scale = bmax<TH>(mx, red);
                double part = 0.0;
                if (scale > 0.0)
                    for (int r = k + 1 + threadIdx.x; r < m; r += TH) {
                        const double q = ck[r] / scale;
                        part += q * q;
                    }
                const double ssq = bsum<TH>(part, red);
                if (threadIdx.x == 0) {
                    const double alpha = ck[k];
                    if (scale == 0.0) {
                        s_tau = 0.0;
                        s_beta = alpha;
                    } else {
                        const double beta = -copysign(hypot(alpha, scale * sqrt(ssq)), alpha);
                        s_tau = (beta - alpha) / beta;
                        s_scale = 1.0 / (alpha - beta);
                        s_beta = beta;
                    }
                    s_taus[k - j0] = s_tau;
                }
                __syncthreads();
                const double tk = s_tau;
                if (tk != 0.0)
                    for (int r = k + 1 + threadIdx.x; r < m; r += TH) ck[r] *= s_scale;
                __syncthreads();
                if (threadIdx.x == 0) ck[k] = s_beta;
                const int pend = j0 + jb;  // panel columns k + 1 .. pend - 1
                if (tk == 0.0 || k + 1 >= pend) {
                    __syncthreads();
                    continue;
                }
                const int nc = pend - (k + 1);  // <= NB - 1 <= CW
                double acc[CW];
#pragma unroll
                for (int j = 0; j < CW; j++) acc[j] = 0.0;
                for (int r = k + 1 + threadIdx.x; r < m; r += TH) {
                    const double v = ck[r];
#pragma unroll
                    for (int j = 0; j < CW; j++)
                        if (j < nc) acc[j] += v * A[(size_t)r + (size_t)(k + 1 + j) * I.lda];
                }
#pragma unroll
                for (int j = 0; j < CW; j++)
                    for (int o = 16; o > 0; o >>= 1) acc[j] += __shfl_xor_sync(0xffffffffu, acc[j], o);
                if (lane == 0)
#pragma unroll
                    for (int j = 0; j < CW; j++) red[j * 33 + warp] = acc[j];
                __syncthreads();
                if (threadIdx.x < nc) {
                    double sw = 0.0;
                    for (int q = 0; q < TH / 32; q++) sw += red[threadIdx.x * 33 + q];
                    sw += A[(size_t)k + (size_t)(k + 1 + threadIdx.x) * I.lda];  // v_k = 1
                    s_w[threadIdx.x] = tk * sw;
                }
                __syncthreads();
                for (int r = k + threadIdx.x; r < m; r += TH) {
                    const double v = r == k ? 1.0 : ck[r];
#pragma unroll
                    for (int j = 0; j < CW; j++)
                        if (j < nc) A[(size_t)r + (size_t)(k + 1 + j) * I.lda] -= s_w[j] * v;
                }
                __syncthreads();
            }
            if (j0 + jb >= ncol) continue;
            // ---- T of the panel from G = V^T V (strictly upper part)
            // v_i(r) = A(r, j0 + i) below the diagonal, 1 on it, 0 above
            {
                double g[NB * (NB - 1) / 2];
#pragma unroll
                for (int q = 0; q < NB * (NB - 1) / 2; q++) g[q] = 0.0;
                for (int r = j0 + 1 + threadIdx.x; r < m; r += TH) {
                    double v[NB];
#pragma unroll
                    for (int i = 0; i < NB; i++) {
                        const int d = j0 + i;
                        v[i] = (i < jb) ? (r > d ? A[(size_t)r + (size_t)d * I.lda] : (r == d ? 1.0 : 0.0)) : 0.0;
                    }
                    int q = 0;
#pragma unroll
                    for (int a2 = 0; a2 < NB; a2++)
#pragma unroll
                        for (int b2 = a2 + 1; b2 < NB; b2++) g[q++] += v[a2] * v[b2];
                }
#pragma unroll
                for (int q = 0; q < NB * (NB - 1) / 2; q++) {
                    double x = g[q];
                    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
                    if (lane == 0) s_red[warp][q] = x;
                }
                __syncthreads();
                if (threadIdx.x < NB * (NB - 1) / 2) {
                    double x = 0.0;
                    for (int w = 0; w < TH / 32; w++) x += s_red[w][threadIdx.x];
                    // pair index -> (a2, b2)
                    int q = threadIdx.x, a2 = 0;
                    while (q >= NB - 1 - a2) {
                        q -= NB - 1 - a2;
                        a2++;
                    }
                    s_G[a2 + NB * (a2 + 1 + q)] = x;
                }
                __syncthreads();
                if (threadIdx.x == 0) {
                    for (int i = 0; i < jb; i++) {
                        const double ti = s_taus[i];
                        for (int r = 0; r < i; r++) {
                            double x = 0.0;
                            for (int p2 = r; p2 < i; p2++) x += s_T[r + NB * p2] * s_G[p2 + NB * i];
                            s_T[r + NB * i] = -ti * x;
                        }
                        s_T[i + NB * i] = ti;
                    }
                }
                __syncthreads();
            }
            // ---- block reflector on the trailing columns of A and on B
            for (int c0 = j0 + jb; c0 < ncol; c0 += UW) {
                const int nc = min(UW, ncol - c0);
                double w[NB][UW];
#pragma unroll
                for (int i = 0; i < NB; i++)
#pragma unroll
                    for (int j = 0; j < UW; j++) w[i][j] = 0.0;
                for (int r = j0 + threadIdx.x; r < m; r += TH) {
                    double v[NB];
#pragma unroll
                    for (int i = 0; i < NB; i++) {
                        const int d = j0 + i;
                        v[i] = (i < jb) ? (r > d ? A[(size_t)r + (size_t)d * I.lda] : (r == d ? 1.0 : 0.0)) : 0.0;
                    }
#pragma unroll
                    for (int j = 0; j < UW; j++)
                        if (j < nc) {
                            const double cv = colp(A, I.lda, B, I.ldb, n, c0 + j)[r];
#pragma unroll
                            for (int i = 0; i < NB; i++) w[i][j] += v[i] * cv;
                        }
                }
#pragma unroll
                for (int i = 0; i < NB; i++)
#pragma unroll
                    for (int j = 0; j < UW; j++) {
                        double x = w[i][j];
                        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
                        if (lane == 0) s_red[warp][i * UW + j] = x;
                    }
                __syncthreads();
                if (threadIdx.x < NB * UW) {
                    double x = 0.0;
                    for (int q = 0; q < TH / 32; q++) x += s_red[q][threadIdx.x];
                    red[threadIdx.x] = x;  // W(i, j), i = idx / UW
                }
                __syncthreads();
                if (threadIdx.x < NB * UW) {  // W := T^T W
                    const int i = threadIdx.x / UW, j = threadIdx.x % UW;
                    double x = 0.0;
                    for (int p2 = 0; p2 <= i && p2 < jb; p2++) x += s_T[p2 + NB * i] * red[p2 * UW + j];
                    s_W[i * UW + j] = (i < jb) ? x : 0.0;
                }
                __syncthreads();
                for (int r = j0 + threadIdx.x; r < m; r += TH) {
                    double v[NB];
#pragma unroll
                    for (int i = 0; i < NB; i++) {
                        const int d = j0 + i;
                        v[i] = (i < jb) ? (r > d ? A[(size_t)r + (size_t)d * I.lda] : (r == d ? 1.0 : 0.0)) : 0.0;
                    }
#pragma unroll
                    for (int j = 0; j < UW; j++)
                        if (j < nc) {
                            double x = 0.0;
#pragma unroll
                            for (int i = 0; i < NB; i++) x += v[i] * s_W[i * UW + j];
                            colp(A, I.lda, B, I.ldb, n, c0 + j)[r] -= x;
                        }
                }
                __syncthreads();
            }
        }
        // back substitution R x = y, x over B(0:n, :)
        for (int k = n - 1; k >= 0; k--) {
            const double d = A[(size_t)k + (size_t)k * I.lda];
            if (threadIdx.x < nrhs) {
                double *bk = B + (size_t)threadIdx.x * I.ldb;
                if (d == 0.0 || !isfinite(d)) {
                    bad = k + 1;
                    bk[k] = NAN;
                } else {
                    bk[k] /= d;
                }
            }
            __syncthreads();
            for (int idx2 = threadIdx.x; idx2 < k * nrhs; idx2 += TH) {
                const int r = idx2 % k, j = idx2 / k;
                double *bj = B + (size_t)j * I.ldb;
                bj[r] -= A[(size_t)r + (size_t)k * I.lda] * bj[k];
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) info[t] = bad;
        __syncthreads();
    }
}

}  // namespace bat

struct BatchMeta {
    int count, nrhs;
    bat::Inst *inst;
    double **Aptr, **Bptr;
    int *order, *counter;
};

static long long batch_bytes(int count)
{
    return 256 + (long long)count * ((long long)sizeof(bat::Inst) + 2 * sizeof(double *) + sizeof(int)) + 256;
}

static BatchMeta carve_meta(void *work, int count)
{
    BatchMeta b;
    uint8_t *p = (uint8_t *)work;
    b.counter = (int *)p;
    p += 256;
    b.inst = (bat::Inst *)p;
    p += (size_t)count * sizeof(bat::Inst);
    b.Aptr = (double **)p;
    p += (size_t)count * sizeof(double *);
    b.Bptr = (double **)p;
    p += (size_t)count * sizeof(double *);
    b.order = (int *)p;
    b.count = count;
    b.nrhs = 0;
    return b;
}

// launch configuration (threads, CTAs per SM), chosen by lila_gpu_gels_autotune
static int g_gels_threads = 256, g_gels_per_sm = 2;

static void launch_gels(const BatchMeta &b, int nrhs, int *info)
{
    cudaStream_t st = stream();
    cudaMemsetAsync(b.counter, 0, sizeof(int), st);
    const int grid = sm_count() * g_gels_per_sm;
    trace_begin();
    if (g_gels_threads == 128)
        bat::k_gels<128><<<grid, 128, 0, st>>>(b.count, nrhs, b.inst, b.Aptr, b.Bptr, b.order, b.counter, info);
    else if (g_gels_threads == 512)
        bat::k_gels<512><<<grid, 512, 0, st>>>(b.count, nrhs, b.inst, b.Aptr, b.Bptr, b.order, b.counter, info);
    else
        bat::k_gels<256><<<grid, 256, 0, st>>>(b.count, nrhs, b.inst, b.Aptr, b.Bptr, b.order, b.counter, info);
    note_launch("gels_batched");
}

}  // namespace lg

using namespace lg;

extern "C" {

long long lila_query_dgels_batched(int count) { return batch_bytes(count); }

int lila_dgels_batched_prepare(int count, const int *m, const int *n, int nrhs, double *const *A, const int *lda,
                               double *const *B, const int *ldb, void *work, long long work_bytes)
{
    if (count < 0) return -1;
    if (nrhs < 1 || nrhs > 8) return -4;
    if (work_bytes < batch_bytes(count)) return -10;
    std::vector<bat::Inst> inst(count);
    std::vector<int> order(count);
    for (int t = 0; t < count; t++) {
        if (m[t] < n[t] || n[t] < 1) return -2;
        if (lda[t] < m[t] || ldb[t] < m[t]) return -6;
        inst[t] = bat::Inst{m[t], n[t], lda[t], ldb[t]};
        order[t] = t;
    }
    // largest work first: m n^2
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return (double)inst[a].m * inst[a].n * inst[a].n > (double)inst[b].m * inst[b].n * inst[b].n;
    });
    BatchMeta b = carve_meta(work, count);
    cudaStream_t st = stream();
    cudaMemcpyAsync(b.inst, inst.data(), sizeof(bat::Inst) * count, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(b.Aptr, A, sizeof(double *) * count, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(b.Bptr, B, sizeof(double *) * count, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(b.order, order.data(), sizeof(int) * count, cudaMemcpyHostToDevice, st);
    cudaStreamSynchronize(st);  // host vectors go out of scope
    return 0;
}

// One persistent launch over every prepared instance (stream-capturable).
int lila_dgels_batched_run(int count, int nrhs, void *work, int *info)
{
    if (count <= 0) return 0;
    BatchMeta b = carve_meta(work, count);
    launch_gels(b, nrhs, info);
    return 0;
}

// Captures lila_dgels_batched_run into a CUDA graph (on a private stream) and
// returns its executable handle; lila_gpu_graph_launch replays it on the
// library stream.
void *lila_dgels_batched_graph(int count, int nrhs, void *work, int *info)
{
    cudaStream_t cap;
    if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
    void *prev = lila_gpu_get_stream();
    lila_gpu_set_stream(cap);
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        lila_dgels_batched_run(count, nrhs, work, info);
        if (cudaStreamEndCapture(cap, &g) == cudaSuccess && g) {
            if (cudaGraphInstantiate(&ge, g, 0) != cudaSuccess) ge = nullptr;
            cudaGraphDestroy(g);
        }
    }
    lila_gpu_set_stream(prev);
    cudaStreamDestroy(cap);
    return (void *)ge;
}

int lila_gpu_graph_launch(void *exec)
{
    if (!exec) return -1;
    return cudaGraphLaunch((cudaGraphExec_t)exec, lg::stream()) == cudaSuccess ? 0 : -2;
}

int lila_gpu_graph_destroy(void *exec)
{
    if (!exec) return 0;
    return cudaGraphExecDestroy((cudaGraphExec_t)exec) == cudaSuccess ? 0 : -1;
}

// Times (threads, CTAs per SM) candidates on the prepared batch (its A and B
// are overwritten: call on a scratch copy) and keeps the fastest for later
// launches.  Returns threads * 100 + CTAs per SM.
int lila_gpu_gels_autotune(int count, int nrhs, void *work, int *info, double *const *Asave, double *const *A,
                           const long long *bytesA, double *const *Bsave, double *const *B, const long long *bytesB)
{
    const int cand_th[3] = {128, 256, 512};
    const int cand_sm[3] = {1, 2, 4};
    float best = 1e30f;
    int bth = 256, bsm = 2;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int a = 0; a < 3; a++)
        for (int c = 0; c < 3; c++) {
            if (cand_th[a] * cand_sm[c] > 1024) continue;
            for (int t = 0; t < count; t++) {
                cudaMemcpyAsync(A[t], Asave[t], bytesA[t], cudaMemcpyDeviceToDevice, lg::stream());
                cudaMemcpyAsync(B[t], Bsave[t], bytesB[t], cudaMemcpyDeviceToDevice, lg::stream());
            }
            g_gels_threads = cand_th[a];
            g_gels_per_sm = cand_sm[c];
            cudaEventRecord(e0, lg::stream());
            lila_dgels_batched_run(count, nrhs, work, info);
            cudaEventRecord(e1, lg::stream());
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) {
                best = ms;
                bth = cand_th[a];
                bsm = cand_sm[c];
            }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    g_gels_threads = bth;
    g_gels_per_sm = bsm;
    return bth * 100 + bsm;
}

int lila_gpu_gels_config(int threads, int per_sm)
{
    if (threads != 128 && threads != 256 && threads != 512) return -1;
    if (per_sm < 1 || per_sm > 8) return -2;
    g_gels_threads = threads;
    g_gels_per_sm = per_sm;
    return 0;
}

}  // extern "C"
