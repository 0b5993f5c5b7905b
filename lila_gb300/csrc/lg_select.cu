// lg_select.cu -- the learned variant selector: a 5 -> 64 -> 64 -> 64 -> 3
// FP32 multilayer perceptron (ReLU hidden layers, softmax output) with
// hand-written inference, gradient and Adam kernels.
//
// Parameters are one flat FP32 array of LILA_SEL_PARAMS floats:
//   W1 64x5 | b1 64 | W2 64x64 | b2 64 | W3 64x64 | b3 64 | W4 3x64 | b4 3
// (W row-major: W[j * in + i] maps input i to output j).  The loss of a batch
// is the class-weighted mean cross entropy
//   L = (1/N) sum_s cw[y_s] (-log softmax(z_s)[y_s]).
// The gradient kernel processes 64 samples per CTA and writes one partial
// gradient per CTA; a second kernel sums the partials in a fixed order, so
// gradients are deterministic.
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <random>
#include <vector>

#include "lg_common.cuh"
#include "../../include/lila_gpu.h"

namespace lg {
namespace sel {

constexpr int NIN = 5, H = 64, NOUT = 3, SB = 64, NT = 256;
constexpr int OW1 = 0, OB1 = OW1 + H * NIN, OW2 = OB1 + H, OB2 = OW2 + H * H, OW3 = OB2 + H, OB3 = OW3 + H * H,
              OW4 = OB3 + H, OB4 = OW4 + NOUT * H, NPAR = OB4 + NOUT;
static_assert(NPAR == LILA_SEL_PARAMS, "parameter count");

// smem (floats): params NPAR | X SB*NIN | H1 | H2 | H3 (SB*H each) | Z SB*NOUT | D1 | D2 (SB*H)
constexpr int S_X = (NPAR + 3) / 4 * 4, S_H1 = S_X + SB * NIN, S_H2 = S_H1 + SB * H, S_H3 = S_H2 + SB * H,
              S_Z = S_H3 + SB * H, S_D1 = S_Z + SB * NOUT, S_D2 = S_D1 + SB * H, S_END = S_D2 + SB * H;

// out[s][j] = relu(b[j] + sum_i W[j][i] in[s][i]) for the ns valid samples
__device__ __forceinline__ void dense_relu(const float *W, const float *b, const float *in, int nin, float *out, int ns)
{
    for (int idx = threadIdx.x; idx < SB * H; idx += NT) {
        const int s = idx / H, j = idx % H;
        float v = 0.0f;
        if (s < ns) {
            v = b[j];
            for (int i = 0; i < nin; i++) v = fmaf(W[j * nin + i], in[s * nin + i], v);
            v = fmaxf(v, 0.0f);
        }
        out[idx] = v;
    }
    __syncthreads();
}

// forward of the samples [s0, s0 + ns) into shared memory
__device__ void forward(const float *P, const float *F, const int *idx, int s0, int ns, float *sm)
{
    float *X = sm + S_X, *H1 = sm + S_H1, *H2 = sm + S_H2, *H3 = sm + S_H3, *Z = sm + S_Z;
    for (int k = threadIdx.x; k < SB * NIN; k += NT) {
        const int s = k / NIN, i = k % NIN;
        float v = 0.0f;
        if (s < ns) {
            const int g = idx ? idx[s0 + s] : s0 + s;
            v = F[(size_t)g * NIN + i];
        }
        X[k] = v;
    }
    __syncthreads();
    dense_relu(P + OW1, P + OB1, X, NIN, H1, ns);
    dense_relu(P + OW2, P + OB2, H1, H, H2, ns);
    dense_relu(P + OW3, P + OB3, H2, H, H3, ns);
    for (int k = threadIdx.x; k < SB * NOUT; k += NT) {
        const int s = k / NOUT, j = k % NOUT;
        float v = P[OB4 + j];
        for (int i = 0; i < H; i++) v = fmaf(P[OW4 + j * H + i], H3[s * H + i], v);
        Z[k] = v;
    }
    __syncthreads();
}

__device__ void load_params(const float *params, float *sm)
{
    for (int k = threadIdx.x; k < NPAR; k += NT) sm[k] = params[k];
    __syncthreads();
}

__global__ void __launch_bounds__(NT) k_infer(int count, const float *params, const float *F, float *logits,
                                              int *choice)
{
    extern __shared__ float sm[];
    load_params(params, sm);
    for (int s0 = blockIdx.x * SB; s0 < count; s0 += gridDim.x * SB) {
        const int ns = min(SB, count - s0);
        forward(sm, F, nullptr, s0, ns, sm);
        const float *Z = sm + S_Z;
        for (int s = threadIdx.x; s < ns; s += NT) {
            const float *z = Z + s * NOUT;
            int best = 0;
            for (int j = 1; j < NOUT; j++)
                if (z[j] > z[best]) best = j;
            if (choice) choice[s0 + s] = best;
            if (logits)
                for (int j = 0; j < NOUT; j++) logits[(size_t)(s0 + s) * NOUT + j] = z[j];
        }
        __syncthreads();
    }
}

// dW[j][i] = sum_s D[s][j] A[s][i], db[j] = sum_s D[s][j] (written to g)
__device__ __forceinline__ void outer_acc(const float *D, int nout, const float *A, int nin, float *gW, float *gb)
{
    for (int k = threadIdx.x; k < nout * nin; k += NT) {
        const int j = k / nin, i = k % nin;
        float v = 0.0f;
        for (int s = 0; s < SB; s++) v = fmaf(D[s * nout + j], A[s * nin + i], v);
        gW[k] = v;
    }
    for (int j = threadIdx.x; j < nout; j += NT) {
        float v = 0.0f;
        for (int s = 0; s < SB; s++) v += D[s * nout + j];
        gb[j] = v;
    }
}

// Din[s][i] = (sum_j W[j][i] D[s][j]) * (A[s][i] > 0)
__device__ __forceinline__ void back_relu(const float *W, const float *D, int nout, const float *A, float *Din)
{
    for (int k = threadIdx.x; k < SB * H; k += NT) {
        const int s = k / H, i = k % H;
        float v = 0.0f;
        for (int j = 0; j < nout; j++) v = fmaf(W[j * H + i], D[s * nout + j], v);
        Din[k] = A[k] > 0.0f ? v : 0.0f;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(NT) k_grad(int count, const float *params, const float *F, const int *label,
                                             const int *idx, const float *cw, float *partial, float *loss_part)
{
    extern __shared__ float sm[];
    __shared__ float lred[NT];
    load_params(params, sm);
    const int s0 = blockIdx.x * SB;
    const int ns = min(SB, count - s0);
    forward(sm, F, idx, s0, ns, sm);
    float *X = sm + S_X, *H1 = sm + S_H1, *H2 = sm + S_H2, *H3 = sm + S_H3, *Z = sm + S_Z;
    float *D1 = sm + S_D1, *D2 = sm + S_D2;
    // dZ = cw[y] (softmax(z) - onehot(y)) / count, in place of Z
    float lpart = 0.0f;
    if (threadIdx.x < SB) {
        const int s = threadIdx.x;
        float *z = Z + s * NOUT;
        if (s < ns) {
            const int g = idx ? idx[s0 + s] : s0 + s;
            const int y = label[g];
            float mx = z[0];
            for (int j = 1; j < NOUT; j++) mx = fmaxf(mx, z[j]);
            float e[NOUT], se = 0.0f;
            for (int j = 0; j < NOUT; j++) {
                e[j] = expf(z[j] - mx);
                se += e[j];
            }
            const float w = cw[y] / (float)count;
            lpart = cw[y] * (logf(se) - (z[y] - mx));
            for (int j = 0; j < NOUT; j++) z[j] = w * (e[j] / se - (j == y ? 1.0f : 0.0f));
        } else {
            for (int j = 0; j < NOUT; j++) z[j] = 0.0f;
        }
    }
    lred[threadIdx.x] = lpart;
    __syncthreads();
    for (int o = NT / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) lred[threadIdx.x] += lred[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) loss_part[blockIdx.x] = lred[0] / (float)count;
    float *g = partial + (size_t)blockIdx.x * NPAR;
    outer_acc(Z, NOUT, H3, H, g + OW4, g + OB4);
    back_relu(sm + OW4, Z, NOUT, H3, D1);  // D3 in D1
    outer_acc(D1, H, H2, H, g + OW3, g + OB3);
    back_relu(sm + OW3, D1, H, H2, D2);  // D2
    outer_acc(D2, H, H1, H, g + OW2, g + OB2);
    back_relu(sm + OW2, D2, H, H1, D1);  // D1
    outer_acc(D1, H, X, NIN, g + OW1, g + OB1);
}

__global__ void k_reduce(int nparts, const float *partial, const float *loss_part, float *grad, float *loss)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < NPAR) {
        float v = 0.0f;
        for (int p = 0; p < nparts; p++) v += partial[(size_t)p * NPAR + k];
        grad[k] = v;
    }
    if (k == 0 && loss) {
        float v = 0.0f;
        for (int p = 0; p < nparts; p++) v += loss_part[p];
        *loss = v;
    }
}

__global__ void k_adam(const float *grad, float *params, float *m1, float *m2, float lr, float b1, float b2,
                       float c1, float c2, float eps)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= NPAR) return;
    const float gk = grad[k];
    const float a = b1 * m1[k] + (1.0f - b1) * gk;
    const float b = b2 * m2[k] + (1.0f - b2) * gk * gk;
    m1[k] = a;
    m2[k] = b;
    params[k] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
}

// He-uniform weights, zero biases, from a counter-based hash of (seed, k).
__global__ void k_init(float *params, uint32_t seed)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= NPAR) return;
    int fan_in = 0;
    if (k < OB1) fan_in = NIN;
    else if (k >= OW2 && k < OB2) fan_in = H;
    else if (k >= OW3 && k < OB3) fan_in = H;
    else if (k >= OW4 && k < OB4) fan_in = H;
    float v = 0.0f;
    if (fan_in) {
        uint32_t x = (uint32_t)k * 0x9E3779B9u ^ (seed * 0x85EBCA6Bu + 0xC2B2AE35u);
        x ^= x >> 16;
        x *= 0x7FEB352Du;
        x ^= x >> 15;
        x *= 0x846CA68Bu;
        x ^= x >> 16;
        const float u = (x >> 8) * (1.0f / 16777216.0f) * 2.0f - 1.0f;
        v = u * sqrtf(6.0f / (float)fan_in);
    }
    params[k] = v;
}

constexpr size_t SMEM = (size_t)S_END * sizeof(float);

}  // namespace sel
}  // namespace lg

using namespace lg;

extern "C" {

int lila_sel_params(void) { return sel::NPAR; }

long long lila_sel_grad_work(int count) { return (long long)((count + sel::SB - 1) / sel::SB) * (sel::NPAR + 1); }

int lila_sel_init(float *params, unsigned seed)
{
    trace_begin();
    sel::k_init<<<(sel::NPAR + 255) / 256, 256, 0, stream()>>>(params, seed);
    note_launch("sel_init");
    return 0;
}

int lila_sel_infer(int count, const float *params, const float *F, float *logits, int *choice)
{
    if (count < 0) return -1;
    if (count == 0) return 0;
    cudaFuncSetAttribute(sel::k_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sel::SMEM);
    int blocks = (count + sel::SB - 1) / sel::SB;
    const int cap = 2 * sm_count();
    if (blocks > cap) blocks = cap;
    trace_begin();
    sel::k_infer<<<blocks, sel::NT, sel::SMEM, stream()>>>(count, params, F, logits, choice);
    note_launch("sel_infer");
    return 0;
}

int lila_sel_grad(int count, const float *params, const float *F, const int *label, const int *idx, const float *cw,
                  float *grad, float *loss, float *work, long long lwork)
{
    if (count <= 0) return -1;
    if (lwork < lila_sel_grad_work(count)) return -10;
    const int parts = (count + sel::SB - 1) / sel::SB;
    float *partial = work, *loss_part = work + (size_t)parts * sel::NPAR;
    cudaFuncSetAttribute(sel::k_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sel::SMEM);
    trace_begin();
    sel::k_grad<<<parts, sel::NT, sel::SMEM, stream()>>>(count, params, F, label, idx, cw, partial, loss_part);
    note_launch("sel_grad");
    trace_begin();
    sel::k_reduce<<<(sel::NPAR + 255) / 256, 256, 0, stream()>>>(parts, partial, loss_part, grad, loss);
    note_launch("sel_reduce");
    return 0;
}

int lila_sel_adam(const float *grad, float *params, float *m1, float *m2, int step, float lr)
{
    if (step < 1) return -5;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
    trace_begin();
    sel::k_adam<<<(sel::NPAR + 255) / 256, 256, 0, stream()>>>(grad, params, m1, m2, lr, b1, b2, c1, c2, 1e-8f);
    note_launch("sel_adam");
    return 0;
}

// Mini-batch Adam over `epochs` passes of the n samples (features F, labels),
// a fresh permutation per epoch from std::mt19937(seed).  Work (device floats):
// lila_sel_train_work(n, batch).  The mean loss of each epoch's last batch
// goes to loss_host[epoch] when loss_host is not NULL.
long long lila_sel_train_work(int n, int batch)
{
    return 3LL * sel::NPAR + 1 + (long long)n + lila_sel_grad_work(batch);
}

int lila_sel_train(int n, const float *F, const int *label, const float *cw, float *params, int epochs, int batch,
                   float lr, unsigned seed, float *work, long long lwork, float *loss_host)
{
    if (n <= 0) return -1;
    if (batch <= 0) return -7;
    if (lwork < lila_sel_train_work(n, batch)) return -11;
    float *grad = work, *m1 = work + sel::NPAR, *m2 = work + 2 * sel::NPAR, *loss = work + 3 * sel::NPAR;
    int *perm = (int *)(loss + 1);
    float *gwork = (float *)(perm + n);
    cudaStream_t st = stream();
    cudaMemsetAsync(m1, 0, sizeof(float) * 2 * sel::NPAR, st);
    std::mt19937 rng(seed);
    std::vector<int> p(n);
    for (int i = 0; i < n; i++) p[i] = i;
    int step = 0;
    for (int e = 0; e < epochs; e++) {
        std::shuffle(p.begin(), p.end(), rng);
        cudaMemcpyAsync(perm, p.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st);
        for (int b0 = 0; b0 < n; b0 += batch) {
            const int nb = n - b0 < batch ? n - b0 : batch;
            lila_sel_grad(nb, params, F, label, perm + b0, cw, grad, loss, gwork, lila_sel_grad_work(batch));
            lila_sel_adam(grad, params, m1, m2, ++step, lr);
        }
        if (loss_host) cudaMemcpyAsync(loss_host + e, loss, sizeof(float), cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);  // p is rewritten by the next shuffle
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -100;
}

}  // extern "C"
