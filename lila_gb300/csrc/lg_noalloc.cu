// lg_noalloc.cu -- lila_dormqrf_w03 for callers that cannot allocate device memory.
//
// Who needs it: code that applies the block reflectors from inside a fixed,
// pre-reserved device-memory budget -- an application or framework that owns
// the whole GPU memory pool and does not allow cudaMalloc, or the inner loop
// of a block-Krylov solver (new columns are orthogonalised against the ones
// already factored, the appended-columns use case of the w03 interface) that
// must not call cudaMalloc because an allocation can synchronise the device
// and stall the stream.  lila_dormqrf_w03 needs a caller-supplied `work`
// buffer; this variant needs none: its scratch is the file-scope device array
// below, LILA_NOALLOC_SCRATCH_DOUBLES doubles (4 MiB), which every GPU that
// loads this library holds until the process exits.
//
// Limits and rules (also stated in include/lila_gpu.h):
//   * 2 * min(mt, k) * n doubles must fit in the array; larger problems are
//     rejected with LILA_NOALLOC_TOO_LARGE before anything is enqueued.  What
//     is left of the array beyond that feeds the split-K partial products.
//   * All calls share the one array and it keeps the last call's contents.
//     Nothing in it has to start at zero: every scratch word is written by
//     this call before it is read.  Calls that overlap on the GPU (on
//     different streams, or from several host threads without ordering)
//     race on the array and give wrong results.
//   * The device address of the array is looked up once per device, with
//     that device current, by the first call made on that device
//     (cudaGetSymbolAddress); make that first call before any stream
//     capture starts on the device.  Turning the library's graph mode on
//     (lila_gpu_graph_mode) does this lookup for the current device.
//   * No cudaMalloc, cudaFree or allocating library routine is called.
#include <atomic>
#include <mutex>

#include "lg_common.cuh"
#include "../../include/lila_gpu.h"

namespace lg {
void apply_qt_scratch(int m, int n, int k, int i, int mt, const double *A, int lda, const double *T, int ldt,
                      double *C, int ldc, double *scratch, long long scratch_len);
}

static __device__ __align__(256) double g_noalloc_scratch[LILA_NOALLOC_SCRATCH_DOUBLES];

static std::atomic<double *> g_noalloc_addr[64];
static std::mutex g_noalloc_mu;

namespace lg {
// Device address of the scratch array for the current device, looked up once
// per device (first calls from several host threads take the lock in turn).
double *noalloc_scratch_addr()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    double *p = g_noalloc_addr[dev].load(std::memory_order_acquire);
    if (p) return p;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    p = g_noalloc_addr[dev].load(std::memory_order_relaxed);
    if (!p) {
        if (cudaGetSymbolAddress((void **)&p, g_noalloc_scratch) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        g_noalloc_addr[dev].store(p, std::memory_order_release);
    }
    return p;
}
}  // namespace lg

extern "C" int lila_dormqrf_w03_noalloc(int m, int n, int k, int i, int j, int mt, double *A, int lda,
                                        double *T, int ldt)
{
    if (m < 0) return -1;
    if (n < 0) return -2;
    if (k < 0 || i + k > m) return -3;
    if (i < 0) return -4;
    if (j < 0 || (j < i + k && n > 0 && k > 0)) return -5;
    if (mt <= 0) return -6;
    if (lda < (m > 1 ? m : 1)) return -8;
    if (ldt < mt) return -10;
    if (n == 0 || k == 0) return 0;
    const long long vb = mt < k ? mt : k;
    if (2 * vb * (long long)n > LILA_NOALLOC_SCRATCH_DOUBLES) return LILA_NOALLOC_TOO_LARGE;
    double *scratch = lg::noalloc_scratch_addr();
    if (!scratch) return LILA_NOALLOC_NO_DEVICE;
    lg::apply_qt_scratch(m, n, k, i, mt, A, lda, T, ldt, A + (size_t)j * lda, lda, scratch,
                         LILA_NOALLOC_SCRATCH_DOUBLES);
    return 0;
}
