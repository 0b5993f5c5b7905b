// lg_runtime.cu -- library stream, device status word and launch checking.
#include <mutex>
#include <string>
#include <vector>
#include <string.h>

#include "lg_common.cuh"
#include "../../include/lila_gpu.h"

namespace lg {

static thread_local cudaStream_t t_stream = 0;   // legacy default stream until set
static int h_launch_error = 0;                   // sticky host-side launch failure flag
static std::mutex g_mu;
static unsigned long long h_launches = 0;        // kernels this library has launched

// Optional per-launch CUDA-event tracing (off by default): a pair of events
// on the library stream around each traced launch, filed under its name.
struct TraceRec {
    const char *name;
    cudaEvent_t a, b;
};
static bool g_trace = false;
static std::vector<TraceRec> g_recs;
static cudaEvent_t g_pending = nullptr;

// One status word per device; its device address is looked up once per device
// (with that device current) and cached.
__device__ int d_status_word;
static int *g_status_addr[64];

int *status_ptr()
{
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return nullptr;
    if (!g_status_addr[dev]) {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_status_addr[dev]) {
            void *p = nullptr;
            if (cudaGetSymbolAddress(&p, d_status_word) == cudaSuccess) {
                cudaMemset(p, 0, sizeof(int));
                g_status_addr[dev] = (int *)p;
            }
        }
    }
    return g_status_addr[dev];
}

cudaStream_t stream() { return t_stream; }

void trace_begin()
{
    if (!g_trace) return;
    if (cudaEventCreate(&g_pending) == cudaSuccess) cudaEventRecord(g_pending, t_stream);
}

void note_launch(const char *what)
{
    h_launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        h_launch_error = 1;
        fprintf(stderr, "lila_gb300: launch of %s failed: %s\n", what, cudaGetErrorString(e));
    }
    if (g_trace && g_pending) {
        cudaEvent_t b;
        if (cudaEventCreate(&b) == cudaSuccess) {
            cudaEventRecord(b, t_stream);
            g_recs.push_back(TraceRec{what, g_pending, b});
        }
        g_pending = nullptr;
    }
}

}  // namespace lg

extern "C" {

int lila_gpu_set_stream(void *stream)
{
    lg::t_stream = (cudaStream_t)stream;
    return 0;
}

void *lila_gpu_get_stream(void) { return (void *)lg::t_stream; }

int lila_gpu_sync(void)
{
    cudaError_t e = cudaStreamSynchronize(lg::t_stream);
    return e == cudaSuccess ? 0 : -(int)e;
}

int lila_gpu_status(void)
{
    int v = 0;
    int *p = lg::status_ptr();
    if (p) {
        cudaStreamSynchronize(lg::t_stream);
        cudaMemcpy(&v, p, sizeof(int), cudaMemcpyDeviceToHost);
    }
    if (lg::h_launch_error) v |= lg::ST_LAUNCH_ERROR;
    return v;
}

int lila_gpu_clear_status(void)
{
    int *p = lg::status_ptr();
    lg::h_launch_error = 0;
    if (!p) return -1;
    cudaStreamSynchronize(lg::t_stream);
    return cudaMemset(p, 0, sizeof(int)) == cudaSuccess ? 0 : -1;
}

int lila_gpu_version(void) { return LILA_GPU_VERSION; }

unsigned long long lila_gpu_launch_count(void) { return lg::h_launches; }

static void trace_clear()
{
    for (auto &r : lg::g_recs) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    lg::g_recs.clear();
}

int lila_gpu_trace(int on)
{
    cudaStreamSynchronize(lg::t_stream);
    trace_clear();
    lg::g_trace = on != 0;
    return 0;
}

/* "name launches total_ms" lines, one per traced kernel name; returns the
 * number of bytes written (excluding the terminating NUL). */
int lila_gpu_trace_summary(char *buf, int len)
{
    cudaStreamSynchronize(lg::t_stream);
    std::vector<std::string> names;
    std::vector<double> tot;
    std::vector<int> cnt;
    for (auto &r : lg::g_recs) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, r.a, r.b);
        size_t k = 0;
        for (; k < names.size(); k++)
            if (names[k] == r.name) break;
        if (k == names.size()) {
            names.push_back(r.name);
            tot.push_back(0.0);
            cnt.push_back(0);
        }
        tot[k] += ms;
        cnt[k] += 1;
    }
    std::string out;
    for (size_t k = 0; k < names.size(); k++) {
        char line[256];
        snprintf(line, sizeof line, "%s %d %.6f\n", names[k].c_str(), cnt[k], tot[k]);
        out += line;
    }
    if (buf && len > 0) {
        int n = (int)out.size() < len - 1 ? (int)out.size() : len - 1;
        memcpy(buf, out.data(), n);
        buf[n] = 0;
        return n;
    }
    return (int)out.size();
}

}  // extern "C"
