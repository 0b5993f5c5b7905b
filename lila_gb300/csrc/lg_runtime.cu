// lg_runtime.cu -- library stream, device status word and launch checking.
#include <functional>
#include <initializer_list>
#include <mutex>
#include <string>
#include <vector>
#include <string.h>

#include "lg_common.cuh"
#include "../../include/lila_gpu.h"

namespace lg {

// Clock-cycle limit of the cooperative panel's grid-barrier waits
// (lila_gpu_set_wait_limit); ~2 s at 2 GHz by default.
long long g_wait_limit = 4000000000LL;
long long wait_limit() { return g_wait_limit; }

static thread_local cudaStream_t t_stream = 0;   // legacy default stream until set
static int h_launch_error = 0;                   // sticky host-side launch failure flag
static std::mutex g_mu;
static unsigned long long h_launches = 0;        // kernels this library has launched

// Optional per-launch CUDA-event tracing (off by default): a pair of events
// on the library stream around each traced launch, filed under its name.
// The end event of one traced launch is the start event of the next while
// the device has not reached it when the next launch is queued (the next
// kernel then starts as soon as that event completes, so no idle time is
// counted); an event between two kernels costs device time, and sharing it
// halves the events in a traced run.  An untraced launch or other stream
// work (trace_break) in between ends the chain, so that its time is not
// counted in the next traced launch.
struct TraceRec {
    const char *name;
    cudaEvent_t a, b;
    bool own_a;  // a is not the previous record's b
};
static bool g_trace = false;
static std::vector<TraceRec> g_recs;
static cudaEvent_t g_pending = nullptr;
static bool g_pending_shared = false;
static cudaEvent_t g_chain = nullptr;  // end event of the last traced launch
// Events of finished traces, reused (creating an event costs host time
// inside the traced region; turning tracing on fills the pool).
static std::vector<cudaEvent_t> g_event_pool;
static constexpr size_t kEventPool = 4096;

static cudaEvent_t trace_event()
{
    cudaEvent_t e = nullptr;
    if (!g_event_pool.empty()) {
        e = g_event_pool.back();
        g_event_pool.pop_back();
    } else if (cudaEventCreate(&e) != cudaSuccess) {
        cudaGetLastError();
        e = nullptr;
    }
    return e;
}

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

static int g_precision = 0;
int precision() { return g_precision; }

void trace_begin()
{
    if (!g_trace) return;
    if (g_chain) {
        const cudaError_t before = cudaPeekAtLastError();
        const cudaError_t q = cudaEventQuery(g_chain);
        // a not-ready answer is not an error of any launch
        if (q == cudaErrorNotReady && before == cudaSuccess && cudaPeekAtLastError() == cudaErrorNotReady)
            cudaGetLastError();
        if (q == cudaErrorNotReady) {
            g_pending = g_chain;
            g_pending_shared = true;
            return;
        }
    }
    g_pending = trace_event();
    g_pending_shared = false;
    if (g_pending) cudaEventRecord(g_pending, t_stream);
}

void trace_cancel()
{
    if (g_pending) {
        if (!g_pending_shared) g_event_pool.push_back(g_pending);
        g_pending = nullptr;
    }
}

void trace_break() { g_chain = nullptr; }

void note_launch(const char *what)
{
    h_launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        h_launch_error = 1;
        fprintf(stderr, "lila_gb300: launch of %s failed: %s\n", what, cudaGetErrorString(e));
    }
    if (g_trace && !g_pending) g_chain = nullptr;  // an untraced launch: its time is nobody's
    if (g_trace && g_pending) {
        cudaEvent_t b = trace_event();
        if (b) {
            cudaEventRecord(b, t_stream);
            g_recs.push_back(TraceRec{what, g_pending, b, !g_pending_shared});
            g_chain = b;
        } else {
            if (!g_pending_shared) g_event_pool.push_back(g_pending);
            g_chain = nullptr;
        }
        g_pending = nullptr;
    }
}

// ---------------------------------------------------------------------------
// Graph cache.  With graph mode on, a public call whose scalar and pointer
// arguments (and lila_param contents) equal an earlier call's replays the
// CUDA graph captured from that earlier call: the same kernels with the same
// parameters, one cudaGraphLaunch instead of thousands of launches.  A call
// whose body cannot be captured (it synchronises the host to branch on device
// data, or allocates) runs directly and its key is remembered as such.
// ---------------------------------------------------------------------------
struct GraphEntry {
    std::vector<long long> key;
    cudaGraphExec_t exec;
    unsigned long long kernels, last_use;
    bool capturable;
};
static std::mutex g_graph_mu;
static std::vector<GraphEntry> g_graphs;
static int g_graph_mode = 0;
static unsigned long long g_graph_clock = 0, g_graph_replays = 0;
static thread_local bool t_capturing = false;
static thread_local cudaStream_t t_cap_stream = nullptr;
constexpr size_t GRAPH_CACHE_MAX = 64;

static void evict_lru_locked()
{
    size_t worst = 0;
    for (size_t k = 1; k < g_graphs.size(); k++)
        if (g_graphs[k].last_use < g_graphs[worst].last_use) worst = k;
    if (g_graphs[worst].exec) cudaGraphExecDestroy(g_graphs[worst].exec);
    g_graphs.erase(g_graphs.begin() + worst);
}

int graph_call(const char *fn, std::initializer_list<long long> args, const std::function<int()> &body)
{
    if (!g_graph_mode || t_capturing) return body();
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(t_stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        return body();  // the caller is capturing: become part of its graph
    }
    std::vector<long long> key(args);
    int dev = 0;
    cudaGetDevice(&dev);
    key.push_back((long long)(uintptr_t)fn);
    key.push_back(dev);
    {
        std::lock_guard<std::mutex> lk(g_graph_mu);
        for (auto &e : g_graphs)
            if (e.key == key) {
                e.last_use = ++g_graph_clock;
                if (!e.capturable) break;
                if (cudaGraphLaunch(e.exec, t_stream) != cudaSuccess) {
                    h_launch_error = 1;
                    return -100;
                }
                h_launches += e.kernels;
                g_graph_replays++;
                return 0;
            }
    }
    bool known_bad = false;
    {
        std::lock_guard<std::mutex> lk(g_graph_mu);
        for (auto &e : g_graphs)
            if (e.key == key && !e.capturable) known_bad = true;
    }
    if (known_bad) return body();
    if (!t_cap_stream && cudaStreamCreateWithFlags(&t_cap_stream, cudaStreamNonBlocking) != cudaSuccess) return body();
    const cudaStream_t prev = t_stream;
    const unsigned long long l0 = h_launches;
    const int err0 = h_launch_error;
    const bool tr = g_trace;
    g_trace = false;
    t_stream = t_cap_stream;
    t_capturing = true;
    cudaGraph_t g = nullptr;
    int rc = -1;
    bool ok = cudaStreamBeginCapture(t_cap_stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
        rc = body();
        ok = cudaStreamEndCapture(t_cap_stream, &g) == cudaSuccess && g && rc == 0;
    }
    t_capturing = false;
    t_stream = prev;
    g_trace = tr;
    const unsigned long long kernels = h_launches - l0;
    h_launches = l0;
    h_launch_error = err0;
    cudaGetLastError();  // a failed capture leaves an error behind
    cudaGraphExec_t ex = nullptr;
    if (ok && cudaGraphInstantiate(&ex, g, 0) != cudaSuccess) {
        cudaGetLastError();
        ex = nullptr;
        ok = false;
    }
    if (g) cudaGraphDestroy(g);
    {
        std::lock_guard<std::mutex> lk(g_graph_mu);
        if (g_graphs.size() >= GRAPH_CACHE_MAX) evict_lru_locked();
        g_graphs.push_back(GraphEntry{key, ex, kernels, ++g_graph_clock, ok});
    }
    if (!ok) return body();  // run it for real, uncaptured
    if (cudaGraphLaunch(ex, t_stream) != cudaSuccess) {
        h_launch_error = 1;
        return -100;
    }
    h_launches += kernels;
    return 0;
}

}  // namespace lg

extern "C" {

int lila_gpu_set_precision(int mode)
{
    const int prev = lg::g_precision;
    if (mode == 0 || mode == 1) lg::g_precision = mode;
    return prev;
}

int lila_gpu_graph_mode(int on)
{
    const int prev = lg::g_graph_mode;
    if (on > 0) {
        lg::status_ptr();  // one-time device lookups must not happen inside a capture
        lg::sm_count();
        lg::noalloc_scratch_addr();
    }
    if (on >= 0) lg::g_graph_mode = on ? 1 : 0;
    return prev;
}

int lila_gpu_graph_cache_clear(void)
{
    std::lock_guard<std::mutex> lk(lg::g_graph_mu);
    for (auto &e : lg::g_graphs)
        if (e.exec) cudaGraphExecDestroy(e.exec);
    const int n = (int)lg::g_graphs.size();
    lg::g_graphs.clear();
    return n;
}

unsigned long long lila_gpu_graph_replays(void) { return lg::g_graph_replays; }

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
        cudaMemcpyAsync(&v, p, sizeof(int), cudaMemcpyDeviceToHost, lg::t_stream);
        cudaStreamSynchronize(lg::t_stream);
    }
    if (lg::h_launch_error) v |= lg::ST_LAUNCH_ERROR;
    return v;
}

int lila_gpu_clear_status(void)
{
    int *p = lg::status_ptr();
    lg::h_launch_error = 0;
    if (!p) return -1;
    const cudaError_t e = cudaMemsetAsync(p, 0, sizeof(int), lg::t_stream);
    return (e == cudaSuccess && cudaStreamSynchronize(lg::t_stream) == cudaSuccess) ? 0 : -1;
}

int lila_gpu_version(void) { return LILA_GPU_VERSION; }

long long lila_gpu_set_wait_limit(long long cycles)
{
    const long long prev = lg::g_wait_limit;
    if (cycles > 0) lg::g_wait_limit = cycles;
    return prev;
}

unsigned long long lila_gpu_launch_count(void) { return lg::h_launches; }

static void trace_clear()
{
    for (auto &r : lg::g_recs) {
        if (r.own_a) lg::g_event_pool.push_back(r.a);
        lg::g_event_pool.push_back(r.b);
    }
    lg::g_recs.clear();
    lg::g_chain = nullptr;
}

int lila_gpu_trace(int on)
{
    cudaStreamSynchronize(lg::t_stream);
    trace_clear();
    lg::g_trace = on != 0;
    while (lg::g_trace && lg::g_event_pool.size() < lg::kEventPool) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) {
            cudaGetLastError();
            break;
        }
        lg::g_event_pool.push_back(e);
    }
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
