// profile.cu — optional per-kernel timing with CUDA events on the launching stream.
//
// When enabled, every public call records an event pair around each of its kernels. The pairs
// are resolved (synchronously) by se_gpu_profiling_read, which returns the accumulated device
// time and the number of launches per kernel. Disabled by default; no cost when off.
#include <cstring>
#include <mutex>
#include <vector>

#include "profile.cuh"

namespace se_gpu {

namespace {
struct Pending {
    int kernel;
    cudaEvent_t start, stop;
};
std::mutex g_mu;
bool g_enabled = false;
int g_suspended = 0; // > 0 while a CUDA graph is being captured
std::vector<Pending> g_pending;
std::vector<cudaEvent_t> g_free;
double g_total_ms[kProfCount];
long long g_launches[kProfCount];

cudaEvent_t take_event()
{
    if (!g_free.empty()) {
        cudaEvent_t e = g_free.back();
        g_free.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}
} // namespace

const char* const kProfNames[kProfCount] = {"integrate_prep", "carve", "frustum", "update", "raycast",
                                            "track_prep", "icp_iter", "icp_check", "frame_graph"};

bool profiling_enabled() { return g_enabled && g_suspended == 0; }

void profiling_suspend(bool suspend)
{
    std::lock_guard<std::mutex> lk(g_mu);
    g_suspended += suspend ? 1 : -1;
}

ProfScope::ProfScope(int kernel, cudaStream_t stream) : kernel_(kernel), stream_(stream), start_(nullptr)
{
    if (!g_enabled || g_suspended)
        return;
    std::lock_guard<std::mutex> lk(g_mu);
    start_ = take_event();
    cudaEventRecord(start_, stream_);
}

ProfScope::~ProfScope()
{
    if (!start_)
        return;
    std::lock_guard<std::mutex> lk(g_mu);
    cudaEvent_t stop = take_event();
    cudaEventRecord(stop, stream_);
    g_pending.push_back(Pending{kernel_, start_, stop});
}

} // namespace se_gpu

using namespace se_gpu;

extern "C" {

SE_GPU_API se_gpu_status se_gpu_profiling_enable(int enable)
{
    std::lock_guard<std::mutex> lk(g_mu);
    g_enabled = enable != 0;
    return SE_GPU_OK;
}

SE_GPU_API se_gpu_status se_gpu_profiling_read(int n, double* total_ms, int64_t* launches, int reset)
{
    std::lock_guard<std::mutex> lk(g_mu);
    for (const Pending& p : g_pending) {
        cudaError_t e = cudaEventSynchronize(p.stop);
        if (e != cudaSuccess)
            return cuda_status(e, "se_gpu_profiling_read");
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, p.start, p.stop);
        g_total_ms[p.kernel] += ms;
        g_launches[p.kernel] += 1;
        g_free.push_back(p.start);
        g_free.push_back(p.stop);
    }
    g_pending.clear();
    for (int i = 0; i < n && i < kProfCount; ++i) {
        if (total_ms)
            total_ms[i] = g_total_ms[i];
        if (launches)
            launches[i] = g_launches[i];
    }
    if (reset) {
        std::memset(g_total_ms, 0, sizeof(g_total_ms));
        std::memset(g_launches, 0, sizeof(g_launches));
    }
    return SE_GPU_OK;
}

SE_GPU_API const char* se_gpu_profiling_name(int i)
{
    return (i >= 0 && i < kProfCount) ? kProfNames[i] : "";
}

SE_GPU_API int se_gpu_profiling_count(void) { return kProfCount; }

} // extern "C"
