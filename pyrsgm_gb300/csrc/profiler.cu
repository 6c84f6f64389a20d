// profiler.cu -- opt-in per-kernel timing with CUDA events on the launching
// stream, plus the algorithmic bytes of every launch.  Off by default (no
// events are recorded); enabled by pyrsgm_gb300_profile(1).
#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include "pyrsgm/pyrsgm_gb300.h"
#include "profiler.h"

namespace pg {
namespace {

struct Rec {
    int kind;
    cudaEvent_t a, b;
    double bytes;
};

std::mutex g_mu;
bool g_on = false;
std::vector<Rec> g_recs;
std::vector<cudaEvent_t> g_pool;
thread_local cudaEvent_t t_open = nullptr;

cudaEvent_t take()
{
    if (!g_pool.empty()) {
        cudaEvent_t e = g_pool.back();
        g_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    return e;
}

}  // namespace

bool prof_enabled() { return g_on; }

void prof_begin(cudaStream_t st)
{
    if (!g_on) return;
    std::lock_guard<std::mutex> lk(g_mu);
    t_open = take();
    if (t_open) cudaEventRecord(t_open, st);
}

void prof_end(int kind, double bytes, cudaStream_t st)
{
    if (!g_on || !t_open) return;
    std::lock_guard<std::mutex> lk(g_mu);
    cudaEvent_t b = take();
    if (!b) return;
    cudaEventRecord(b, st);
    g_recs.push_back({kind, t_open, b, bytes});
    t_open = nullptr;
}

}  // namespace pg

extern "C" {

int pyrsgm_gb300_profile(int enable)
{
    std::lock_guard<std::mutex> lk(pg::g_mu);
    for (auto& r : pg::g_recs) {
        pg::g_pool.push_back(r.a);
        pg::g_pool.push_back(r.b);
    }
    pg::g_recs.clear();
    if (enable && pg::g_pool.size() < 4096) {
        for (int i = 0; i < 4096; ++i) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return -1;
            pg::g_pool.push_back(e);
        }
    }
    pg::g_on = enable != 0;
    return 0;
}

int pyrsgm_gb300_profile_read(int kind, double* ms_total, long long* launches, double* bytes_total)
{
    std::lock_guard<std::mutex> lk(pg::g_mu);
    double ms = 0.0, by = 0.0;
    long long n = 0;
    for (auto& r : pg::g_recs) {
        if (r.kind != kind) continue;
        if (cudaEventSynchronize(r.b) != cudaSuccess) return -1;
        float t = 0.0f;
        if (cudaEventElapsedTime(&t, r.a, r.b) != cudaSuccess) return -1;
        ms += t;
        by += r.bytes;
        ++n;
    }
    if (ms_total) *ms_total = ms;
    if (launches) *launches = n;
    if (bytes_total) *bytes_total = by;
    return 0;
}

}  // extern "C"
