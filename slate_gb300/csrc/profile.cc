// profile.cc -- launch counting and optional per-kernel CUDA-event timing.
//
// Every kernel launcher in this library calls count_launch(); the launchers of
// the heavy kernels additionally bracket their launch with prof_begin /
// prof_end when profiling is on, recording CUDA events on the launch stream
// and the launch's algorithmic flops and bytes.  slt_profile_read resolves
// the events (device synchronisation) and sums per kernel class.

#include <atomic>
#include <mutex>
#include <vector>

#include "prof.h"
#include "status.h"

namespace slt {

static std::atomic<long long> g_launches{0};
static std::atomic<bool> g_on{false};
static std::mutex g_mtx;

struct Rec {
    int kind;
    cudaEvent_t a, b;
    double flops, bytes;
    bool closed;
};
static std::vector<Rec> g_recs;

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

static thread_local int t_sm_cap = 0;

int capped_sms(int sms) { return (t_sm_cap > 0 && t_sm_cap < sms) ? t_sm_cap : sms; }

int prof_begin(int kind, cudaStream_t s)
{
    if (!g_on.load(std::memory_order_relaxed)) return -1;
    Rec r{kind, nullptr, nullptr, 0, 0, false};
    if (cudaEventCreate(&r.a) != cudaSuccess || cudaEventCreate(&r.b) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    cudaEventRecord(r.a, s);
    std::lock_guard<std::mutex> lk(g_mtx);
    g_recs.push_back(r);
    return int(g_recs.size()) - 1;
}

void prof_end(int idx, cudaStream_t s, double flops, double bytes)
{
    if (idx < 0) return;
    std::lock_guard<std::mutex> lk(g_mtx);
    if (idx >= int(g_recs.size())) return;
    Rec& r = g_recs[idx];
    cudaEventRecord(r.b, s);
    r.flops = flops;
    r.bytes = bytes;
    r.closed = true;
}

} // namespace slt

using namespace slt;

extern "C" long long slt_launch_count(void) { return g_launches.load(); }

extern "C" void slt_profile_enable(int on)
{
    std::lock_guard<std::mutex> lk(g_mtx);
    for (auto& r : g_recs) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    g_recs.clear();
    g_on.store(on != 0);
}

extern "C" int slt_profile_read(int kind, double* flops, double* bytes, double* seconds, long long* launches)
{
    SLT_CUDA_TRY(cudaDeviceSynchronize());
    std::lock_guard<std::mutex> lk(g_mtx);
    double f = 0, by = 0, t = 0;
    long long c = 0;
    for (auto& r : g_recs) {
        if (r.kind != kind || !r.closed) continue;
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, r.a, r.b) != cudaSuccess) { cudaGetLastError(); continue; }
        f += r.flops;
        by += r.bytes;
        t += ms * 1e-3;
        ++c;
    }
    if (flops) *flops = f;
    if (bytes) *bytes = by;
    if (seconds) *seconds = t;
    if (launches) *launches = c;
    return SLT_OK;
}

extern "C" int slt_set_sm_cap(int sms)
{
    const int prev = slt::t_sm_cap;
    slt::t_sm_cap = sms > 0 ? sms : 0;
    return prev;
}

extern "C" int slt_sm_cap(void) { return slt::t_sm_cap; }
