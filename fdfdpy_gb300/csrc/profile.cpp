// Kernel-class profiler of the engine (see profile.h).
#include "profile.h"

#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "fdfd_internal.h"

namespace fdfd {

namespace {
struct Pending {
    int cls;
    cudaEvent_t a, b;
};
std::atomic<bool> g_enabled{false};
std::atomic<long long> g_launches[PROF_NCLASS];
std::mutex g_mu;  // event bookkeeping (timing is meant for one stream at a time)
double g_ms[PROF_NCLASS] = {};
std::vector<Pending> g_pending;
std::vector<cudaEvent_t> g_free;
cudaEvent_t g_open[PROF_NCLASS] = {};

cudaEvent_t take() {
    if (!g_free.empty()) {
        cudaEvent_t e = g_free.back();
        g_free.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}
}  // namespace

void prof_begin(int cls, cudaStream_t st) {
    if (!g_enabled) return;
    std::lock_guard<std::mutex> lk(g_mu);
    cudaEvent_t e = take();
    cudaEventRecord(e, st);
    g_open[cls] = e;
}

bool prof_enabled() { return g_enabled; }
long long prof_launches(int cls) { return g_launches[cls]; }
void prof_count(int cls, long long launches) { g_launches[cls] += launches; }

void prof_end(int cls, cudaStream_t st, int launches) {
    g_launches[cls] += launches;
    if (!g_enabled) return;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_open[cls]) return;
    cudaEvent_t e = take();
    cudaEventRecord(e, st);
    g_pending.push_back({cls, g_open[cls], e});
    g_open[cls] = nullptr;
}

}  // namespace fdfd

using namespace fdfd;

extern "C" int fdfd_profile_enable(int32_t on) {
    g_enabled = on != 0;
    return FDFD_OK;
}

extern "C" int fdfd_profile_reset(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    for (int c = 0; c < PROF_NCLASS; ++c) {
        g_launches[c] = 0;
        g_ms[c] = 0.0;
    }
    for (auto &p : g_pending) {
        g_free.push_back(p.a);
        g_free.push_back(p.b);
    }
    g_pending.clear();
    return FDFD_OK;
}

extern "C" int fdfd_profile_read(int32_t nclass, double *ms, int64_t *launches) {
    if (nclass < 1 || !ms || !launches) return fail(FDFD_ERR_BAD_ARG, "profile_read: bad argument");
    std::lock_guard<std::mutex> lk(g_mu);
    for (auto &p : g_pending) {
        if (cudaEventSynchronize(p.b) != cudaSuccess) {
            cudaGetLastError();
            return fail(FDFD_ERR_CUDA, "profile_read: event synchronisation failed");
        }
        float t = 0.f;
        if (cudaEventElapsedTime(&t, p.a, p.b) == cudaSuccess) g_ms[p.cls] += t;
        g_free.push_back(p.a);
        g_free.push_back(p.b);
    }
    g_pending.clear();
    for (int c = 0; c < nclass && c < PROF_NCLASS; ++c) {
        ms[c] = g_ms[c];
        launches[c] = g_launches[c];
    }
    return FDFD_OK;
}
