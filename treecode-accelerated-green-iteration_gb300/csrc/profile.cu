// Launch counter and per-phase CUDA-event timing.
//
// Phases: tree (sort + octree + boxes), lists (batches, traversal, slots,
// weight charges), upward (modified charges), near field, far field, glue
// (charge sorting, epilogue).  Events are recorded on the stream the phase's
// kernels are launched on, so elapsed times are device times of that stream.
#include "tagi_internal.h"

#include <atomic>
#include <mutex>

namespace tagi {

namespace {
std::atomic<long long> g_launches{0};
std::atomic<int> g_profile{0};
std::mutex g_pmu;
struct Mark {
    int phase;
    cudaEvent_t a, b;
};
std::vector<Mark> g_marks;
cudaEvent_t g_open[PH_COUNT] = {};
}  // namespace

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

void phase_mark(int phase, bool begin, cudaStream_t s) {
    if (!g_profile.load(std::memory_order_relaxed) || phase < 0 || phase >= PH_COUNT) return;
    if (stream_capturing(s)) return;  // events inside a graph would be read before they run
    std::lock_guard<std::mutex> lk(g_pmu);
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return;
    cudaEventRecord(e, s);
    if (begin) {
        if (g_open[phase]) cudaEventDestroy(g_open[phase]);
        g_open[phase] = e;
    } else if (g_open[phase]) {
        g_marks.push_back({phase, g_open[phase], e});
        g_open[phase] = nullptr;
    } else {
        cudaEventDestroy(e);
    }
}

}  // namespace tagi

using namespace tagi;

extern "C" {

long long tagi_launch_count(void) { return g_launches.load(); }

int tagi_profile(int enable) {
    g_profile.store(enable ? 1 : 0);
    return TAGI_OK;
}

int tagi_profile_read(double *ms, long long *count, int nphase) {
    if (!ms || !count || nphase < PH_COUNT) return set_error(TAGI_ERR_ARG, "tagi_profile_read needs %d slots", (int)PH_COUNT);
    std::lock_guard<std::mutex> lk(g_pmu);
    for (int i = 0; i < nphase; i++) {
        ms[i] = 0.0;
        count[i] = 0;
    }
    int rc = TAGI_OK;
    for (const Mark &m : g_marks) {
        float t = 0.f;
        if (cudaEventSynchronize(m.b) != cudaSuccess || cudaEventElapsedTime(&t, m.a, m.b) != cudaSuccess)
            rc = set_error(TAGI_ERR_CUDA, "profile event read failed");
        ms[m.phase] += t;
        count[m.phase] += 1;
        cudaEventDestroy(m.a);
        cudaEventDestroy(m.b);
    }
    g_marks.clear();
    return rc;
}

}  // extern "C"
