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

// ---------------------------------------------------------------------------
// Hardware pipe rates.  Every thread runs 8 independent dependency chains of
// one instruction kind, every SM holds 2048 threads, nothing touches memory
// until the end.  OP 0: FFMA; 1: FFMA2 (packed pair, 2 lanes); 2: MUFU ex2;
// 3: MUFU rsqrt; 4: DFMA (FP64); 5: MUFU lg2.  The ex2 and lg2 chains leave
// the finite range after a few steps (inf, NaN); the MUFU pipe's rate does not
// depend on the operand.  Each block's thread 0 records the clock64 span of its
// block; the longest span over event time is the SM clock during the run.
// ---------------------------------------------------------------------------
namespace {
constexpr int PR_THREADS = 256;
constexpr int PR_CHAINS = 8;

template <int OP>
__global__ void __launch_bounds__(PR_THREADS) pipe_rate_kernel(int reps, float *out, unsigned long long *cycles) {
    const long long c0 = clock64();
    float a[PR_CHAINS];
    float2 b[PR_CHAINS];
    double c[PR_CHAINS];
#pragma unroll
    for (int i = 0; i < PR_CHAINS; i++) {
        a[i] = 0.5f + 1e-3f * (threadIdx.x + i);
        b[i] = make_float2(a[i], a[i] + 0.25f);
        c[i] = (double)a[i];
    }
    const float2 m2 = make_float2(0.9999f, 0.9998f), c2 = make_float2(1e-4f, 2e-4f);
    for (int r = 0; r < reps; r++) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
#pragma unroll
            for (int i = 0; i < PR_CHAINS; i++) {
                if (OP == 0) a[i] = fmaf(a[i], 0.9999f, 1e-4f);
                if (OP == 1) b[i] = __ffma2_rn(b[i], m2, c2);
                if (OP == 2) asm volatile("ex2.approx.ftz.f32 %0, %0;" : "+f"(a[i]));
                if (OP == 3) asm volatile("rsqrt.approx.ftz.f32 %0, %0;" : "+f"(a[i]));
                if (OP == 4) c[i] = fma(c[i], 0.9999, 1e-4);
                if (OP == 5) asm volatile("lg2.approx.ftz.f32 %0, %0;" : "+f"(a[i]));
            }
        }
    }
    float acc = 0.f;
#pragma unroll
    for (int i = 0; i < PR_CHAINS; i++) acc += a[i] + b[i].x + b[i].y + (float)c[i];
    out[blockIdx.x * PR_THREADS + threadIdx.x] = acc;
    if (threadIdx.x == 0) atomicMax(cycles, (unsigned long long)(clock64() - c0));   // the longest-running block
}

template <int OP>
int time_pipe(int grid, float *out, unsigned long long *d_cycles, cudaStream_t s, double *lane_ops_per_s,
              double *mhz) {
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    int reps = 64, rc = TAGI_OK;
    float ms = 0.f;
    for (int attempt = 0; attempt < 8; attempt++) {   // grow until the timed launch lasts >= 20 ms
        launch(pipe_rate_kernel<OP>, grid, PR_THREADS, 0, s, reps, out, d_cycles);
        cudaMemsetAsync(d_cycles, 0, sizeof(long long), s);
        cudaEventRecord(a, s);
        launch(pipe_rate_kernel<OP>, grid, PR_THREADS, 0, s, reps, out, d_cycles);
        cudaEventRecord(b, s);
        if (cudaEventSynchronize(b) != cudaSuccess) {
            rc = set_error(TAGI_ERR_CUDA, "pipe-rate launch failed");
            break;
        }
        cudaEventElapsedTime(&ms, a, b);
        if (ms >= 20.f) break;
        reps *= 4;
    }
    unsigned long long cyc = 0;
    if (!rc && cudaMemcpy(&cyc, d_cycles, sizeof(cyc), cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = set_error(TAGI_ERR_CUDA, "pipe-rate clock read failed");
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (rc) return rc;
    const double lanes_per_inst = OP == 1 ? 2.0 : 1.0;
    *lane_ops_per_s = (double)grid * PR_THREADS * PR_CHAINS * 4.0 * reps * lanes_per_inst / (ms * 1e-3);
    *mhz = (double)cyc / (ms * 1e-3) / 1e6;
    return TAGI_OK;
}
}  // namespace

// One wave: as many blocks as fit on the SMs at once, so every block runs
// from the first to the last cycle of the launch and the longest block's
// clock64 span is the launch's span.
template <int OP>
int pipe_grid(int sms, int *grid) {
    int per = 0;
    TAGI_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, pipe_rate_kernel<OP>, PR_THREADS, 0));
    *grid = sms * (per > 0 ? per : 1);
    return TAGI_OK;
}

int pipe_rates(double *rates, cudaStream_t s) {
    int dev = 0, sms = 0;
    TAGI_CUDA(cudaGetDevice(&dev));
    TAGI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    int grid = 0, g[6];
    TAGI_TRY(pipe_grid<0>(sms, &g[0]));
    TAGI_TRY(pipe_grid<1>(sms, &g[1]));
    TAGI_TRY(pipe_grid<2>(sms, &g[2]));
    TAGI_TRY(pipe_grid<3>(sms, &g[3]));
    TAGI_TRY(pipe_grid<4>(sms, &g[4]));
    TAGI_TRY(pipe_grid<5>(sms, &g[5]));
    for (int i = 0; i < 6; i++) grid = g[i] > grid ? g[i] : grid;
    Arena tmp;
    tmp.stream = s;
    float *out = nullptr;
    unsigned long long *cyc = nullptr;
    int rc = TAGI_OK;
    double mhz[6] = {0, 0, 0, 0, 0, 0};
    do {
        if ((rc = tmp.alloc(&out, (size_t)grid * PR_THREADS)) || (rc = tmp.alloc(&cyc, 1))) break;
        if ((rc = time_pipe<0>(g[0], out, cyc, s, &rates[0], &mhz[0]))) break;
        if ((rc = time_pipe<1>(g[1], out, cyc, s, &rates[1], &mhz[1]))) break;
        if ((rc = time_pipe<2>(g[2], out, cyc, s, &rates[2], &mhz[2]))) break;
        if ((rc = time_pipe<3>(g[3], out, cyc, s, &rates[3], &mhz[3]))) break;
        if ((rc = time_pipe<4>(g[4], out, cyc, s, &rates[6], &mhz[4]))) break;
        if ((rc = time_pipe<5>(g[5], out, cyc, s, &rates[7], &mhz[5]))) break;
    } while (0);
    tmp.release();
    if (rc) return rc;
    rates[4] = mhz[0];
    rates[5] = (double)sms;
    return TAGI_OK;
}

}  // namespace tagi

using namespace tagi;

extern "C" {

long long tagi_launch_count(void) { return g_launches.load(); }

int tagi_pipe_rates(double *rates, void *stream) {
    if (!rates) return set_error(TAGI_ERR_ARG, "null output");
    return pipe_rates(rates, (cudaStream_t)stream);
}

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
