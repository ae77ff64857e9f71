// Internal declarations shared by the CUDA translation units of libtagi_gb300.
//
// Data layout in HBM (one plan = one mesh / one source-target pair):
//   sorted sources   x,y,z,w  FP64 SoA in Morton order (plus FP32 w for the
//                    mixed path); perm maps sorted position -> caller index
//   sorted targets   x,y,z    FP64 SoA in Morton order
//   tree nodes       begin,end,parent,first_child,nchild (int32 SoA);
//                    center, half (FP64, 3 per node), radius (FP64)
//   lists            CSR per target batch: near node ids, far node ids, and
//                    the near list merged into contiguous source ranges
//   slots            one per far-list node: proxy geometry + modified charges
//                    [slot][P] (P = (degree+1)^3), FP32 (mixed) or FP64
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <utility>
#include <vector>

#include "../../include/tagi_gb300.h"  // status codes TAGI_OK, TAGI_ERR_*

namespace tagi {

// Kernel / singularity / approximation / compute-type values are those of
// 3D-GreenIteration/src/utilities/BaryTreeInterface.py:20-46.
enum { KERNEL_COULOMB = 1, KERNEL_YUKAWA = 2 };
enum { SING_NONE = 0, SING_SKIPPING = 1, SING_SUBTRACTION = 2 };
enum { APPROX_LAGRANGE = 1 };
enum { COMPUTE_PARTICLE_CLUSTER = 1 };
enum { PREC_MIXED = 0, PREC_FP64 = 1 };

constexpr int MAX_DEGREE = 10;        // far-field kernels are instantiated for 1..10
constexpr int TRAVERSAL_STACK = 256;  // DFS stack entries per target batch

int set_error(int code, const char *fmt, ...);
int last_error();
// Argument checks shared by the C entry points (capi.cu).
int validate(int nt, int ns, int kernel, int nkp, const double *kp, int sing, int approx, int ctype, double theta,
             int degree, int sl, int tl, double size_check, int precision);
int validate_kparam(int kernel, int sing, double k);

#define TAGI_CUDA(call)                                                                   \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return ::tagi::set_error(::TAGI_ERR_CUDA, "%s: %s (%s:%d)", #call,      \
                                     cudaGetErrorString(e_), __FILE__, __LINE__);         \
    } while (0)

#define TAGI_TRY(expr)                 \
    do {                               \
        int s_ = (expr);               \
        if (s_ != 0) return s_;        \
    } while (0)

#define TAGI_LAUNCH_CHECK() TAGI_CUDA(cudaGetLastError())

// Every kernel of the library goes through launch(): it counts launches
// (tagi_launch_count) so a caller can state how many kernels ran.
void count_launch();
template <typename... KArgs, typename... Args>
inline void launch(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                   Args &&...args) {
    count_launch();
    kern<<<grid, block, smem, s>>>(std::forward<Args>(args)...);
}

// Merged near ranges are int2 {begin, end} in sorted source order; bit 31 of
// begin marks a CLOSE range: its box lies within 0.1 batch radii of the
// batch's box (touching included).  Close ranges hold the short pairs whose
// FP32 batch-relative coordinates would lose relative precision, and any
// source that may coincide with a target; the field kernels give them
// double-float coordinates and the r = 0 mask.  Decode only through these.
__host__ __device__ __forceinline__ int range_begin(int2 r) { return r.x & 0x7fffffff; }
__host__ __device__ __forceinline__ bool range_is_close(int2 r) { return r.x < 0; }
constexpr double CLOSE_RANGE_FRACTION = 0.1;

// Optional per-phase timing with CUDA events on the launching stream
// (tagi_profile / tagi_profile_read); no-ops unless enabled.
enum Phase { PH_TREE = 0, PH_LISTS, PH_UPWARD, PH_NEAR, PH_FAR, PH_GLUE, PH_NEAR_CLOSE, PH_COUNT };
void phase_mark(int phase, bool begin, cudaStream_t s);

// Stream-ordered device allocations owned by a plan (freed on destroy).
struct Arena {
    std::vector<void *> ptrs;
    cudaStream_t stream = nullptr;
    template <typename T>
    int alloc(T **p, size_t count) {
        void *v = nullptr;
        size_t bytes = count * sizeof(T);
        if (bytes == 0) bytes = 16;
        cudaError_t e = cudaMallocAsync(&v, bytes, stream);
        if (e != cudaSuccess)
            return set_error(TAGI_ERR_CUDA, "device allocation of %zu bytes failed: %s", bytes,
                             cudaGetErrorString(e));
        ptrs.push_back(v);
        *p = static_cast<T *>(v);
        return TAGI_OK;
    }
    void release() {
        for (void *p : ptrs) cudaFreeAsync(p, stream);
        ptrs.clear();
    }
};

struct Tree {
    int n = 0;
    int nnodes = 0;
    int nlevels = 0;
    std::vector<int> level_start;  // host copy: node index where each BFS level begins
    uint64_t *codes = nullptr;     // sorted Morton codes
    int *perm = nullptr;           // sorted position -> caller index
    double *x = nullptr, *y = nullptr, *z = nullptr;  // sorted coordinates
    int *begin = nullptr, *end = nullptr, *parent = nullptr, *first_child = nullptr,
        *nchild = nullptr;
    double *center = nullptr, *half = nullptr, *radius = nullptr;
};

// Work list of one field launch: items {batch, sys << 16 | first orbital},
// heaviest first, in three segments: near pass 0 (every batch), near close
// pass (batches with close ranges), far field (batches with far entries).
// og orbitals per item (orbital-group kernels) or 1.
struct Schedule {
    int og = 0;                 // 0 = not built
    std::vector<int> norb;      // orbitals per system the schedule was built for
    int2 *items = nullptr;      // device, owned
    int count[3] = {0, 0, 0};
    long off[3] = {0, 0, 0};
    void release() {  // caller makes sure no launch still reads the list
        if (items) cudaFree(items);
        items = nullptr;
        og = 0;
        norb.clear();
    }
};

struct Plan {
    int device = 0;
    Arena arena;
    Tree src, tgt;
    int degree = 7, n1 = 8, P = 512;
    double theta = 0.7, size_check = 1.0;
    int source_leaf = 500, target_leaf = 500;
    int nbatch = 0, max_batch = 0;
    int *batch_node = nullptr;             // target-tree leaf of each batch
    int *near_off = nullptr, *near_list = nullptr;
    int *far_off = nullptr, *far_list = nullptr;
    int near_total = 0, far_total = 0;
    int *rng_off = nullptr;                // merged near ranges (CSR)
    int2 *rng = nullptr;
    float *rng_dmin = nullptr;             // lower bound of batch-to-range distance
    int rng_total = 0;
    int nslots = 0;
    int *node_slot = nullptr, *slot_node = nullptr;
    double *slot_geom = nullptr;           // [slot][6] = center xyz, proxy half xyz
    // upward-pass work items (slot, source chunk)
    int nitems = 0;
    int *item_slot = nullptr, *item_begin = nullptr, *item_end = nullptr;
    int *slot_item_off = nullptr;          // [nslots+1]
    float4 *src_hi = nullptr, *src_lo = nullptr;  // FP32 hi/lo of sorted source x, y, z
    float4 *tgt_hi = nullptr, *tgt_lo = nullptr;  // same for targets
    double *sw64 = nullptr;                // sorted source weights
    float *sw32 = nullptr;
    float *what32 = nullptr;               // weight modified charges [slot][P]
    double *what64 = nullptr;              // FP64 set, built on first FP64 use
    bool what64_ready = false;
    int *queue = nullptr;                  // work-queue counters (3 ints)
    int *err_flag = nullptr;               // [0] tree/list build, [1] unusable kernel parameter
    double cheb[MAX_DEGREE + 1];           // cos(m pi / degree)
    // per-convolution scratch (grown on demand)
    size_t scratch_orbitals = 0;
    float *q32 = nullptr;                  // [norb][ns] sorted charges f*w (FP32)
    float *ft32 = nullptr;                 // [norb][nt] sorted target values (FP32)
    double *q64 = nullptr;                 // [norb][ns] sorted charges f*w
    double *f64s = nullptr;                // [norb][ns] sorted source values f
    double *ft64 = nullptr;                // [norb][nt] sorted target values
    double *part = nullptr;                // upward-pass partials [norb][nitems][P]
    float *qhat32 = nullptr;               // [norb][nslots][P]
    double *qhat64 = nullptr;
    double *near_out = nullptr, *far_out = nullptr;  // [norb][nt] sorted order
    double *near2_out = nullptr;           // close-range pass of the near field
    float *d_kc = nullptr;                 // [norb] exp2 constants
    double *d_kp = nullptr, *d_ss = nullptr;         // [norb] k (or a), SS factor
    std::vector<float> h_kc;
    std::vector<double> h_kp, h_ss;
    std::vector<void *> scratch;           // freed on regrow / destroy
    // statistics (host)
    double near_pairs = 0, far_pairs = 0;  // pair interactions per orbital
    double near_close_pairs = 0;           // part of near_pairs in close ranges
    // per-batch pair counts (host) for work ordering: ordinary near ranges,
    // close ranges, far field
    std::vector<long long> cost_near, cost_close, cost_far;
    std::vector<Schedule> scheds;          // single-plan work lists by (orbitals, group), cached
};

// One system of a (possibly multi-system) convolution call.
struct SysCall {
    Plan *p = nullptr;
    const double *tv = nullptr, *sv = nullptr;  // device [norb][nt], [norb][ns], caller order
    double *out = nullptr;                      // device [norb][nt], caller order
    int norb = 1;
    const double *kp = nullptr;  // kernel parameters: k (or a) of orbital o at kp[o * nkp]
    int nkp = 1;
    bool kp_device = false;      // kp is a device pointer (graph-capturable calls)
};

struct Plan;
int plan_create(Plan **out, int nt, const double *tx, const double *ty, const double *tz, int ns,
                const double *sx, const double *sy, const double *sz, const double *sw, double theta, int degree,
                int sl, int tl, double size_check, cudaStream_t s);
void plan_destroy(Plan *p);

// scan_sort.cu
int exclusive_scan(const int *in, int *out, int n, int *d_total, Arena &ar, cudaStream_t s);
int radix_sort_u64(uint64_t *keys, int *vals, int n, Arena &ar, cudaStream_t s);

// tree.cu
int build_tree(Tree &t, const double *x, const double *y, const double *z, int n, int leaf,
               Arena &ar, int *err_flag, cudaStream_t s);
int build_lists(Plan &p, cudaStream_t s);

// upward.cu
int build_weight_charges(Plan &p, cudaStream_t s);
int ensure_weight_charges64(Plan &p, cudaStream_t s);
int modified_charges(Plan &p, int precision, int norb, cudaStream_t s);

// fields.cu
constexpr int MAX_SYSTEMS = 8;  // systems per field launch
int ensure_scratch(Plan &p, int norb);
int orbitals_per_item(int kernel, int precision, const int *norb, const double *weight, int nsys, int requested,
                      int max_n1);
int build_schedule(Plan *const *plans, const int *norb, int nsys, int og, Schedule &sc, cudaStream_t s);
bool schedule_matches(const Schedule &sc, const int *norb, int nsys, int og);
int convolve_systems(SysCall *calls, int nsys, int kernel, int singularity, int precision,
                     const Schedule &sc, int *queue, cudaStream_t s, int nt_request = 0);
int convolve(Plan &p, const double *tv, const double *sv, double *out, int norb, int kernel,
             const double *kparams, int nkp, int singularity, int precision, cudaStream_t s,
             bool kp_device = false, int og_request = 0, int nt_request = 0);
bool stream_capturing(cudaStream_t s);
int direct_sum(int nt, const double *tx, const double *ty, const double *tz, const double *tv,
               int nsub, const int *sub, int ns, const double *sx, const double *sy,
               const double *sz, const double *sv, const double *sw, double *out, int kernel,
               double kp, int singularity, int precision, cudaStream_t s);

int pair_peak(int kernel, int singularity, int variant, double kp, double *pairs_per_s, cudaStream_t s);
int pipe_rates(double *rates, cudaStream_t s);

// mgs.cu / interp.cu
int mgs_device(double *V, double *U, const double *W, int target, int npts, int nwave,
               cudaStream_t s);
int interp_device(const double *cX, const double *cY, const double *cZ, const double *cF,
                  const int *ppc_c, int coarseN, const double *fX, const double *fY,
                  const double *fZ, double *fF, const int *ppc_f, int fineN, int ncells,
                  int order, const int *h_ppc_c, const int *h_ppc_f, cudaStream_t s);

}  // namespace tagi
