// Subsystem (e), part 1: quadrature-weighted Gram-Schmidt of one orbital,
// the device counterpart of modifiedGramSchmidt_singleWavefunction
// (3D-GreenIteration/src/utilities/Orthogonalization.c:14-119), one GPU, FP64:
//   r_i = sum_j V_ij U_j W_j          (i < target)         :44-54
//   U_j -= sum_i r_i V_ij  (i in order, per point)         :71-79
//   U  /= sqrt(sum_j U_j^2 W_j);  V[target] = U            :85-106
// The projections use the incoming U (classical order inside one call), as the
// reference does.  HBM-bound: V's rows are read twice (dots, then subtract);
// U and W are read per row group from L2.  Reductions are per block then
// summed in block order, so results do not depend on scheduling.
#include "tagi_internal.h"

#include <algorithm>
#include <mutex>

namespace tagi {

namespace {

constexpr int MT = 256;
constexpr int RB = 8;   // rows per thread in the dot kernel

__device__ __forceinline__ double block_sum(double v, double *sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < MT / 32; w++) s += sh[w];
    return s;  // valid in thread 0
}

// partial[blk][i] for rows i in this block's row group.
__global__ void __launch_bounds__(MT) mgs_dots(const double *__restrict__ V,
                                               const double *__restrict__ U,
                                               const double *__restrict__ W, int target,
                                               long npts, long chunk,
                                               double *__restrict__ partial) {
    __shared__ double sh[MT / 32];
    const int r0 = blockIdx.y * RB;
    const long j0 = (long)blockIdx.x * chunk;
    const long j1 = min(j0 + chunk, npts);
    double acc[RB];
#pragma unroll
    for (int r = 0; r < RB; r++) acc[r] = 0.0;
    for (long j = j0 + threadIdx.x; j < j1; j += MT) {
        const double uw = U[j] * W[j];
#pragma unroll
        for (int r = 0; r < RB; r++)
            if (r0 + r < target) acc[r] += V[(long)(r0 + r) * npts + j] * uw;
    }
#pragma unroll
    for (int r = 0; r < RB; r++) {
        double s = block_sum(acc[r], sh);
        if (threadIdx.x == 0 && r0 + r < target) partial[(long)blockIdx.x * target + r0 + r] = s;
    }
}

__global__ void mgs_reduce_rows(const double *__restrict__ partial, int nblk, int target,
                                double *__restrict__ r) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= target) return;
    double s = 0.0;
    for (int b = 0; b < nblk; b++) s += partial[(long)b * target + i];
    r[i] = s;
}

__global__ void __launch_bounds__(MT) mgs_subtract(const double *__restrict__ V,
                                                   double *__restrict__ U,
                                                   const double *__restrict__ W,
                                                   const double *__restrict__ r, int target,
                                                   long npts, long chunk,
                                                   double *__restrict__ npart) {
    __shared__ double sh[MT / 32];
    const long j0 = (long)blockIdx.x * chunk;
    const long j1 = min(j0 + chunk, npts);
    double acc = 0.0;
    for (long j = j0 + threadIdx.x; j < j1; j += MT) {
        double u = U[j];
        for (int i = 0; i < target; i++) u = __dsub_rn(u, __dmul_rn(V[(long)i * npts + j], r[i]));
        U[j] = u;
        acc += u * u * W[j];
    }
    double s = block_sum(acc, sh);
    if (threadIdx.x == 0) npart[blockIdx.x] = s;
}

__global__ void __launch_bounds__(MT) mgs_normalize(double *__restrict__ V,
                                                    double *__restrict__ U,
                                                    const double *__restrict__ npart, int nblk,
                                                    int target, long npts, long chunk) {
    __shared__ double s_norm;
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int b = 0; b < nblk; b++) s += npart[b];
        s_norm = sqrt(s);
    }
    __syncthreads();
    const double nrm = s_norm;
    const long j0 = (long)blockIdx.x * chunk;
    const long j1 = min(j0 + chunk, npts);
    for (long j = j0 + threadIdx.x; j < j1; j += MT) {
        double u = U[j] / nrm;
        U[j] = u;
        V[(long)target * npts + j] = u;
    }
}

}  // namespace

int mgs_device(double *V, double *U, const double *W, int target, int npts, int nwave,
               cudaStream_t s) {
    if (npts <= 0) return TAGI_OK;
    if (target < 0 || target >= nwave)
        return set_error(TAGI_ERR_ARG, "targetWavefunction %d outside [0, %d)", target, nwave);
    int dev = 0, sms = 0;
    TAGI_CUDA(cudaGetDevice(&dev));
    TAGI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    long nblk = 4L * sms;
    long chunk = ((long)npts + nblk - 1) / nblk;
    chunk = ((chunk + MT - 1) / MT) * MT;
    nblk = ((long)npts + chunk - 1) / chunk;
    Arena tmp;
    tmp.stream = s;
    double *partial = nullptr, *r = nullptr, *npart = nullptr;
    int rc = TAGI_OK;
    do {
        if ((rc = tmp.alloc(&partial, (size_t)nblk * (target > 0 ? target : 1))) ||
            (rc = tmp.alloc(&r, target > 0 ? target : 1)) || (rc = tmp.alloc(&npart, nblk)))
            break;
        if (target > 0) {
            dim3 g((unsigned)nblk, (unsigned)((target + RB - 1) / RB));
            launch(mgs_dots, g, MT, 0, s, V, U, W, target, npts, chunk, partial);
            launch(mgs_reduce_rows, (target + 127) / 128, 128, 0, s, partial, (int)nblk, target, r);
        }
        launch(mgs_subtract, (unsigned)nblk, MT, 0, s, V, U, W, r, target, npts, chunk, npart);
        launch(mgs_normalize, (unsigned)nblk, MT, 0, s, V, U, npart, (int)nblk, target, npts, chunk);
        if (cudaGetLastError() != cudaSuccess) rc = set_error(TAGI_ERR_CUDA, "MGS kernels failed");
    } while (0);
    tmp.release();
    return rc;
}

}  // namespace tagi

// ---------------------------------------------------------------------------
// Weighted Gram-Schmidt without any device allocation.
//
// Some callers cannot allocate device memory while they run: a process whose
// device memory is handed entirely to another allocator (a framework's caching
// pool, a fixed per-job budget), or a latency-critical Green-iteration loop in
// which a cudaMalloc/cudaFree would synchronize the device and stall other
// streams.  tagi_mgs_dev_noalloc does the same work as tagi_mgs_dev with its
// scratch (per-block partial sums, projection coefficients, norm partials) in
// the fixed device array below instead of freshly allocated memory.
//
// * The array is MGS_NOALLOC_BLOCKS x (MGS_NOALLOC_ROWS + 1) + MGS_NOALLOC_ROWS
//   doubles (about 1.06 MB); every GPU that loads this library holds it until
//   the process exits.  Requests with targetWavefunction > MGS_NOALLOC_ROWS are
//   rejected with TAGI_ERR_ARG.
// * Host code cannot use the array's name as a device address: the first call
//   on each device (with that device current) looks the address up with
//   cudaGetSymbolAddress and keeps it.  Make that first call before any stream
//   capture.
// * All calls share the array and it keeps the last call's contents.  Every
//   entry a call reads is written earlier in the same call, so nothing needs
//   clearing; two calls that overlap on the GPU (different streams, or
//   different host threads on one device) race on it.
// ---------------------------------------------------------------------------
namespace tagi {
namespace {

constexpr int MGS_NOALLOC_BLOCKS = 1024;
constexpr int MGS_NOALLOC_ROWS = 128;
constexpr long MGS_NOALLOC_DOUBLES =
    (long)MGS_NOALLOC_BLOCKS * (MGS_NOALLOC_ROWS + 1) + MGS_NOALLOC_ROWS;

static __device__ __align__(256) double g_mgs_noalloc_scratch[MGS_NOALLOC_DOUBLES];

std::mutex g_mgs_noalloc_mu;
double *g_mgs_noalloc_ptr[64] = {};

int mgs_noalloc_scratch(double **out) {
    int dev = 0;
    TAGI_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_error(TAGI_ERR_DEVICE, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_mgs_noalloc_mu);
    if (!g_mgs_noalloc_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_mgs_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return set_error(TAGI_ERR_CUDA, "cudaGetSymbolAddress of the MGS scratch array failed: %s",
                             cudaGetErrorString(e));
        g_mgs_noalloc_ptr[dev] = static_cast<double *>(p);
    }
    *out = g_mgs_noalloc_ptr[dev];
    return TAGI_OK;
}

}  // namespace

}  // namespace tagi

extern "C" int tagi_mgs_dev_noalloc(double *V, double *U, const double *W, int targetWavefunction,
                                    int numPoints, int numWavefunctions, void *stream) {
    using namespace tagi;
    if (numPoints < 0 || numWavefunctions < 1) return set_error(TAGI_ERR_ARG, "bad MGS sizes");
    if (targetWavefunction < 0 || targetWavefunction >= numWavefunctions)
        return set_error(TAGI_ERR_ARG, "targetWavefunction %d outside [0, %d)", targetWavefunction,
                         numWavefunctions);
    if (targetWavefunction > MGS_NOALLOC_ROWS)
        return set_error(TAGI_ERR_ARG,
                         "tagi_mgs_dev_noalloc handles targetWavefunction <= %d (got %d); use tagi_mgs_dev",
                         MGS_NOALLOC_ROWS, targetWavefunction);
    if (numPoints == 0) return TAGI_OK;
    if (!V || !U || !W) return set_error(TAGI_ERR_ARG, "null device pointer");
    cudaStream_t s = (cudaStream_t)stream;
    double *scratch = nullptr;
    TAGI_TRY(mgs_noalloc_scratch(&scratch));
    int dev = 0, sms = 0;
    TAGI_CUDA(cudaGetDevice(&dev));
    TAGI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    long nblk = std::min(4L * sms, (long)MGS_NOALLOC_BLOCKS);
    long chunk = ((long)numPoints + nblk - 1) / nblk;
    chunk = ((chunk + MT - 1) / MT) * MT;
    nblk = ((long)numPoints + chunk - 1) / chunk;
    const int target = targetWavefunction;
    double *partial = scratch;                                   // [nblk][target]
    double *r = scratch + (long)MGS_NOALLOC_BLOCKS * MGS_NOALLOC_ROWS;   // [target]
    double *npart = r + MGS_NOALLOC_ROWS;                        // [nblk]
    if (target > 0) {
        dim3 g((unsigned)nblk, (unsigned)((target + RB - 1) / RB));
        launch(mgs_dots, g, MT, 0, s, V, U, W, target, (long)numPoints, chunk, partial);
        launch(mgs_reduce_rows, (target + 127) / 128, 128, 0, s, partial, (int)nblk, target, r);
    }
    launch(mgs_subtract, (unsigned)nblk, MT, 0, s, V, U, W, r, target, (long)numPoints, chunk, npart);
    launch(mgs_normalize, (unsigned)nblk, MT, 0, s, V, U, npart, (int)nblk, target, (long)numPoints, chunk);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

