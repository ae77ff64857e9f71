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
