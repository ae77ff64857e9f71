// Subsystem (e), part 2: cell-wise Chebyshev interpolation between two
// meshes, the device counterpart of InterpolateBetweenTwoMeshes /
// interapolateBetweenTwoMeshesSingleCell
// (3D-GreenIteration/src/utilities/TwoMeshInterpolation.c:12-153,163-234), FP64.
//
// Semantics kept from the reference:
//  * coarseN == fineN: fineF = coarseF (overwrite) and nothing else   :175-180
//  * a cell whose coarse and fine counts match adds coarseF to fineF  :202-205,228-230
//  * otherwise fineF += barycentric interpolant of the coarse cell      :147
//  * nodes are read from the coarse cell assuming x-major order        :40-44
//  * first-kind weights (-1)^i sin((2i+1) pi / (2p+2))                 :49-51
//  * exact-node guard |t - node| < DBL_MIN; as in the reference, the x and z
//    exact-node tests compare against the z and x loop indices (:127,:139)
// One CTA per interpolated cell, coarse values staged in shared memory; each
// fine point evaluates the tensor-product sum with the y direction innermost.
#include "tagi_internal.h"

#include <cfloat>
#include <cmath>

namespace tagi {

namespace {

constexpr int IT = 256;
constexpr int MAXP1 = 12;

__global__ void __launch_bounds__(IT) interp_cells(
    const double *__restrict__ cX, const double *__restrict__ cY, const double *__restrict__ cZ,
    const double *__restrict__ cF, const int *__restrict__ ppc_c, const int *__restrict__ off_c,
    const double *__restrict__ fX, const double *__restrict__ fY, const double *__restrict__ fZ,
    double *__restrict__ fF, const int *__restrict__ ppc_f, const int *__restrict__ off_f, int p1,
    const double *__restrict__ wts, int *__restrict__ err) {
    __shared__ double s_c[MAXP1 * MAXP1 * MAXP1];
    __shared__ double s_nx[MAXP1], s_ny[MAXP1], s_nz[MAXP1], s_w[MAXP1];
    const int cell = blockIdx.x;
    const int nc = ppc_c[cell], nf = ppc_f[cell];
    const int c0 = off_c[cell], f0 = off_f[cell];
    if (nc == nf) {
        for (int j = threadIdx.x; j < nf; j += IT) fF[f0 + j] = fF[f0 + j] + cF[c0 + j];
        return;
    }
    if (nc != p1 * p1 * p1) {  // a coarse cell must hold the full (p+1)^3 grid
        if (threadIdx.x == 0) atomicOr(err, 1);
        return;
    }
    for (int j = threadIdx.x; j < nc; j += IT) s_c[j] = cF[c0 + j];
    if (threadIdx.x < p1) {
        int i = threadIdx.x;
        s_nx[i] = cX[c0 + i * p1 * p1];
        s_ny[i] = cY[c0 + i * p1];
        s_nz[i] = cZ[c0 + i];
        s_w[i] = wts[i];
    }
    __syncthreads();
    for (int q = threadIdx.x; q < nf; q += IT) {
        const double tx = fX[f0 + q], ty = fY[f0 + q], tz = fZ[f0 + q];
        double sx = 0.0, sy = 0.0, sz = 0.0;
        int eix = -1, eiy = -1, eiz = -1;
        double ax[MAXP1], ay[MAXP1], az[MAXP1];
        for (int k = 0; k < p1; k++) {
            const double dx = tx - s_nx[k], dy = ty - s_ny[k], dz = tz - s_nz[k];
            if (fabs(dx) < DBL_MIN) eix = k;
            if (fabs(dy) < DBL_MIN) eiy = k;
            if (fabs(dz) < DBL_MIN) eiz = k;
            ax[k] = s_w[k] / dx;
            ay[k] = s_w[k] / dy;
            az[k] = s_w[k] / dz;
            sx += ax[k];
            sy += ay[k];
            sz += az[k];
        }
        double den = 1.0;
        if (eix == -1) den /= sx;
        if (eiy == -1) den /= sy;
        if (eiz == -1) den /= sz;
        // y factor depends on k2 only; x and z factors as in the reference.
        for (int k = 0; k < p1; k++) ay[k] = (eiy == -1) ? ay[k] : (eiy == k ? 1.0 : 0.0);
        double temp = 0.0;
        for (int k3 = 0; k3 < p1; k3++) {
            for (int k1 = 0; k1 < p1; k1++) {
                const double fx = (eix == -1) ? ax[k3] : (eix == k1 ? 1.0 : 0.0);
                const double fz = (eiz == -1) ? az[k1] : (eiz == k3 ? 1.0 : 0.0);
                const double fxz = fx * fz;
                if (fxz == 0.0) continue;
                const double *col = s_c + k3 * p1 * p1 + k1;
                double g = 0.0;
                for (int k2 = 0; k2 < p1; k2++) g += ay[k2] * col[k2 * p1];
                temp += fxz * g;
            }
        }
        fF[f0 + q] = fF[f0 + q] + temp * den;
    }
}

__global__ void copy_all(const double *__restrict__ a, double *__restrict__ b, long n) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = a[i];
}

}  // namespace

int interp_device(const double *cX, const double *cY, const double *cZ, const double *cF,
                  const int *ppc_c, int coarseN, const double *fX, const double *fY,
                  const double *fZ, double *fF, const int *ppc_f, int fineN, int ncells,
                  int order, const int *h_ppc_c, const int *h_ppc_f, cudaStream_t s) {
    (void)h_ppc_c;
    (void)h_ppc_f;
    if (coarseN == fineN) {
        if (coarseN > 0) launch(copy_all, (coarseN + 255) / 256, 256, 0, s, cF, fF, coarseN);
        TAGI_LAUNCH_CHECK();
        return TAGI_OK;
    }
    const int p1 = order + 1;
    if (p1 < 1 || p1 > MAXP1)
        return set_error(TAGI_ERR_UNSUPPORTED, "interpolation order %d outside [0, %d]", order, MAXP1 - 1);
    if (ncells <= 0) return TAGI_OK;
    double w[MAXP1];
    for (int i = 0; i < p1; i++)
        w[i] = pow(-1, i) * sin((2 * i + 1) * M_PI / (2 * (p1 - 1) + 2));
    Arena tmp;
    tmp.stream = s;
    int *off_c = nullptr, *off_f = nullptr, *err = nullptr;
    double *d_w = nullptr;
    int rc = TAGI_OK;
    do {
        if ((rc = tmp.alloc(&off_c, ncells + 1)) || (rc = tmp.alloc(&off_f, ncells + 1)) ||
            (rc = tmp.alloc(&d_w, MAXP1)) || (rc = tmp.alloc(&err, 1)))
            break;
        cudaMemsetAsync(err, 0, sizeof(int), s);
        if ((rc = exclusive_scan(ppc_c, off_c, ncells, off_c + ncells, tmp, s))) break;
        if ((rc = exclusive_scan(ppc_f, off_f, ncells, off_f + ncells, tmp, s))) break;
        int tot[2] = {0, 0};
        if (cudaMemcpyAsync(&tot[0], off_c + ncells, sizeof(int), cudaMemcpyDeviceToHost, s) ||
            cudaMemcpyAsync(&tot[1], off_f + ncells, sizeof(int), cudaMemcpyDeviceToHost, s) ||
            cudaStreamSynchronize(s)) {
            rc = set_error(TAGI_ERR_CUDA, "interpolation offsets copy failed");
            break;
        }
        if (tot[0] > coarseN || tot[1] > fineN) {
            rc = set_error(TAGI_ERR_ARG, "points per cell sum to %d coarse / %d fine, arrays hold %d / %d",
                           tot[0], tot[1], coarseN, fineN);
            break;
        }
        if (cudaMemcpyAsync(d_w, w, sizeof(double) * p1, cudaMemcpyHostToDevice, s) != cudaSuccess) {
            rc = set_error(TAGI_ERR_CUDA, "interpolation weight upload failed");
            break;
        }
        launch(interp_cells, ncells, IT, 0, s, cX, cY, cZ, cF, ppc_c, off_c, fX, fY, fZ, fF, ppc_f, off_f,
                                           p1, d_w, err);
        int h_err = 0;
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            rc = set_error(TAGI_ERR_CUDA, "interpolation kernel failed");
            break;
        }
        if (h_err) rc = set_error(TAGI_ERR_ARG, "an interpolated coarse cell does not hold (order+1)^3 points");
    } while (0);
    tmp.release();
    return rc;
}

}  // namespace tagi
