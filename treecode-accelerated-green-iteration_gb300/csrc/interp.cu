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
// One CTA per interpolated cell, coarse values staged in shared memory; fine
// points on tensor grids (the mesh builders' layout) take a sum-factorised
// path, any other point the reference's per-point formula (see interp_cells).
#include "tagi_internal.h"

#include <cfloat>
#include <cmath>

namespace tagi {

namespace {

constexpr int IT = 256;
constexpr int MAXP1 = 12;

// One fine point by the reference's formula (TwoMeshInterpolation.c:59-147):
// per-axis barycentric terms w_k / (t - node_k), the exact-node guard with its
// swapped x/z index tests, the tensor sum with y innermost, times the
// product of the inverse sums.
__device__ double interp_point(double tx, double ty, double tz, const double *s_c, const double *s_nx,
                               const double *s_ny, const double *s_nz, const double *s_w, int p1) {
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
    return temp * den;
}

// One CTA per interpolated cell.  A cell's fine points come in blocks of
// (p+1)^3 (one block per child cell).  When a block is a tensor grid in
// x-major order (x depends on the block index i only, y on j, z on k -- the
// layout the mesh builders write) and none of its 1-D coordinates sits on a
// coarse node, the interpolant is the sum-factorised product
//     out[a][b][c] = sum_i Lx[a][i] sum_j Ly[b][j] sum_k Lz[c][k] F[i][j][k],
//     Lx[a][i] = (w_i / (x_a - xn_i)) / sum_i' (w_i' / (x_a - xn_i'))
// (three 1-D contractions: 3 (p+1)^4 multiply-adds per block instead of
// ~(p+1)^6); otherwise every point of the block takes the reference's
// per-point formula (interp_point).  Both agree to rounding.
__global__ void __launch_bounds__(IT) interp_cells(
    const double *__restrict__ cX, const double *__restrict__ cY, const double *__restrict__ cZ,
    const double *__restrict__ cF, const int *__restrict__ ppc_c, const int *__restrict__ off_c,
    const double *__restrict__ fX, const double *__restrict__ fY, const double *__restrict__ fZ,
    double *__restrict__ fF, const int *__restrict__ ppc_f, const int *__restrict__ off_f, int p1,
    const double *__restrict__ wts, int *__restrict__ err) {
    constexpr int MAXP3 = MAXP1 * MAXP1 * MAXP1;
    __shared__ double s_c[MAXP3];
    __shared__ double s_t[2][MAXP3];                // contraction stages
    __shared__ double s_L[3][MAXP1 * MAXP1];        // Lx, Ly, Lz: [fine index][node]
    __shared__ double s_f[3][MAXP1];                // the block's 1-D fine coordinates
    __shared__ double s_nx[MAXP1], s_ny[MAXP1], s_nz[MAXP1], s_w[MAXP1];
    const int cell = blockIdx.x;
    const int nc = ppc_c[cell], nf = ppc_f[cell];
    const int c0 = off_c[cell], f0 = off_f[cell];
    const int tid = threadIdx.x;
    if (nc == nf) {
        for (int j = tid; j < nf; j += IT) fF[f0 + j] = fF[f0 + j] + cF[c0 + j];
        return;
    }
    const int p2 = p1 * p1, p3 = p2 * p1;
    if (nc != p3) {  // a coarse cell must hold the full (p+1)^3 grid
        if (tid == 0) atomicOr(err, 1);
        return;
    }
    for (int j = tid; j < nc; j += IT) s_c[j] = cF[c0 + j];
    if (tid < p1) {
        const int i = tid;
        s_nx[i] = cX[c0 + i * p2];
        s_ny[i] = cY[c0 + i * p1];
        s_nz[i] = cZ[c0 + i];
        s_w[i] = wts[i];
    }
    __syncthreads();
    const int nblk = nf / p3, rest = nf - nblk * p3;
    for (int blk = 0; blk < nblk; blk++) {
        const int b0 = f0 + blk * p3;
        // tensor-grid check (bitwise) and exact-node check on the 1-D coordinates
        if (tid < 3 * p1) {
            const int d = tid / p1, m = tid - d * p1;
            s_f[d][m] = d == 0 ? fX[b0 + m * p2] : (d == 1 ? fY[b0 + m * p1] : fZ[b0 + m]);
        }
        __syncthreads();
        int bad = 0;
        for (int q = tid; q < p3; q += IT) {
            const int i = q / p2, j = (q / p1) % p1, k = q % p1;
            bad |= __double_as_longlong(fX[b0 + q]) != __double_as_longlong(s_f[0][i]);
            bad |= __double_as_longlong(fY[b0 + q]) != __double_as_longlong(s_f[1][j]);
            bad |= __double_as_longlong(fZ[b0 + q]) != __double_as_longlong(s_f[2][k]);
        }
        if (tid < 3 * p1) {
            const int d = tid / p1, m = tid - d * p1;
            const double *nodes = d == 0 ? s_nx : (d == 1 ? s_ny : s_nz);
            for (int k = 0; k < p1; k++) bad |= fabs(s_f[d][m] - nodes[k]) < DBL_MIN;
        }
        if (__syncthreads_or(bad)) {
            for (int q = tid; q < p3; q += IT)
                fF[b0 + q] = fF[b0 + q] + interp_point(fX[b0 + q], fY[b0 + q], fZ[b0 + q], s_c, s_nx, s_ny, s_nz,
                                                       s_w, p1);
            __syncthreads();
            continue;
        }
        // normalised 1-D barycentric rows
        if (tid < 3 * p1) {
            const int d = tid / p1, m = tid - d * p1;
            const double *nodes = d == 0 ? s_nx : (d == 1 ? s_ny : s_nz);
            double sum = 0.0, a[MAXP1];
            for (int k = 0; k < p1; k++) {
                a[k] = s_w[k] / (s_f[d][m] - nodes[k]);
                sum += a[k];
            }
            for (int k = 0; k < p1; k++) s_L[d][m * p1 + k] = a[k] / sum;
        }
        __syncthreads();
        // T1[i][j][c] = sum_k Lz[c][k] F[i][j][k]
        for (int q = tid; q < p3; q += IT) {
            const int ij = q / p1, c = q - ij * p1;
            double v = 0.0;
            for (int k = 0; k < p1; k++) v += s_L[2][c * p1 + k] * s_c[ij * p1 + k];
            s_t[0][q] = v;
        }
        __syncthreads();
        // T2[i][b][c] = sum_j Ly[b][j] T1[i][j][c]
        for (int q = tid; q < p3; q += IT) {
            const int i = q / p2, bc = q - i * p2, bb = bc / p1, c = bc - bb * p1;
            double v = 0.0;
            for (int j = 0; j < p1; j++) v += s_L[1][bb * p1 + j] * s_t[0][i * p2 + j * p1 + c];
            s_t[1][q] = v;
        }
        __syncthreads();
        // out[a][b][c] = sum_i Lx[a][i] T2[i][b][c]
        for (int q = tid; q < p3; q += IT) {
            const int aa = q / p2, bc = q - aa * p2;
            double v = 0.0;
            for (int i = 0; i < p1; i++) v += s_L[0][aa * p1 + i] * s_t[1][i * p2 + bc];
            fF[b0 + q] = fF[b0 + q] + v;
        }
        __syncthreads();
    }
    // points past the last whole block (a cell whose fine count is not a multiple of (p+1)^3)
    for (int q = tid; q < rest; q += IT) {
        const int g = f0 + nblk * p3 + q;
        fF[g] = fF[g] + interp_point(fX[g], fY[g], fZ[g], s_c, s_nx, s_ny, s_nz, s_w, p1);
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
