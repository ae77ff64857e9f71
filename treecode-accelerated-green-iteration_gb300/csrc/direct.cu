// FP64 direct sum over all sources for a list of targets: the exact
// convolution (no tree), used to state the relative error of the treecode on
// seeded samples and as the O(N^2) plain path.  Same pair terms and
// singularity handling as the treecode (fields.cu).
#include "tagi_internal.h"

#include <cmath>

namespace tagi {

namespace {

constexpr int DT = 256;

template <int KERN, bool SS>
__global__ void __launch_bounds__(DT) direct_f64(int nsub, const int *__restrict__ sub,
                                                 const double *__restrict__ tx,
                                                 const double *__restrict__ ty,
                                                 const double *__restrict__ tz,
                                                 const double *__restrict__ tv, int ns,
                                                 const double *__restrict__ sx,
                                                 const double *__restrict__ sy,
                                                 const double *__restrict__ sz,
                                                 const double *__restrict__ sv,
                                                 const double *__restrict__ sw, double kp,
                                                 double ssc, double *__restrict__ out) {
    __shared__ double s_x[DT], s_y[DT], s_z[DT], s_f[DT], s_w[DT];
    const int q = blockIdx.x * DT + threadIdx.x;
    const bool v = q < nsub;
    const int i = v ? (sub ? sub[q] : q) : 0;
    const double xi = tx[i], yi = ty[i], zi = tz[i], fi = tv[i];
    double acc = 0.0;
    for (int t0 = 0; t0 < ns; t0 += DT) {
        const int cnt = min(DT, ns - t0);
        __syncthreads();
        if (threadIdx.x < cnt) {
            int j = t0 + threadIdx.x;
            s_x[threadIdx.x] = sx[j];
            s_y[threadIdx.x] = sy[j];
            s_z[threadIdx.x] = sz[j];
            s_f[threadIdx.x] = sv[j];
            s_w[threadIdx.x] = sw[j];
        }
        __syncthreads();
        for (int j = 0; j < cnt; j++) {
            double dx = xi - s_x[j], dy = yi - s_y[j], dz = zi - s_z[j];
            double r2 = dx * dx + dy * dy + dz * dz;
            if (!(r2 > 0.0)) continue;
            double r = sqrt(r2);
            if (KERN == KERNEL_YUKAWA) {
                double g = exp(-kp * r) / r;
                acc += SS ? s_w[j] * (s_f[j] - fi) * g : s_w[j] * s_f[j] * g;
            } else {
                acc += SS ? s_w[j] * (s_f[j] - fi * exp(-kp * kp * r2)) / r : s_w[j] * s_f[j] / r;
            }
        }
    }
    if (v) out[q] = acc + ssc * fi;
}

}  // namespace

int direct_sum(int nt, const double *tx, const double *ty, const double *tz, const double *tv,
               int nsub, const int *sub, int ns, const double *sx, const double *sy,
               const double *sz, const double *sv, const double *sw, double *out, int kernel,
               double kp, int singularity, int precision, cudaStream_t s) {
    (void)nt;
    (void)precision;
    if (nsub <= 0) return TAGI_OK;
    const bool ss = singularity == SING_SUBTRACTION;
    double ssc = 0.0;
    if (ss) ssc = kernel == KERNEL_YUKAWA ? 4.0 * M_PI / (kp * kp) : 2.0 * M_PI / (kp * kp);
    const int grid = (nsub + DT - 1) / DT;
    if (kernel == KERNEL_YUKAWA) {
        if (ss) launch(direct_f64<KERNEL_YUKAWA, true>, grid, DT, 0, s, nsub, sub, tx, ty, tz, tv, ns, sx, sy, sz, sv, sw, kp, ssc, out);
        else launch(direct_f64<KERNEL_YUKAWA, false>, grid, DT, 0, s, nsub, sub, tx, ty, tz, tv, ns, sx, sy, sz, sv, sw, kp, ssc, out);
    } else {
        if (ss) launch(direct_f64<KERNEL_COULOMB, true>, grid, DT, 0, s, nsub, sub, tx, ty, tz, tv, ns, sx, sy, sz, sv, sw, kp, ssc, out);
        else launch(direct_f64<KERNEL_COULOMB, false>, grid, DT, 0, s, nsub, sub, tx, ty, tz, tv, ns, sx, sy, sz, sv, sw, kp, ssc, out);
    }
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

}  // namespace tagi
