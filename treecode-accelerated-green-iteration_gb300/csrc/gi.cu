// Green-iteration and SCF pieces around the convolution, on the device, so a
// whole Green-iteration sweep (all orbitals) is one stream of launches that
// can be captured as one CUDA graph.  Reference steps (3D-GreenIteration/src):
//   f_m = -2 psi_m V_eff                                greenIterationFixedPoint.py:155
//   k_m = sqrt(-2 eps_m)                                 :207
//   psi_new = (1/4pi) G_k * f  (Yukawa, subtraction)     :314-324
//   dE = -<psi V_eff (psi - psi_new)>_W / <psi_new^2>_W  :373-398
//   eps += dE; psi <- psi_new; Gram-Schmidt              :399-432
//   eps > 0  ->  eps = gaugeShift - 3 rand               :470-477 (here a fixed gaugeShift - 1.5)
//   residual = |(psi, eps)_out - (psi, eps)_in| with weights (W, 1)
//                                                        scfFixedPoint.py:62-67, greenIterationFixedPoint.py:484
//   rho = sum_m occ_m psi_m^2, scaled to N electrons     scfFixedPoint.py:624-636
//   Slater exchange (LDA, unpolarized), V_eff assembly   scfFixedPoint.py:332-345
//   Anderson mixing: F_k = out_k - in_k, linear system of
//   weighted dots, next = b * out_mix + (1 - b) * in_mix densityMixingSchemes.py:30-97
//
// All arithmetic is FP64.  Every reduction is a fixed number of per-block
// partial sums (set by n alone) added in block order, so results do not
// depend on the GPU or on scheduling.  No entry point allocates: callers pass
// a workspace (tagi_gi_workspace_doubles gives its size).
#include "tagi_internal.h"

#include <cmath>

namespace tagi {

namespace {

constexpr int GT = 256;
constexpr long GI_CHUNK_MIN = 4096;  // points per partial block, at least
constexpr int GI_MAX_BLOCKS = 1024;

__device__ __forceinline__ double block_sum(double v, double *sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < GT / 32; w++) s += sh[w];
    return s;  // valid in thread 0
}

struct Chunks {
    long chunk;
    int nblk;
};

Chunks chunks_for(long n) {
    long nb = (n + GI_CHUNK_MIN - 1) / GI_CHUNK_MIN;
    if (nb > GI_MAX_BLOCKS) nb = GI_MAX_BLOCKS;
    if (nb < 1) nb = 1;
    long chunk = (n + nb - 1) / nb;
    chunk = ((chunk + GT - 1) / GT) * GT;
    nb = (n + chunk - 1) / chunk;
    return {chunk, (int)(nb < 1 ? 1 : nb)};
}

__global__ void gi_source(const double *__restrict__ psi, const double *__restrict__ veff, long n,
                          double *__restrict__ f) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long o = (long)blockIdx.y * n + i;
    f[o] = -2.0 * psi[o] * veff[i];
}

// Per orbital (blockIdx.y) and chunk: num = sum w psi V (psi - s c),
// den = sum w (s c)^2; psi <- s c.
__global__ void __launch_bounds__(GT) gi_update_partial(double *__restrict__ psi, const double *__restrict__ conv,
                                                        const double *__restrict__ veff,
                                                        const double *__restrict__ w, long n, long chunk, double s,
                                                        int nblk, double *__restrict__ part) {
    __shared__ double sh[GT / 32];
    const long base = (long)blockIdx.y * n;
    const long j0 = (long)blockIdx.x * chunk, j1 = min(j0 + chunk, n);
    double num = 0.0, den = 0.0;
    for (long j = j0 + threadIdx.x; j < j1; j += GT) {
        const double p = psi[base + j], q = s * conv[base + j], wj = w[j];
        num += wj * p * veff[j] * (p - q);
        den += wj * q * q;
        psi[base + j] = q;
    }
    const double a = block_sum(num, sh);
    const double b = block_sum(den, sh);
    if (threadIdx.x == 0) {
        part[((long)blockIdx.y * nblk + blockIdx.x) * 2] = a;
        part[((long)blockIdx.y * nblk + blockIdx.x) * 2 + 1] = b;
    }
}

__global__ void gi_update_final(const double *__restrict__ part, int nblk, int norb, double *__restrict__ eps,
                                double *__restrict__ eps_prev, double *__restrict__ k, double gauge,
                                double *__restrict__ dE, int *__restrict__ flags) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= norb) return;
    double num = 0.0, den = 0.0;
    for (int b = 0; b < nblk; b++) {
        num += part[((long)m * nblk + b) * 2];
        den += part[((long)m * nblk + b) * 2 + 1];
    }
    const double d = -num / den;
    const double e0 = eps[m];
    double e = e0 + d;
    if (!(e < 0.0)) {  // positive (or NaN) eigenvalue: back below the gauge shift
        e = gauge - 1.5;
        flags[m] = 1;
    } else {
        flags[m] = 0;
    }
    eps_prev[m] = e0;
    eps[m] = e;
    dE[m] = d;
    k[m] = sqrt(-2.0 * e);
}

// out[r] partials: sum_i w_i a[r][i] b[r][i]  (b_stride 0: one vector b for all
// rows; b == nullptr: b = 1, a weighted sum; w == nullptr: w = 1)
__global__ void __launch_bounds__(GT) wdot_partial(const double *__restrict__ a, long a_stride,
                                                   const double *__restrict__ b, long b_stride,
                                                   const double *__restrict__ w, long n, long chunk, int nblk,
                                                   double *__restrict__ part) {
    __shared__ double sh[GT / 32];
    const int r = blockIdx.y;
    const double *ar = a + (long)r * a_stride;
    const double *br = b ? b + (long)r * b_stride : nullptr;
    const long j0 = (long)blockIdx.x * chunk, j1 = min(j0 + chunk, n);
    double acc = 0.0;
    for (long j = j0 + threadIdx.x; j < j1; j += GT) acc += (w ? w[j] : 1.0) * ar[j] * (br ? br[j] : 1.0);
    const double s = block_sum(acc, sh);
    if (threadIdx.x == 0) part[(long)r * nblk + blockIdx.x] = s;
}

__global__ void wdot_final(const double *__restrict__ part, int nblk, int rows, double *__restrict__ out) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    double s = 0.0;
    for (int b = 0; b < nblk; b++) s += part[(long)r * nblk + b];
    out[r] = s;
}

// residual partials: sum w (psi - prev)^2 per orbital
__global__ void __launch_bounds__(GT) gi_residual_partial(const double *__restrict__ psi,
                                                          const double *__restrict__ prev,
                                                          const double *__restrict__ w, long n, long chunk,
                                                          int nblk, double *__restrict__ part) {
    __shared__ double sh[GT / 32];
    const long base = (long)blockIdx.y * n;
    const long j0 = (long)blockIdx.x * chunk, j1 = min(j0 + chunk, n);
    double acc = 0.0;
    for (long j = j0 + threadIdx.x; j < j1; j += GT) {
        const double d = psi[base + j] - prev[base + j];
        acc += w[j] * d * d;
    }
    const double s = block_sum(acc, sh);
    if (threadIdx.x == 0) part[(long)blockIdx.y * nblk + blockIdx.x] = s;
}

__global__ void gi_residual_final(const double *__restrict__ part, int nblk, int norb, const double *__restrict__ eps,
                                  const double *__restrict__ eps_prev, double *__restrict__ res,
                                  double *__restrict__ psi_res) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= norb) return;
    double s = 0.0;
    for (int b = 0; b < nblk; b++) s += part[(long)m * nblk + b];
    const double de = eps[m] - eps_prev[m];
    psi_res[m] = sqrt(s);
    res[m] = sqrt(s + de * de);
}

__global__ void scf_density(const double *__restrict__ psi, const double *__restrict__ occ, int norb, long n,
                            double *__restrict__ rho) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double r = 0.0;
    for (int m = 0; m < norb; m++) {
        const double p = psi[(long)m * n + i];
        r += occ[m] * p * p;
    }
    rho[i] = r;
}

// x *= target / (*integral)
__global__ void scale_to(double *__restrict__ x, long n, double target, const double *__restrict__ integral) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    x[i] *= target / *integral;
}

// Slater exchange, spin-unpolarized LDA: e_x = -(3/4)(3/pi)^(1/3) rho^(1/3) per
// electron, v_x = d(rho e_x)/d rho = -(3/pi)^(1/3) rho^(1/3).
__global__ void lda_exchange(const double *__restrict__ rho, long n, double *__restrict__ vx,
                             double *__restrict__ ex) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double c = cbrt(3.0 / M_PI);
    const double r = rho[i] > 0.0 ? cbrt(rho[i]) : 0.0;
    vx[i] = -c * r;
    ex[i] = -0.75 * c * r;
}

__global__ void veff_assemble(const double *__restrict__ vh, const double *__restrict__ vx,
                              const double *__restrict__ vext, double gauge, long n, double *__restrict__ veff) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    veff[i] = vh[i] + vx[i] + vext[i] + gauge;
}

// Anderson combination of nh history rows (ring buffers [H][n]; row `last` is
// the newest): mix_in = in_last + sum_k c_k (in_k' - in_last) over the other
// rows k' in age order, the same for out; next = b mix_out + (1 - b) mix_in.
// rows[k] gives the ring row of the k-th older entry (k = 0 newest-but-one).
__global__ void anderson_combine(const double *__restrict__ in_hist, const double *__restrict__ out_hist, int nh,
                                 int last, const int *__restrict__ rows, const double *__restrict__ c, double beta,
                                 long n, double *__restrict__ next) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double il = in_hist[(long)last * n + i], ol = out_hist[(long)last * n + i];
    double mi = il, mo = ol;
    for (int k = 0; k < nh - 1; k++) {
        const long r = (long)rows[k] * n + i;
        mi += c[k] * (in_hist[r] - il);
        mo += c[k] * (out_hist[r] - ol);
    }
    next[i] = beta * mo + (1.0 - beta) * mi;
}

// Anderson mixing of each orbital's (psi, eps) over its last H sweeps
// (scfFixedPoint.py:483-597 does it orbital by orbital; here all orbitals at
// once).  F = out - in rows, layout [H][norb][n].  Gram partials of every
// pair a <= b of history rows, per orbital and chunk, in a fixed order.
constexpr int AND_MAXH = 8;

__global__ void __launch_bounds__(GT) anderson_gram_partial(const double *__restrict__ F, int H, int norb, long n,
                                                            const double *__restrict__ w, long chunk, int nblk,
                                                            double *__restrict__ part) {
    __shared__ double sh[GT / 32];
    const int m = blockIdx.y;
    const long j0 = (long)blockIdx.x * chunk, j1 = min(j0 + chunk, n);
    constexpr int NP = AND_MAXH * (AND_MAXH + 1) / 2;
    double acc[NP];
#pragma unroll
    for (int p = 0; p < NP; p++) acc[p] = 0.0;
    for (long j = j0 + threadIdx.x; j < j1; j += GT) {
        double f[AND_MAXH];
#pragma unroll
        for (int a = 0; a < AND_MAXH; a++) f[a] = a < H ? F[((long)a * norb + m) * n + j] : 0.0;
        const double wj = w[j];
        int p = 0;
#pragma unroll
        for (int a = 0; a < AND_MAXH; a++)
#pragma unroll
            for (int b = a; b < AND_MAXH; b++) acc[p++] += wj * f[a] * f[b];
    }
    const int np = H * (H + 1) / 2;
    int p = 0;
#pragma unroll
    for (int a = 0; a < AND_MAXH; a++)
#pragma unroll
        for (int b = a; b < AND_MAXH; b++, p++) {
            if (a >= H || b >= H) continue;
            const double t = block_sum(acc[p], sh);
            // pair index among the first H rows, in the same (a, b) order
            const int q = a * H - a * (a - 1) / 2 + (b - a);
            if (threadIdx.x == 0) part[((long)m * nblk + blockIdx.x) * np + q] = t;
        }
}

__global__ void anderson_gram_final(const double *__restrict__ part, int nblk, int norb, int np,
                                    double *__restrict__ gram) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= norb * np) return;
    const int m = i / np, q = i - m * np;
    double s = 0.0;
    for (int b = 0; b < nblk; b++) s += part[((long)m * nblk + b) * np + q];
    gram[i] = s;
}

// psi[m] = x_l + sum_k c_mk (x_k - x_l) + beta (F_l + sum_k c_mk (F_k - F_l))
__global__ void anderson_mix(const double *__restrict__ X, const double *__restrict__ F, int nh, int last,
                             const int *__restrict__ rows, const double *__restrict__ c, double beta, int norb,
                             long n, double *__restrict__ psi) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int m = blockIdx.y;
    const long ol = ((long)last * norb + m) * n + i;
    const double xl = X[ol], fl = F[ol];
    double xm = xl, fm = fl;
    for (int k = 0; k < nh - 1; k++) {
        const long o = ((long)rows[k] * norb + m) * n + i;
        const double ck = c[(long)m * (nh - 1) + k];
        xm += ck * (X[o] - xl);
        fm += ck * (F[o] - fl);
    }
    psi[(long)m * n + i] = xm + beta * fm;
}

}  // namespace

}  // namespace tagi

using namespace tagi;

extern "C" {

long long tagi_gi_workspace_doubles(long long numPoints, int rows) {
    const Chunks c = chunks_for(numPoints > 0 ? numPoints : 1);
    return (long long)c.nblk * (rows > 0 ? rows : 1) * 2 + 64;
}

int tagi_gi_source(const double *psi, const double *veff, long long numPoints, int numOrbitals, double *f,
                   void *stream) {
    if (!psi || !veff || !f) return set_error(TAGI_ERR_ARG, "null pointer");
    if (numPoints <= 0 || numOrbitals <= 0 || numOrbitals > 65535) return set_error(TAGI_ERR_ARG, "bad sizes");
    dim3 g((unsigned)((numPoints + 255) / 256), numOrbitals);
    launch(gi_source, g, 256, 0, (cudaStream_t)stream, psi, veff, (long)numPoints, f);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

int tagi_gi_update(double *psi, const double *conv, const double *veff, const double *weights, long long numPoints,
                   int numOrbitals, double convScale, double *eps, double *epsPrev, double *k, double gaugeShift,
                   double *deltaE, int *flags, double *work, long long workDoubles, void *stream) {
    if (!psi || !conv || !veff || !weights || !eps || !epsPrev || !k || !deltaE || !flags || !work)
        return set_error(TAGI_ERR_ARG, "null pointer");
    if (numPoints <= 0 || numOrbitals <= 0 || numOrbitals > 65535) return set_error(TAGI_ERR_ARG, "bad sizes");
    const Chunks c = chunks_for(numPoints);
    if (workDoubles < tagi_gi_workspace_doubles(numPoints, numOrbitals))
        return set_error(TAGI_ERR_ARG, "workspace of %lld doubles, %lld needed", workDoubles,
                         tagi_gi_workspace_doubles(numPoints, numOrbitals));
    cudaStream_t s = (cudaStream_t)stream;
    launch(gi_update_partial, dim3(c.nblk, numOrbitals), GT, 0, s, psi, conv, veff, weights, (long)numPoints, c.chunk,
           convScale, c.nblk, work);
    launch(gi_update_final, (numOrbitals + 63) / 64, 64, 0, s, work, c.nblk, numOrbitals, eps, epsPrev, k,
           gaugeShift, deltaE, flags);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

int tagi_gi_residual(const double *psi, const double *psiPrev, const double *weights, long long numPoints,
                     int numOrbitals, const double *eps, const double *epsPrev, double *residual,
                     double *psiResidual, double *work, long long workDoubles, void *stream) {
    if (!psi || !psiPrev || !weights || !eps || !epsPrev || !residual || !psiResidual || !work)
        return set_error(TAGI_ERR_ARG, "null pointer");
    if (numPoints <= 0 || numOrbitals <= 0 || numOrbitals > 65535) return set_error(TAGI_ERR_ARG, "bad sizes");
    const Chunks c = chunks_for(numPoints);
    if (workDoubles < tagi_gi_workspace_doubles(numPoints, numOrbitals))
        return set_error(TAGI_ERR_ARG, "workspace too small");
    cudaStream_t s = (cudaStream_t)stream;
    launch(gi_residual_partial, dim3(c.nblk, numOrbitals), GT, 0, s, psi, psiPrev, weights, (long)numPoints, c.chunk,
           c.nblk, work);
    launch(gi_residual_final, (numOrbitals + 63) / 64, 64, 0, s, work, c.nblk, numOrbitals, eps, epsPrev, residual,
           psiResidual);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

int tagi_wdot_rows(const double *a, long long aStride, const double *b, long long bStride, const double *weights,
                   long long numPoints, int rows, double *out, double *work, long long workDoubles, void *stream) {
    if (!a || !out || !work) return set_error(TAGI_ERR_ARG, "null pointer");
    if (numPoints <= 0 || rows <= 0 || rows > 65535) return set_error(TAGI_ERR_ARG, "bad sizes");
    const Chunks c = chunks_for(numPoints);
    if (workDoubles < tagi_gi_workspace_doubles(numPoints, rows)) return set_error(TAGI_ERR_ARG, "workspace too small");
    cudaStream_t s = (cudaStream_t)stream;
    launch(wdot_partial, dim3(c.nblk, rows), GT, 0, s, a, (long)aStride, b, (long)bStride, weights, (long)numPoints,
           c.chunk, c.nblk, work);
    launch(wdot_final, (rows + 63) / 64, 64, 0, s, work, c.nblk, rows, out);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

int tagi_scf_density(const double *psi, const double *occupations, int numOrbitals, long long numPoints,
                     const double *weights, double numElectrons, double *rho, double *work, long long workDoubles,
                     void *stream) {
    if (!psi || !occupations || !rho || !weights || !work) return set_error(TAGI_ERR_ARG, "null pointer");
    if (numPoints <= 0 || numOrbitals <= 0) return set_error(TAGI_ERR_ARG, "bad sizes");
    if (workDoubles < tagi_gi_workspace_doubles(numPoints, 1) + 1) return set_error(TAGI_ERR_ARG, "workspace too small");
    cudaStream_t s = (cudaStream_t)stream;
    const unsigned g = (unsigned)((numPoints + 255) / 256);
    launch(scf_density, g, 256, 0, s, psi, occupations, numOrbitals, (long)numPoints, rho);
    if (numElectrons > 0.0) {  // rho *= N / sum_i w_i rho_i
        double *integral = work + (workDoubles - 1);
        TAGI_TRY(tagi_wdot_rows(rho, 0, nullptr, 0, weights, numPoints, 1, integral, work, workDoubles - 1, stream));
        launch(scale_to, g, 256, 0, s, rho, (long)numPoints, numElectrons, integral);
    }
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

long long tagi_gi_anderson_workspace_doubles(long long numPoints, int numHistory, int numOrbitals) {
    const Chunks c = chunks_for(numPoints > 0 ? numPoints : 1);
    return (long long)c.nblk * numOrbitals * (numHistory * (numHistory + 1) / 2);
}

int tagi_gi_anderson_gram(const double *F, int numHistory, int numOrbitals, long long numPoints,
                          const double *weights, double *gram, double *work, long long workDoubles, void *stream) {
    if (!F || !weights || !gram || !work) return set_error(TAGI_ERR_ARG, "null pointer");
    if (numHistory < 1 || numHistory > AND_MAXH)
        return set_error(TAGI_ERR_ARG, "history %d outside [1, %d]", numHistory, AND_MAXH);
    if (numPoints <= 0 || numOrbitals <= 0 || numOrbitals > 65535) return set_error(TAGI_ERR_ARG, "bad sizes");
    const Chunks c = chunks_for(numPoints);
    const int np = numHistory * (numHistory + 1) / 2;
    if (workDoubles < (long long)c.nblk * numOrbitals * np) return set_error(TAGI_ERR_ARG, "workspace too small");
    cudaStream_t s = (cudaStream_t)stream;
    launch(anderson_gram_partial, dim3(c.nblk, numOrbitals), GT, 0, s, F, numHistory, numOrbitals, (long)numPoints,
           weights, c.chunk, c.nblk, work);
    launch(anderson_gram_final, (numOrbitals * np + 127) / 128, 128, 0, s, work, c.nblk, numOrbitals, np, gram);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

int tagi_gi_anderson_mix(const double *X, const double *F, int numHistory, int newestRow, const int *olderRows,
                         const double *coefficients, double mixingParameter, int numOrbitals, long long numPoints,
                         double *psi, void *stream) {
    if (!X || !F || !psi || (numHistory > 1 && (!olderRows || !coefficients)))
        return set_error(TAGI_ERR_ARG, "null pointer");
    if (numHistory < 1 || numHistory > AND_MAXH || numPoints <= 0 || numOrbitals <= 0 || numOrbitals > 65535)
        return set_error(TAGI_ERR_ARG, "bad sizes");
    launch(anderson_mix, dim3((unsigned)((numPoints + 255) / 256), numOrbitals), 256, 0, (cudaStream_t)stream, X, F,
           numHistory, newestRow, olderRows, coefficients, mixingParameter, numOrbitals, (long)numPoints, psi);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

int tagi_lda_exchange(const double *rho, long long numPoints, double *vx, double *ex, void *stream) {
    if (!rho || !vx || !ex) return set_error(TAGI_ERR_ARG, "null pointer");
    if (numPoints <= 0) return set_error(TAGI_ERR_ARG, "bad sizes");
    launch(lda_exchange, (unsigned)((numPoints + 255) / 256), 256, 0, (cudaStream_t)stream, rho, (long)numPoints, vx,
           ex);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

int tagi_veff(const double *vHartree, const double *vx, const double *vExternal, double gaugeShift,
              long long numPoints, double *veff, void *stream) {
    if (!vHartree || !vx || !vExternal || !veff) return set_error(TAGI_ERR_ARG, "null pointer");
    if (numPoints <= 0) return set_error(TAGI_ERR_ARG, "bad sizes");
    launch(veff_assemble, (unsigned)((numPoints + 255) / 256), 256, 0, (cudaStream_t)stream, vHartree, vx, vExternal,
           gaugeShift, (long)numPoints, veff);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

int tagi_anderson_combine(const double *inHistory, const double *outHistory, int numHistory, int newestRow,
                          const int *olderRows, const double *coefficients, double mixingParameter,
                          long long numPoints, double *next, void *stream) {
    if (!inHistory || !outHistory || !next || (numHistory > 1 && (!olderRows || !coefficients)))
        return set_error(TAGI_ERR_ARG, "null pointer");
    if (numPoints <= 0 || numHistory < 1) return set_error(TAGI_ERR_ARG, "bad sizes");
    launch(anderson_combine, (unsigned)((numPoints + 255) / 256), 256, 0, (cudaStream_t)stream, inHistory, outHistory,
           numHistory, newestRow, olderRows, coefficients, mixingParameter, (long)numPoints, next);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

}  // extern "C"
