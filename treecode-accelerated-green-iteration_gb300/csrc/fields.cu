// Subsystems (c) far field and (d) near field, plus the per-call glue.
//
// One CTA works on one (target batch, orbital) item at a time, pulled from a
// global counter in heaviest-batch-first order (persistent launch, grid =
// resident CTAs).  Each target's sum is formed in a fixed order (list order,
// then source order), so results do not depend on scheduling.
//
// Mixed precision (default fast path):
//   * coordinates are translated to the batch center in FP64, then rounded to
//     FP32 (targets once per batch, sources/proxy points while staging into
//     shared memory), so pair distances keep FP32 precision relative to the
//     batch size rather than to the domain size;
//   * pair terms and per-tile sums in FP32, rsqrt and exp2 on the MUFU pipe;
//   * tiles (near) and clusters (far) are added with Kahan compensation;
//   * the singularity-subtraction term f_i * 4pi/k^2 (Yukawa) or
//     f_i * 2pi/a^2 (Coulomb) is added in FP64 in the epilogue.
// FP64 mode: identical structure, FP64 everywhere (exp, sqrt, division).
//
// Pair terms (targets i, sources j, r = |x_i - y_j| > 0):
//   Yukawa  SS  w_j (f_j - f_i) e^{-k r}/r        skip  w_j f_j e^{-k r}/r
//   Coulomb SS  w_j (f_j - f_i e^{-a^2 r^2})/r    skip  w_j f_j / r
// (TreeStruct_CC.py:2782,2795,2931; greenIterationFixedPoint.py:314-324;
//  scfFixedPoint.py:297-303).  Far field: the same with (y_j, w_j f_j, w_j)
// replaced by (proxy point s_k, qhat_k, what_k).
#include "tagi_internal.h"

#include <cmath>

namespace tagi {

namespace {

constexpr int FT = 256;        // threads per field CTA
constexpr int NTILE = 512;     // sources per near-field tile
constexpr double LOG2E = 1.4426950408889634;

__device__ __forceinline__ float rsqrt_mufu(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float ex2_mufu(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

struct Fields {
    // target side (sorted order)
    const double *tx, *ty, *tz;
    const int *tbegin, *tend;
    const double *tcenter;
    const int *batch_node;
    const int *order;
    int nbatch, nt, norb;
    int *queue;
    // near side
    const int *rng_off;
    const int2 *rng;
    const double *sx, *sy, *sz;
    int ns;
    const float *q32, *w32;       // [norb][ns] charges f*w, [ns] weights
    const double *f64, *w64;      // [norb][ns] values f, [ns] weights
    // far side
    const int *far_off, *far_list, *node_slot;
    const double *geom;
    const float *qhat32, *what32; // [norb][nslots][P], [nslots][P]
    const double *qhat64, *what64;
    int nslots, n1, P;
    double tn[MAX_DEGREE + 1];
    // per orbital
    const float *ft32;            // [norb][nt] sorted target values
    const double *ft64;
    const float *kc32;            // [norb] kernel constant (see kernel_constant)
    const double *kp64;           // [norb] kernel parameter k or a
    double *out;                  // [norb][nt] sorted order
};

// Kernel constant for the exp2 argument: Yukawa -k log2(e), Coulomb SS -a^2 log2(e).
inline float kernel_constant(int kernel, double kp) {
    return kernel == KERNEL_YUKAWA ? (float)(-kp * LOG2E) : (float)(-kp * kp * LOG2E);
}

__device__ __forceinline__ int next_item(int *queue, int *s_item) {
    __syncthreads();
    if (threadIdx.x == 0) *s_item = atomicAdd(queue, 1);
    __syncthreads();
    return *s_item;
}

template <int KERN, bool SS>
__device__ __forceinline__ float pair_near(float dx, float dy, float dz, float q, float w,
                                           float fi, float kc, float acc) {
    float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    float rinv = rsqrt_mufu(r2);
    rinv = r2 > 0.f ? rinv : 0.f;  // excludes the coincident (self) pair
    if (KERN == KERNEL_YUKAWA) {
        float g = ex2_mufu(kc * (r2 * rinv)) * rinv;
        float c = SS ? fmaf(-fi, w, q) : q;
        return fmaf(g, c, acc);
    } else {
        if (SS) {
            float e = ex2_mufu(kc * r2);
            return fmaf(rinv, fmaf(-fi * e, w, q), acc);
        }
        return fmaf(rinv, q, acc);
    }
}

// ---------------------------------------------------------------------------
// Near field, mixed precision.
// ---------------------------------------------------------------------------
template <int KERN, bool SS, int NT>
__global__ void __launch_bounds__(FT) near_mixed(Fields a) {
    __shared__ float4 s_src[NTILE];
    __shared__ float s_w[NTILE];
    __shared__ int s_item;
    const int tid = threadIdx.x;
    const int total = a.nbatch * a.norb;
    for (;;) {
        const int item = next_item(a.queue, &s_item);
        if (item >= total) break;
        const int b = a.order[item / a.norb];
        const int orb = item - (item / a.norb) * a.norb;
        const int bn = a.batch_node[b];
        const int tb = a.tbegin[bn], te = a.tend[bn];
        const double cbx = a.tcenter[3L * bn], cby = a.tcenter[3L * bn + 1],
                     cbz = a.tcenter[3L * bn + 2];
        const float kc = a.kc32[orb];
        const float *q = a.q32 + (long)orb * a.ns;
        const float *ft = a.ft32 + (long)orb * a.nt;
        const int r0 = a.rng_off[b], r1 = a.rng_off[b + 1];
        for (int base = tb; base < te; base += FT * NT) {
            float tx[NT], ty[NT], tz[NT], fi[NT], sum[NT], cmp[NT];
#pragma unroll
            for (int k = 0; k < NT; k++) {
                int i = base + tid + k * FT;
                bool v = i < te;
                tx[k] = v ? (float)(a.tx[i] - cbx) : 0.f;
                ty[k] = v ? (float)(a.ty[i] - cby) : 0.f;
                tz[k] = v ? (float)(a.tz[i] - cbz) : 0.f;
                fi[k] = v ? ft[i] : 0.f;
                sum[k] = 0.f;
                cmp[k] = 0.f;
            }
            for (int e = r0; e < r1; e++) {
                const int2 r = a.rng[e];
                for (int t0 = r.x; t0 < r.y; t0 += NTILE) {
                    const int cnt = min(NTILE, r.y - t0);
                    __syncthreads();
                    for (int j = tid; j < cnt; j += FT) {
                        int jj = t0 + j;
                        s_src[j] = make_float4((float)(a.sx[jj] - cbx), (float)(a.sy[jj] - cby),
                                               (float)(a.sz[jj] - cbz), q[jj]);
                        s_w[j] = a.w32[jj];
                    }
                    __syncthreads();
                    float part[NT];
#pragma unroll
                    for (int k = 0; k < NT; k++) part[k] = 0.f;
#pragma unroll 4
                    for (int j = 0; j < cnt; j++) {
                        const float4 s = s_src[j];
                        const float w = s_w[j];
#pragma unroll
                        for (int k = 0; k < NT; k++)
                            part[k] = pair_near<KERN, SS>(tx[k] - s.x, ty[k] - s.y, tz[k] - s.z,
                                                          s.w, w, fi[k], kc, part[k]);
                    }
#pragma unroll
                    for (int k = 0; k < NT; k++) {  // Kahan across tiles
                        float y = part[k] - cmp[k];
                        float t = sum[k] + y;
                        cmp[k] = (t - sum[k]) - y;
                        sum[k] = t;
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < NT; k++) {
                int i = base + tid + k * FT;
                if (i < te) a.out[(long)orb * a.nt + i] = (double)sum[k] - (double)cmp[k];
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Far field, mixed precision.  Proxy grid is a tensor product, so r^2 is
// assembled from per-axis squares: (k1,k2) parts once per 8 pairs.
// ---------------------------------------------------------------------------
template <int KERN, bool SS, int MAXN1>
__global__ void __launch_bounds__(FT) far_mixed(Fields a) {
    constexpr int MAXP = MAXN1 * MAXN1 * MAXN1;
    __shared__ float2 s_qw[MAXP];
    __shared__ float s_p[3][MAXN1];
    __shared__ int s_item;
    const int tid = threadIdx.x;
    const int n1 = a.n1, P = a.P;
    const int total = a.nbatch * a.norb;
    for (;;) {
        const int item = next_item(a.queue + 1, &s_item);
        if (item >= total) break;
        const int b = a.order[item / a.norb];
        const int orb = item - (item / a.norb) * a.norb;
        const int f0 = a.far_off[b], f1 = a.far_off[b + 1];
        if (f0 == f1) continue;
        const int bn = a.batch_node[b];
        const int tb = a.tbegin[bn], te = a.tend[bn];
        const double cb[3] = {a.tcenter[3L * bn], a.tcenter[3L * bn + 1], a.tcenter[3L * bn + 2]};
        const float kc = a.kc32[orb];
        const float *ft = a.ft32 + (long)orb * a.nt;
        const float *qh = a.qhat32 + (long)orb * a.nslots * P;
        for (int base = tb; base < te; base += FT) {
            const int i = base + tid;
            const bool v = i < te;
            const float tx = v ? (float)(a.tx[i] - cb[0]) : 0.f;
            const float ty = v ? (float)(a.ty[i] - cb[1]) : 0.f;
            const float tz = v ? (float)(a.tz[i] - cb[2]) : 0.f;
            const float fi = v ? ft[i] : 0.f;
            float sum = 0.f, cmp = 0.f;
            for (int e = f0; e < f1; e++) {
                const int slot = a.node_slot[a.far_list[e]];
                __syncthreads();
                const float *qs = qh + (long)slot * P;
                const float *ws = a.what32 + (long)slot * P;
                for (int k = tid; k < P; k += FT) s_qw[k] = make_float2(qs[k], ws[k]);
                if (tid < 3 * n1) {
                    int d = tid / n1, m = tid - d * n1;
                    const double *g = a.geom + 6L * slot;
                    s_p[d][m] = (float)((g[d] + g[3 + d] * a.tn[m]) - cb[d]);
                }
                __syncthreads();
                float dz2[MAXN1];
#pragma unroll
                for (int m = 0; m < MAXN1; m++) {
                    float d = tz - s_p[2][m < n1 ? m : 0];
                    dz2[m] = d * d;
                }
                float part = 0.f;
                int idx = 0;
                for (int k1 = 0; k1 < n1; k1++) {
                    const float dx = tx - s_p[0][k1];
                    const float dx2 = dx * dx;
                    for (int k2 = 0; k2 < n1; k2++) {
                        const float dy = ty - s_p[1][k2];
                        const float rxy = fmaf(dy, dy, dx2);
#pragma unroll
                        for (int k3 = 0; k3 < MAXN1; k3++) {
                            if (k3 < n1) {
                                const float r2 = rxy + dz2[k3];
                                const float rinv = rsqrt_mufu(r2);
                                const float2 qw = s_qw[idx + k3];
                                if (KERN == KERNEL_YUKAWA) {
                                    const float g = ex2_mufu(kc * (r2 * rinv)) * rinv;
                                    part = fmaf(g, SS ? fmaf(-fi, qw.y, qw.x) : qw.x, part);
                                } else if (SS) {
                                    const float ex = ex2_mufu(kc * r2);
                                    part = fmaf(rinv, fmaf(-fi * ex, qw.y, qw.x), part);
                                } else {
                                    part = fmaf(rinv, qw.x, part);
                                }
                            }
                        }
                        idx += n1;
                    }
                }
                float y = part - cmp;
                float t = sum + y;
                cmp = (t - sum) - y;
                sum = t;
            }
            if (v) a.out[(long)orb * a.nt + i] = (double)sum - (double)cmp;
        }
    }
}

// ---------------------------------------------------------------------------
// FP64 near and far fields (the plain path).
// ---------------------------------------------------------------------------
template <int KERN, bool SS>
__device__ __forceinline__ double pair_f64(double dx, double dy, double dz, double f, double w,
                                           double fi, double kp) {
    double r2 = dx * dx + dy * dy + dz * dz;
    if (!(r2 > 0.0)) return 0.0;
    double r = sqrt(r2);
    if (KERN == KERNEL_YUKAWA) {
        double g = exp(-kp * r) / r;
        return SS ? w * (f - fi) * g : w * f * g;
    } else {
        if (SS) return w * (f - fi * exp(-kp * kp * r2)) / r;
        return w * f / r;
    }
}

template <int KERN, bool SS>
__global__ void __launch_bounds__(FT) near_f64(Fields a) {
    constexpr int T64 = 256;
    __shared__ double s_x[T64], s_y[T64], s_z[T64], s_f[T64], s_w[T64];
    __shared__ int s_item;
    const int tid = threadIdx.x;
    const int total = a.nbatch * a.norb;
    for (;;) {
        const int item = next_item(a.queue, &s_item);
        if (item >= total) break;
        const int b = a.order[item / a.norb];
        const int orb = item - (item / a.norb) * a.norb;
        const int bn = a.batch_node[b];
        const int tb = a.tbegin[bn], te = a.tend[bn];
        const double kp = a.kp64[orb];
        const double *f = a.f64 + (long)orb * a.ns;
        const double *ft = a.ft64 + (long)orb * a.nt;
        const int r0 = a.rng_off[b], r1 = a.rng_off[b + 1];
        for (int base = tb; base < te; base += FT) {
            const int i = base + tid;
            const bool v = i < te;
            const double xi = v ? a.tx[i] : 0.0, yi = v ? a.ty[i] : 0.0, zi = v ? a.tz[i] : 0.0;
            const double fi = v ? ft[i] : 0.0;
            double acc = 0.0;
            for (int e = r0; e < r1; e++) {
                const int2 r = a.rng[e];
                for (int t0 = r.x; t0 < r.y; t0 += T64) {
                    const int cnt = min(T64, r.y - t0);
                    __syncthreads();
                    if (tid < cnt) {
                        int jj = t0 + tid;
                        s_x[tid] = a.sx[jj];
                        s_y[tid] = a.sy[jj];
                        s_z[tid] = a.sz[jj];
                        s_f[tid] = f[jj];
                        s_w[tid] = a.w64[jj];
                    }
                    __syncthreads();
                    for (int j = 0; j < cnt; j++)
                        acc += pair_f64<KERN, SS>(xi - s_x[j], yi - s_y[j], zi - s_z[j], s_f[j],
                                                  s_w[j], fi, kp);
                }
            }
            if (v) a.out[(long)orb * a.nt + i] = acc;
        }
    }
}

template <int KERN, bool SS, int MAXN1>
__global__ void __launch_bounds__(FT) far_f64(Fields a) {
    constexpr int MAXP = MAXN1 * MAXN1 * MAXN1;
    __shared__ double s_q[MAXP], s_wh[MAXP];
    __shared__ double s_p[3][MAXN1];
    __shared__ int s_item;
    const int tid = threadIdx.x;
    const int n1 = a.n1, P = a.P;
    const int total = a.nbatch * a.norb;
    for (;;) {
        const int item = next_item(a.queue + 1, &s_item);
        if (item >= total) break;
        const int b = a.order[item / a.norb];
        const int orb = item - (item / a.norb) * a.norb;
        const int f0 = a.far_off[b], f1 = a.far_off[b + 1];
        if (f0 == f1) continue;
        const int bn = a.batch_node[b];
        const int tb = a.tbegin[bn], te = a.tend[bn];
        const double kp = a.kp64[orb];
        const double *ft = a.ft64 + (long)orb * a.nt;
        const double *qh = a.qhat64 + (long)orb * a.nslots * P;
        for (int base = tb; base < te; base += FT) {
            const int i = base + tid;
            const bool v = i < te;
            const double xi = v ? a.tx[i] : 0.0, yi = v ? a.ty[i] : 0.0, zi = v ? a.tz[i] : 0.0;
            const double fi = v ? ft[i] : 0.0;
            double acc = 0.0;
            for (int e = f0; e < f1; e++) {
                const int slot = a.node_slot[a.far_list[e]];
                __syncthreads();
                for (int k = tid; k < P; k += FT) {
                    s_q[k] = qh[(long)slot * P + k];
                    s_wh[k] = a.what64[(long)slot * P + k];
                }
                if (tid < 3 * n1) {
                    int d = tid / n1, m = tid - d * n1;
                    const double *g = a.geom + 6L * slot;
                    s_p[d][m] = g[d] + g[3 + d] * a.tn[m];
                }
                __syncthreads();
                int idx = 0;
                for (int k1 = 0; k1 < n1; k1++) {
                    const double dx = xi - s_p[0][k1];
                    for (int k2 = 0; k2 < n1; k2++) {
                        const double dy = yi - s_p[1][k2];
                        for (int k3 = 0; k3 < n1; k3++) {
                            const double dz = zi - s_p[2][k3];
                            const double r2 = dx * dx + dy * dy + dz * dz;
                            const double r = sqrt(r2);
                            const double qk = s_q[idx + k3], wk = s_wh[idx + k3];
                            if (KERN == KERNEL_YUKAWA) {
                                acc += exp(-kp * r) / r * (SS ? (qk - fi * wk) : qk);
                            } else if (SS) {
                                acc += (qk - fi * wk * exp(-kp * kp * r2)) / r;
                            } else {
                                acc += qk / r;
                            }
                        }
                        idx += n1;
                    }
                }
            }
            if (v) a.out[(long)orb * a.nt + i] = acc;
        }
    }
}

// ---------------------------------------------------------------------------
// Per-call glue: sorted charges, epilogue.
// ---------------------------------------------------------------------------
__global__ void prep_sources(const double *__restrict__ sv, const int *__restrict__ perm,
                             const double *__restrict__ w, int ns, int norb,
                             float *__restrict__ q32, double *__restrict__ q64,
                             double *__restrict__ f64) {
    long j = (long)blockIdx.x * blockDim.x + threadIdx.x;
    int orb = blockIdx.y;
    if (j >= ns) return;
    long o = (long)orb * ns + j;
    double f = sv[(long)orb * ns + perm[j]];
    double q = f * w[j];
    q32[o] = (float)q;
    q64[o] = q;
    f64[o] = f;
}

__global__ void prep_targets(const double *__restrict__ tv, const int *__restrict__ perm, int nt,
                             float *__restrict__ f32, double *__restrict__ f64) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    int orb = blockIdx.y;
    if (i >= nt) return;
    double f = tv[(long)orb * nt + perm[i]];
    f32[(long)orb * nt + i] = (float)f;
    f64[(long)orb * nt + i] = f;
}

__global__ void epilogue(const double *__restrict__ nearv, const double *__restrict__ farv,
                         const double *__restrict__ tv, const int *__restrict__ perm, int nt,
                         const double *__restrict__ ss, double *__restrict__ out) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    int orb = blockIdx.y;
    if (i >= nt) return;
    long o = (long)orb * nt + perm[i];
    long si = (long)orb * nt + i;
    out[o] = nearv[si] + farv[si] + ss[orb] * tv[o];
}

template <typename K>
int occupancy_grid(K kern, int *grid) {
    int dev = 0, sms = 0, per = 0;
    TAGI_CUDA(cudaGetDevice(&dev));
    TAGI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    TAGI_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, FT, 0));
    *grid = sms * (per > 0 ? per : 1);
    return TAGI_OK;
}

template <typename K>
int launch_persistent(K kern, const Fields &a, int items, cudaStream_t s) {
    int grid = 0;
    TAGI_TRY(occupancy_grid(kern, &grid));
    if (grid > items) grid = items;
    if (grid < 1) grid = 1;
    kern<<<grid, FT, 0, s>>>(a);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

template <int KERN, bool SS>
int launch_fields(Plan &p, const Fields &a, int precision, cudaStream_t s) {
    const int items = p.nbatch * a.norb;
    Fields an = a, af = a;
    an.order = p.order_near;
    an.out = p.near_out;
    af.order = p.order_far;
    af.out = p.far_out;
    if (precision == PREC_MIXED) {
        if (p.max_batch <= FT) TAGI_TRY(launch_persistent(near_mixed<KERN, SS, 1>, an, items, s));
        else TAGI_TRY(launch_persistent(near_mixed<KERN, SS, 2>, an, items, s));
        if (p.nslots == 0) return TAGI_OK;
        if (p.n1 <= 4) TAGI_TRY(launch_persistent(far_mixed<KERN, SS, 4>, af, items, s));
        else if (p.n1 <= 8) TAGI_TRY(launch_persistent(far_mixed<KERN, SS, 8>, af, items, s));
        else TAGI_TRY(launch_persistent(far_mixed<KERN, SS, MAX_DEGREE + 1>, af, items, s));
    } else {
        TAGI_TRY(launch_persistent(near_f64<KERN, SS>, an, items, s));
        if (p.nslots == 0) return TAGI_OK;
        if (p.n1 <= 4) TAGI_TRY(launch_persistent(far_f64<KERN, SS, 4>, af, items, s));
        else if (p.n1 <= 8) TAGI_TRY(launch_persistent(far_f64<KERN, SS, 8>, af, items, s));
        else TAGI_TRY(launch_persistent(far_f64<KERN, SS, MAX_DEGREE + 1>, af, items, s));
    }
    return TAGI_OK;
}

}  // namespace

int ensure_scratch(Plan &p, int norb) {
    if ((size_t)norb <= p.scratch_orbitals) return TAGI_OK;
    cudaStream_t s = p.arena.stream;
    for (void *v : p.scratch) cudaFreeAsync(v, s);
    p.scratch.clear();
    p.scratch_orbitals = 0;
    Arena a;
    a.stream = s;
    const size_t ns = p.src.n, nt = p.tgt.n, no = norb;
    int rc = TAGI_OK;
    if ((rc = a.alloc(&p.q32, no * ns)) || (rc = a.alloc(&p.ft32, no * nt)) ||
        (rc = a.alloc(&p.q64, no * ns)) || (rc = a.alloc(&p.f64s, no * ns)) ||
        (rc = a.alloc(&p.ft64, no * nt)) || (rc = a.alloc(&p.part, no * p.nitems * p.P)) ||
        (rc = a.alloc(&p.qhat32, no * p.nslots * p.P)) ||
        (rc = a.alloc(&p.qhat64, no * p.nslots * p.P)) || (rc = a.alloc(&p.near_out, no * nt)) ||
        (rc = a.alloc(&p.far_out, no * nt)) || (rc = a.alloc(&p.d_kc, no)) ||
        (rc = a.alloc(&p.d_kp, no)) || (rc = a.alloc(&p.d_ss, no))) {
        p.scratch = a.ptrs;
        return rc;
    }
    p.scratch = a.ptrs;
    p.scratch_orbitals = no;
    return TAGI_OK;
}

int convolve(Plan &p, const double *tv, const double *sv, double *out, int norb, int kernel,
             const double *kparams, int nkp, int singularity, int precision, cudaStream_t s) {
    TAGI_TRY(ensure_scratch(p, norb));
    const int ns = p.src.n, nt = p.tgt.n;
    const bool mixed = precision == PREC_MIXED;
    const bool ss = singularity == SING_SUBTRACTION;

    // Per-orbital constants: k (Yukawa) or a (Coulomb) from kernelParameters[o * nkp].
    p.h_kc.resize(norb);
    p.h_kp.resize(norb);
    p.h_ss.resize(norb);
    for (int o = 0; o < norb; o++) {
        double k = kparams[(long)o * nkp];
        p.h_kp[o] = k;
        p.h_kc[o] = kernel_constant(kernel, k);
        p.h_ss[o] = 0.0;
        if (ss) p.h_ss[o] = kernel == KERNEL_YUKAWA ? 4.0 * M_PI / (k * k) : 2.0 * M_PI / (k * k);
    }
    TAGI_CUDA(cudaMemcpyAsync(p.d_kc, p.h_kc.data(), sizeof(float) * norb, cudaMemcpyHostToDevice, s));
    TAGI_CUDA(cudaMemcpyAsync(p.d_kp, p.h_kp.data(), sizeof(double) * norb, cudaMemcpyHostToDevice, s));
    TAGI_CUDA(cudaMemcpyAsync(p.d_ss, p.h_ss.data(), sizeof(double) * norb, cudaMemcpyHostToDevice, s));

    dim3 gs((ns + 255) / 256, norb), gt((nt + 255) / 256, norb);
    prep_sources<<<gs, 256, 0, s>>>(sv, p.src.perm, p.sw64, ns, norb, p.q32, p.q64, p.f64s);
    prep_targets<<<gt, 256, 0, s>>>(tv, p.tgt.perm, nt, p.ft32, p.ft64);
    TAGI_LAUNCH_CHECK();
    TAGI_TRY(modified_charges(p, mixed ? PREC_MIXED : PREC_FP64, norb, s));

    Fields a{};
    a.tx = p.tgt.x;
    a.ty = p.tgt.y;
    a.tz = p.tgt.z;
    a.tbegin = p.tgt.begin;
    a.tend = p.tgt.end;
    a.tcenter = p.tgt.center;
    a.batch_node = p.batch_node;
    a.nbatch = p.nbatch;
    a.nt = nt;
    a.norb = norb;
    a.queue = p.queue;
    a.rng_off = p.rng_off;
    a.rng = p.rng;
    a.sx = p.src.x;
    a.sy = p.src.y;
    a.sz = p.src.z;
    a.ns = ns;
    a.q32 = p.q32;
    a.w32 = p.sw32;
    a.f64 = p.f64s;
    a.w64 = p.sw64;
    a.far_off = p.far_off;
    a.far_list = p.far_list;
    a.node_slot = p.node_slot;
    a.geom = p.slot_geom;
    a.qhat32 = p.qhat32;
    a.what32 = p.what32;
    a.qhat64 = p.qhat64;
    a.what64 = p.what64;
    a.nslots = p.nslots;
    a.n1 = p.n1;
    a.P = p.P;
    for (int m = 0; m <= MAX_DEGREE; m++) a.tn[m] = m <= p.degree ? p.cheb[m] : 0.0;
    a.ft32 = p.ft32;
    a.ft64 = p.ft64;
    a.kc32 = p.d_kc;
    a.kp64 = p.d_kp;

    TAGI_CUDA(cudaMemsetAsync(p.queue, 0, 2 * sizeof(int), s));
    TAGI_CUDA(cudaMemsetAsync(p.far_out, 0, sizeof(double) * (size_t)norb * nt, s));
    if (kernel == KERNEL_YUKAWA) {
        if (ss) TAGI_TRY((launch_fields<KERNEL_YUKAWA, true>(p, a, precision, s)));
        else TAGI_TRY((launch_fields<KERNEL_YUKAWA, false>(p, a, precision, s)));
    } else {
        if (ss) TAGI_TRY((launch_fields<KERNEL_COULOMB, true>(p, a, precision, s)));
        else TAGI_TRY((launch_fields<KERNEL_COULOMB, false>(p, a, precision, s)));
    }
    epilogue<<<gt, 256, 0, s>>>(p.near_out, p.far_out, tv, p.tgt.perm, nt, p.d_ss, out);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

}  // namespace tagi
