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
//   * coordinates are also multiplied by a per-orbital scale sc, so that with
//     r' = sc r the kernels need no multiply for the exp2 argument:
//       Yukawa       sc = k log2(e):          e^{-k r}/r     = sc 2^{-r'} / r'
//       Coulomb SS   sc = a sqrt(log2(e)):    e^{-a^2 r^2}   = 2^{-r'^2},  1/r = sc / r'
//       Coulomb skip sc = 1
//     and the factor sc multiplies each target's sum once at the end;
//   * pair terms and per-tile sums in FP32, rsqrt and exp2 on the MUFU pipe;
//   * pair terms are summed in FP32 runs of 64 (near) or one (n+1)^2 slab
//     (far) and the runs are added with Kahan compensation;
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

#include <algorithm>
#include <cmath>
#include <type_traits>

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
    const double *tcenter, *tradius;
    const int *batch_node;
    int nbatch, nt, norb;
    // near side
    const int *rng_off;
    const int2 *rng;
    const float *rng_dmin;
    const double *sx, *sy, *sz;
    const float4 *shi, *slo, *thi, *tlo;  // FP32 hi/lo splits of absolute coordinates
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
    const float *kc32;            // [norb] coordinate scale sc (orbital_constants)
    const double *kp64;           // [norb] kernel parameter k or a
    double *out;                  // [norb][nt] sorted order
};

// Argument of every persistent field kernel: the work list of this pass and
// up to MAX_SYSTEMS systems' fields.  It is a __grid_constant__ parameter, so
// a CTA reads the fields of its current item's system straight from the
// parameter bank (dynamic index, no local copy).
struct Work {
    const int2 *items;            // {batch, sys << 16 | first orbital}, heaviest first
    int nitems;
    int *queue;                   // this pass's work counter
    Fields sys[MAX_SYSTEMS];
};
static_assert(sizeof(Work) <= 4096, "field-kernel parameter block above 4 KB");

__device__ __forceinline__ int next_item(int *queue, int *s_item) {
    __syncthreads();
    if (threadIdx.x == 0) *s_item = atomicAdd(queue, 1);
    __syncthreads();
    return *s_item;
}

// One pair from its squared scaled distance r2 = r'^2; MASK drops the
// coincident (r = 0) pair.
template <int KERN, bool SS, bool MASK>
__device__ __forceinline__ float pair_r2(float r2, float q, float w, float fi, float acc) {
    float rinv = rsqrt_mufu(r2);
    if (MASK) rinv = r2 > 0.f ? rinv : 0.f;
    if (KERN == KERNEL_YUKAWA) {
        const float g = ex2_mufu(-(r2 * rinv)) * rinv;
        return fmaf(g, SS ? fmaf(-fi, w, q) : q, acc);
    } else if (SS) {
        const float e = ex2_mufu(-r2);
        return fmaf(rinv, fmaf(-fi * e, w, q), acc);
    } else {
        return fmaf(rinv, q, acc);
    }
}

template <int KERN, bool SS, bool MASK>
__device__ __forceinline__ float pair_scaled(float dx, float dy, float dz, float q, float w, float fi,
                                             float acc) {
    return pair_r2<KERN, SS, MASK>(fmaf(dx, dx, fmaf(dy, dy, dz * dz)), q, w, fi, acc);
}

// Compensated (Kahan) addition of an FP32 partial into (sum, cmp).
__device__ __forceinline__ void kahan_add(float &sum, float &cmp, float part) {
    const float y = part - cmp;
    const float t = sum + y;
    cmp = (t - sum) - y;
    sum = t;
}

// One staged tile against NT targets.  Pairs are summed in FP32 in chunks of
// KCHUNK and each chunk is added to the target's Kahan sum: a long FP32 run
// loses ~sqrt(n) u of its total, and singularity subtraction multiplies that
// loss by |f_i int G| / |phi_i| (often 10-100).
// Ordinary tiles: s_a[j] = (scaled batch-relative x, y, z, q), s_b[j].w = w.
// PRECISE tiles (close ranges): s_a[j] = (x_hi, y_hi, z_hi, q) and
// s_b[j] = (x_lo, y_lo, z_lo, w) are FP32 splits of the absolute FP64
// coordinates, the targets likewise; each difference is (t_hi - s_hi) +
// (t_lo - s_lo) -- exact hi differences for nearby points -- and the unscaled
// r^2 is multiplied by sc2 = sc^2, so the shortest pairs keep FP32 relative
// precision in r whatever the batch size.
constexpr int KCHUNK = 64;
template <int KERN, bool SS, bool MASK, bool PRECISE, int NT>
__device__ __forceinline__ void near_tile(const float4 *__restrict__ s_a, const float4 *__restrict__ s_b,
                                          int cnt, const float (&tx)[NT], const float (&ty)[NT],
                                          const float (&tz)[NT], const float *__restrict__ s_tl, float sc2,
                                          const float (&fi)[NT], float (&sum)[NT], float (&cmp)[NT]) {
    // lo parts of this thread's targets (only live inside PRECISE tiles)
    float lx[NT], ly[NT], lz[NT];
#pragma unroll
    for (int k = 0; k < NT; k++) {
        lx[k] = PRECISE ? s_tl[3 * k] : 0.f;
        ly[k] = PRECISE ? s_tl[3 * k + 1] : 0.f;
        lz[k] = PRECISE ? s_tl[3 * k + 2] : 0.f;
    }
    for (int j0 = 0; j0 < cnt; j0 += KCHUNK) {
        const int j1 = min(j0 + KCHUNK, cnt);
        float part[NT];
#pragma unroll
        for (int k = 0; k < NT; k++) part[k] = 0.f;
        if (j1 - j0 == KCHUNK) {
#pragma unroll 8
            for (int j = j0; j < j0 + KCHUNK; j++) {
                const float4 sa = s_a[j];
                if (PRECISE) {
                    const float4 sb = s_b[j];
#pragma unroll
                    for (int k = 0; k < NT; k++) {
                        const float dx = (tx[k] - sa.x) + (lx[k] - sb.x);
                        const float dy = (ty[k] - sa.y) + (ly[k] - sb.y);
                        const float dz = (tz[k] - sa.z) + (lz[k] - sb.z);
                        part[k] = pair_r2<KERN, SS, MASK>(fmaf(dx, dx, fmaf(dy, dy, dz * dz)) * sc2, sa.w, sb.w,
                                                          fi[k], part[k]);
                    }
                } else {
                    const float w = s_b[j].w;
#pragma unroll
                    for (int k = 0; k < NT; k++)
                        part[k] = pair_scaled<KERN, SS, MASK>(tx[k] - sa.x, ty[k] - sa.y, tz[k] - sa.z, sa.w, w,
                                                              fi[k], part[k]);
                }
            }
        } else {
#pragma unroll 2
            for (int j = j0; j < j1; j++) {
                const float4 sa = s_a[j];
                const float4 sb = s_b[j];
#pragma unroll
                for (int k = 0; k < NT; k++) {
                    const float dx = PRECISE ? (tx[k] - sa.x) + (lx[k] - sb.x) : tx[k] - sa.x;
                    const float dy = PRECISE ? (ty[k] - sa.y) + (ly[k] - sb.y) : ty[k] - sa.y;
                    const float dz = PRECISE ? (tz[k] - sa.z) + (lz[k] - sb.z) : tz[k] - sa.z;
                    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                    part[k] = pair_r2<KERN, SS, MASK>(PRECISE ? r2 * sc2 : r2, sa.w, sb.w, fi[k], part[k]);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < NT; k++) kahan_add(sum[k], cmp[k], part[k]);
    }
}

// Split an FP64 value into FP32 hi + lo.
__device__ __forceinline__ void split_f32(double v, float &hi, float &lo) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

// ---------------------------------------------------------------------------
// Near field, mixed precision.
// ---------------------------------------------------------------------------
// PASS 0 handles the ordinary near ranges, PASS 1 the close ones (double-float
// coordinates, r = 0 mask) into a second output; two passes keep each
// kernel's register footprint at two tile variants.
#ifndef TAGI_NEAR_MINB
#define TAGI_NEAR_MINB 3   // resident CTAs per SM the near kernel is compiled for
#endif
template <int KERN, bool SS, int NT, int PASS>
__global__ void __launch_bounds__(FT, TAGI_NEAR_MINB) near_mixed(const __grid_constant__ Work w) {
    __shared__ float4 s_a[NTILE];
    __shared__ float4 s_b[NTILE];
    __shared__ float s_tlo[FT * NT * 3];
    __shared__ int s_item;
    const int tid = threadIdx.x;
    float *my_tl = s_tlo + 3 * NT * tid;
    for (;;) {
        const int item = next_item(w.queue, &s_item);
        if (item >= w.nitems) break;
        const int2 it = w.items[item];
        const Fields &a = w.sys[it.y >> 16];
        const int b = it.x, orb = it.y & 0xffff;
        const int bn = a.batch_node[b];
        const int tb = a.tbegin[bn], te = a.tend[bn];
        const double cbx = a.tcenter[3L * bn], cby = a.tcenter[3L * bn + 1],
                     cbz = a.tcenter[3L * bn + 2];
        const float scf = a.kc32[orb];
        const double sc = (double)scf;
        const float sc2 = (float)(sc * sc);
        const float *q = a.q32 + (long)orb * a.ns;
        const float *ft = a.ft32 + (long)orb * a.nt;
        const int r0 = a.rng_off[b], r1 = a.rng_off[b + 1];
        for (int base = tb; base < te; base += FT * NT) {
            // consecutive targets per thread: the threads with targets form a
            // prefix, so whole warps past it have none and skip the pair loops
            const bool warp_busy = base + NT * (tid & ~31) < te;
            float tx[NT], ty[NT], tz[NT], fi[NT], sum[NT], cmp[NT];
#pragma unroll
            for (int k = 0; k < NT; k++) {
                int i = base + NT * tid + k;
                bool v = i < te;
                if (PASS == 1) {
                    const float4 h = v ? a.thi[i] : make_float4(0.f, 0.f, 0.f, 0.f);
                    const float4 l = v ? a.tlo[i] : make_float4(0.f, 0.f, 0.f, 0.f);
                    tx[k] = h.x;
                    ty[k] = h.y;
                    tz[k] = h.z;
                    my_tl[3 * k] = l.x;
                    my_tl[3 * k + 1] = l.y;
                    my_tl[3 * k + 2] = l.z;
                } else {
                    tx[k] = v ? (float)((a.tx[i] - cbx) * sc) : 0.f;
                    ty[k] = v ? (float)((a.ty[i] - cby) * sc) : 0.f;
                    tz[k] = v ? (float)((a.tz[i] - cbz) * sc) : 0.f;
                }
                fi[k] = v ? ft[i] : 0.f;
                sum[k] = 0.f;
                cmp[k] = 0.f;
            }
            for (int e = r0; e < r1; e++) {
                const int2 r = a.rng[e];
                const bool close = range_is_close(r);
                if (close != (PASS == 1)) continue;
                const int rb = range_begin(r);
                // Ranges far enough away: Yukawa terms are exactly 0 in FP32
                // (2^{-r'} with r' > 127 flushes to zero); the Coulomb Gaussian
                // correction is below 2^-40 of its term and is left out.
                const float dm = a.rng_dmin[e] * scf;
                if (KERN == KERNEL_YUKAWA && dm > 127.f) continue;
                const bool noexp = KERN == KERNEL_COULOMB && SS && dm * dm > 40.f;
                for (int t0 = rb; t0 < r.y; t0 += NTILE) {
                    const int cnt = min(NTILE, r.y - t0);
                    __syncthreads();
                    for (int j = tid; j < cnt; j += FT) {
                        const int jj = t0 + j;
                        float4 sa, sb;
                        if (PASS == 1) {
                            sa = a.shi[jj];
                            sb = a.slo[jj];
                        } else {
                            sa.x = (float)((a.sx[jj] - cbx) * sc);
                            sa.y = (float)((a.sy[jj] - cby) * sc);
                            sa.z = (float)((a.sz[jj] - cbz) * sc);
                            sb.x = sb.y = sb.z = 0.f;
                        }
                        sa.w = q[jj];
                        sb.w = a.w32[jj];
                        s_a[j] = sa;
                        s_b[j] = sb;
                    }
                    __syncthreads();
                    if (!warp_busy) continue;
                    if (PASS == 1)
                        near_tile<KERN, SS, true, true, NT>(s_a, s_b, cnt, tx, ty, tz, my_tl, sc2, fi, sum, cmp);
                    else if (noexp)
                        near_tile<KERN, false, false, false, NT>(s_a, s_b, cnt, tx, ty, tz, my_tl, sc2, fi, sum,
                                                                 cmp);
                    else
                        near_tile<KERN, SS, false, false, NT>(s_a, s_b, cnt, tx, ty, tz, my_tl, sc2, fi, sum, cmp);
                }
            }
#pragma unroll
            for (int k = 0; k < NT; k++) {
                int i = base + NT * tid + k;
                if (i < te) a.out[(long)orb * a.nt + i] = ((double)sum[k] - (double)cmp[k]) * sc;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Far field, mixed precision.  The proxy grid is a tensor product, so r'^2
// is assembled from per-axis squares (one add per pair).  Two targets per
// thread share every shared-memory read.  Coulomb subtraction: when the
// whole cluster lies so far that r'^2 > 40 for every proxy point, the
// Gaussian term f_i what_k 2^{-r'^2} is below 2^-40 of f_i what_k and is
// dropped (one MUFU op less per pair); Yukawa clusters with r' > 127
// everywhere add exactly 0 in FP32 (2^{-r'} flushes to zero) and are skipped.
// ---------------------------------------------------------------------------
template <int KERN, bool SS, bool EXPTERM, int MAXN1, int NT>
__device__ __forceinline__ void far_cluster(const float2 *__restrict__ s_qw, const float (*s_p)[MAXN1],
                                            int n1, const float (&tx)[NT], const float (&ty)[NT],
                                            const float (&tz)[NT], const float (&fi)[NT],
                                            float (&sum)[NT], float (&cmp)[NT]) {
    float dz2[NT][MAXN1];
#pragma unroll
    for (int k = 0; k < NT; k++)
#pragma unroll
        for (int m = 0; m < MAXN1; m++) {
            float d = tz[k] - s_p[2][m < n1 ? m : 0];
            dz2[k][m] = d * d;
        }
    int idx = 0;
    for (int k1 = 0; k1 < n1; k1++) {  // one (n+1)^2 slab per FP32 partial, then Kahan
        float part[NT];
#pragma unroll
        for (int k = 0; k < NT; k++) part[k] = 0.f;
        float dx2[NT];
#pragma unroll
        for (int k = 0; k < NT; k++) {
            const float dx = tx[k] - s_p[0][k1];
            dx2[k] = dx * dx;
        }
        for (int k2 = 0; k2 < n1; k2++) {
            float rxy[NT];
#pragma unroll
            for (int k = 0; k < NT; k++) {
                const float dy = ty[k] - s_p[1][k2];
                rxy[k] = fmaf(dy, dy, dx2[k]);
            }
#pragma unroll
            for (int k3 = 0; k3 < MAXN1; k3++) {
                if (k3 < n1) {
                    const float2 qw = s_qw[idx + k3];
#pragma unroll
                    for (int k = 0; k < NT; k++) {
                        const float r2 = rxy[k] + dz2[k][k3];
                        const float rinv = rsqrt_mufu(r2);
                        if (KERN == KERNEL_YUKAWA) {
                            const float g = ex2_mufu(-(r2 * rinv)) * rinv;
                            part[k] = fmaf(g, SS ? fmaf(-fi[k], qw.y, qw.x) : qw.x, part[k]);
                        } else if (SS && EXPTERM) {
                            const float ex = ex2_mufu(-r2);
                            part[k] = fmaf(rinv, fmaf(-fi[k] * ex, qw.y, qw.x), part[k]);
                        } else {
                            part[k] = fmaf(rinv, qw.x, part[k]);
                        }
                    }
                }
            }
            idx += n1;
        }
#pragma unroll
        for (int k = 0; k < NT; k++) kahan_add(sum[k], cmp[k], part[k]);
    }
}

template <int KERN, bool SS, int MAXN1, int NT>
__global__ void __launch_bounds__(FT, 2) far_mixed(const __grid_constant__ Work w) {
    constexpr int MAXP = MAXN1 * MAXN1 * MAXN1;
    __shared__ float2 s_qw[MAXP];
    __shared__ float s_p[3][MAXN1];
    __shared__ int s_item, s_mode;
    const int tid = threadIdx.x;
    for (;;) {
        const int item = next_item(w.queue, &s_item);
        if (item >= w.nitems) break;
        const int2 it = w.items[item];
        const Fields &a = w.sys[it.y >> 16];
        const int b = it.x, orb = it.y & 0xffff;
        const int n1 = a.n1, P = a.P;
        const int f0 = a.far_off[b], f1 = a.far_off[b + 1];
        if (f0 == f1) continue;
        const int bn = a.batch_node[b];
        const int tb = a.tbegin[bn], te = a.tend[bn];
        const double cb[3] = {a.tcenter[3L * bn], a.tcenter[3L * bn + 1], a.tcenter[3L * bn + 2]};
        const double rb = a.tradius[bn];
        const float scf = a.kc32[orb];
        const double sc = (double)scf;
        const float *ft = a.ft32 + (long)orb * a.nt;
        const float *qh = a.qhat32 + (long)orb * a.nslots * P;
        for (int base = tb; base < te; base += FT * NT) {
            const bool warp_busy = base + NT * (tid & ~31) < te;
            float tx[NT], ty[NT], tz[NT], fi[NT], sum[NT], cmp[NT];
#pragma unroll
            for (int k = 0; k < NT; k++) {
                const int i = base + NT * tid + k;
                const bool v = i < te;
                tx[k] = v ? (float)(a.tx[i] - cb[0]) * scf : 0.f;
                ty[k] = v ? (float)(a.ty[i] - cb[1]) * scf : 0.f;
                tz[k] = v ? (float)(a.tz[i] - cb[2]) * scf : 0.f;
                fi[k] = v ? ft[i] : 0.f;
                sum[k] = 0.f;
                cmp[k] = 0.f;
            }
            for (int e = f0; e < f1; e++) {
                const int slot = a.node_slot[a.far_list[e]];
                const double *g = a.geom + 6L * slot;
                __syncthreads();
                const float *qs = qh + (long)slot * P;
                const float *ws = a.what32 + (long)slot * P;
                for (int k = tid; k < P; k += FT) s_qw[k] = make_float2(qs[k], ws[k]);
                if (tid < 3 * n1) {
                    const int d = tid / n1, m = tid - d * n1;
                    const double cbd = d == 0 ? cb[0] : (d == 1 ? cb[1] : cb[2]);
                    s_p[d][m] = (float)((g[d] + g[3 + d] * a.tn[m]) - cbd) * scf;
                }
                if (tid == 0) {
                    // smallest scaled distance from the batch to the proxy box (conservative)
                    const double dx = cb[0] - g[0], dy = cb[1] - g[1], dz = cb[2] - g[2];
                    const double rc = sqrt(g[3] * g[3] + g[4] * g[4] + g[5] * g[5]);
                    const double dmin = (sqrt(dx * dx + dy * dy + dz * dz) - rb - rc) * sc * (1.0 - 1e-6);
                    int mode = 0;
                    if (KERN == KERNEL_YUKAWA && dmin > 127.0) mode = 2;  // 2^{-r'} flushes to 0: adds exactly 0
                    // Gaussian correction below 2^-40 of its own term everywhere: dropped
                    if (KERN == KERNEL_COULOMB && SS && dmin > 0.0 && dmin * dmin > 40.0) mode = 1;
                    s_mode = mode;
                }
                __syncthreads();
                const int mode = s_mode;
                if (mode == 2 || !warp_busy) continue;
                if (mode == 1) far_cluster<KERN, SS, false, MAXN1, NT>(s_qw, s_p, n1, tx, ty, tz, fi, sum, cmp);
                else far_cluster<KERN, SS, true, MAXN1, NT>(s_qw, s_p, n1, tx, ty, tz, fi, sum, cmp);
            }
#pragma unroll
            for (int k = 0; k < NT; k++) {
                const int i = base + NT * tid + k;
                if (i < te) a.out[(long)orb * a.nt + i] = ((double)sum[k] - (double)cmp[k]) * sc;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Orbital-group kernels (Yukawa, mixed precision): one item = (batch, group of
// OG orbitals).  Per pair the differences, r^2, rsqrt and r are computed once
// for the group; each orbital then adds exp2(-k_o log2(e) r) * rinv * c.
// Coordinates are translated to the batch center but not scaled (each orbital
// has its own k).  Charges are staged [source][orbital] so four orbitals come
// in one 16-byte shared-memory read.  Orbitals past the last one of the
// request have zero charges and are not written.
// ---------------------------------------------------------------------------
constexpr int GTILE = 256;   // sources per group tile

template <bool SS, bool MASK, bool PRECISE, int OG>
__device__ __forceinline__ void group_tile(const float4 *__restrict__ s_xyzw, const float4 *__restrict__ s_lo,
                                           const float4 *__restrict__ s_q4, int cnt, float tx, float ty,
                                           float tz, float lx, float ly, float lz, const float (&fi)[OG],
                                           const float (&kc)[OG], const float (&kl)[OG], float (&sum)[OG],
                                           float (&cmp)[OG]) {
    for (int j0 = 0; j0 < cnt; j0 += KCHUNK) {
        const int j1 = min(j0 + KCHUNK, cnt);
        float part[OG];
#pragma unroll
        for (int o = 0; o < OG; o++) part[o] = 0.f;
#pragma unroll 2
        for (int j = j0; j < j1; j++) {
            const float4 sj = s_xyzw[j];
            float dx = tx - sj.x, dy = ty - sj.y, dz = tz - sj.z;
            if (PRECISE) {
                const float4 sl = s_lo[j];
                dx += lx - sl.x;
                dy += ly - sl.y;
                dz += lz - sl.z;
            }
            const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            float rinv = rsqrt_mufu(r2);
            if (MASK) rinv = r2 > 0.f ? rinv : 0.f;
            const float r = r2 * rinv;
#pragma unroll
            for (int o4 = 0; o4 < OG / 4; o4++) {
                const float4 q4 = s_q4[j * (OG / 4) + o4];
                const float qv[4] = {q4.x, q4.y, q4.z, q4.w};
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const int o = 4 * o4 + u;
                    // exponent -k log2(e) r with the constant split hi + lo
                    const float g = ex2_mufu(fmaf(kc[o], r, kl[o] * r)) * rinv;
                    part[o] = fmaf(g, SS ? fmaf(-fi[o], sj.w, qv[u]) : qv[u], part[o]);
                }
            }
        }
#pragma unroll
        for (int o = 0; o < OG; o++) kahan_add(sum[o], cmp[o], part[o]);
    }
}

template <bool SS, int OG, int PASS>
__global__ void __launch_bounds__(FT, 2) near_group(const __grid_constant__ Work w) {
    __shared__ float4 s_xyzw[GTILE];
    __shared__ float4 s_lo[GTILE];
    __shared__ float4 s_q4[GTILE * OG / 4];
    __shared__ int s_item;
    const int tid = threadIdx.x;
    for (;;) {
        const int item = next_item(w.queue, &s_item);
        if (item >= w.nitems) break;
        const int2 it = w.items[item];
        const Fields &a = w.sys[it.y >> 16];
        const int b = it.x, g0 = it.y & 0xffff;
        const int bn = a.batch_node[b];
        const int tb = a.tbegin[bn], te = a.tend[bn];
        const double cbx = a.tcenter[3L * bn], cby = a.tcenter[3L * bn + 1], cbz = a.tcenter[3L * bn + 2];
        float kc[OG], kl[OG];
        float kmin = 3.4e38f;
#pragma unroll
        for (int o = 0; o < OG; o++) {
            const int orb = g0 + o;
            const double k2 = orb < a.norb ? -a.kp64[orb] * LOG2E : 0.0;   // -k log2(e)
            split_f32(k2, kc[o], kl[o]);
            if (orb < a.norb) kmin = fminf(kmin, a.kc32[orb]);
        }
        const int r0 = a.rng_off[b], r1 = a.rng_off[b + 1];
        for (int base = tb; base < te; base += FT) {
            const int i = base + tid;
            const bool v = i < te;
            const bool warp_busy = base + (tid & ~31) < te;
            float tx, ty, tz, lx = 0.f, ly = 0.f, lz = 0.f;
            if (PASS == 1) {  // absolute hi/lo splits (see near_tile)
                const float4 h = v ? a.thi[i] : make_float4(0.f, 0.f, 0.f, 0.f);
                const float4 l = v ? a.tlo[i] : make_float4(0.f, 0.f, 0.f, 0.f);
                tx = h.x; ty = h.y; tz = h.z;
                lx = l.x; ly = l.y; lz = l.z;
            } else {
                tx = v ? (float)(a.tx[i] - cbx) : 0.f;
                ty = v ? (float)(a.ty[i] - cby) : 0.f;
                tz = v ? (float)(a.tz[i] - cbz) : 0.f;
            }
            float fi[OG], sum[OG], cmp[OG];
#pragma unroll
            for (int o = 0; o < OG; o++) {
                const int orb = g0 + o;
                fi[o] = (v && orb < a.norb) ? a.ft32[(long)orb * a.nt + i] : 0.f;
                sum[o] = 0.f;
                cmp[o] = 0.f;
            }
            for (int e = r0; e < r1; e++) {
                const int2 r = a.rng[e];
                if (a.rng_dmin[e] * kmin > 127.f) continue;  // every orbital's term is exactly 0
                const bool close = range_is_close(r);
                if (close != (PASS == 1)) continue;
                const int rb = range_begin(r);
                for (int t0 = rb; t0 < r.y; t0 += GTILE) {
                    const int cnt = min(GTILE, r.y - t0);
                    __syncthreads();
                    for (int j = tid; j < cnt; j += FT) {
                        const int jj = t0 + j;
                        float4 sa, sb;
                        if (PASS == 1) {
                            sa = a.shi[jj];
                            sb = a.slo[jj];
                        } else {
                            sa.x = (float)(a.sx[jj] - cbx);
                            sa.y = (float)(a.sy[jj] - cby);
                            sa.z = (float)(a.sz[jj] - cbz);
                            sb.x = sb.y = sb.z = 0.f;
                        }
                        sa.w = a.w32[jj];
                        sb.w = 0.f;
                        s_xyzw[j] = sa;
                        s_lo[j] = sb;
                    }
                    for (int k = tid; k < cnt * OG; k += FT) {
                        const int j = k / OG, o = k - j * OG;
                        const int orb = g0 + o;
                        reinterpret_cast<float *>(s_q4)[k] = orb < a.norb ? a.q32[(long)orb * a.ns + t0 + j] : 0.f;
                    }
                    __syncthreads();
                    if (!warp_busy) continue;
                    if (PASS == 1)
                        group_tile<SS, true, true, OG>(s_xyzw, s_lo, s_q4, cnt, tx, ty, tz, lx, ly, lz, fi, kc, kl,
                                                       sum, cmp);
                    else
                        group_tile<SS, false, false, OG>(s_xyzw, s_lo, s_q4, cnt, tx, ty, tz, lx, ly, lz, fi, kc,
                                                         kl, sum, cmp);
                }
            }
            if (v) {
#pragma unroll
                for (int o = 0; o < OG; o++)
                    if (g0 + o < a.norb) a.out[(long)(g0 + o) * a.nt + i] = (double)sum[o] - (double)cmp[o];
            }
        }
    }
}

template <bool SS, int MAXN1, int OG>
__global__ void __launch_bounds__(FT, 2) far_group(const __grid_constant__ Work w) {
    constexpr int MAXP = MAXN1 * MAXN1 * MAXN1;
    __shared__ float4 s_q4[MAXP * OG / 4];
    __shared__ float s_w[MAXP];
    __shared__ float s_p[3][MAXN1];
    __shared__ int s_item;
    const int tid = threadIdx.x;
    for (;;) {
        const int item = next_item(w.queue, &s_item);
        if (item >= w.nitems) break;
        const int2 it = w.items[item];
        const Fields &a = w.sys[it.y >> 16];
        const int b = it.x, g0 = it.y & 0xffff;
        const int n1 = a.n1, P = a.P;
        const int f0 = a.far_off[b], f1 = a.far_off[b + 1];
        if (f0 == f1) continue;
        const int bn = a.batch_node[b];
        const int tb = a.tbegin[bn], te = a.tend[bn];
        const double cb[3] = {a.tcenter[3L * bn], a.tcenter[3L * bn + 1], a.tcenter[3L * bn + 2]};
        float kc[OG], kl[OG];
#pragma unroll
        for (int o = 0; o < OG; o++) split_f32((g0 + o) < a.norb ? -a.kp64[g0 + o] * LOG2E : 0.0, kc[o], kl[o]);
        for (int base = tb; base < te; base += FT) {
            const int i = base + tid;
            const bool v = i < te;
            const bool warp_busy = base + (tid & ~31) < te;
            const float tx = v ? (float)(a.tx[i] - cb[0]) : 0.f;
            const float ty = v ? (float)(a.ty[i] - cb[1]) : 0.f;
            const float tz = v ? (float)(a.tz[i] - cb[2]) : 0.f;
            float fi[OG], sum[OG], cmp[OG];
#pragma unroll
            for (int o = 0; o < OG; o++) {
                const int orb = g0 + o;
                fi[o] = (v && orb < a.norb) ? a.ft32[(long)orb * a.nt + i] : 0.f;
                sum[o] = 0.f;
                cmp[o] = 0.f;
            }
            for (int e = f0; e < f1; e++) {
                const int slot = a.node_slot[a.far_list[e]];
                const double *gm = a.geom + 6L * slot;
                __syncthreads();
                for (int k = tid; k < P * OG; k += FT) {
                    const int kk = k / OG, o = k - kk * OG;
                    const int orb = g0 + o;
                    reinterpret_cast<float *>(s_q4)[k] =
                        orb < a.norb ? a.qhat32[((long)orb * a.nslots + slot) * P + kk] : 0.f;
                }
                for (int k = tid; k < P; k += FT) s_w[k] = a.what32[(long)slot * P + k];
                if (tid < 3 * n1) {
                    const int d = tid / n1, m = tid - d * n1;
                    const double cbd = d == 0 ? cb[0] : (d == 1 ? cb[1] : cb[2]);
                    s_p[d][m] = (float)((gm[d] + gm[3 + d] * a.tn[m]) - cbd);
                }
                __syncthreads();
                if (!warp_busy) continue;
                float dz2[MAXN1];
#pragma unroll
                for (int m = 0; m < MAXN1; m++) {
                    const float d = tz - s_p[2][m < n1 ? m : 0];
                    dz2[m] = d * d;
                }
                int idx = 0;
                for (int k1 = 0; k1 < n1; k1++) {
                    float part[OG];
#pragma unroll
                    for (int o = 0; o < OG; o++) part[o] = 0.f;
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
                                const float rr = r2 * rinv;
                                const float wk = s_w[idx + k3];
#pragma unroll
                                for (int o4 = 0; o4 < OG / 4; o4++) {
                                    const float4 q4 = s_q4[(idx + k3) * (OG / 4) + o4];
                                    const float qv[4] = {q4.x, q4.y, q4.z, q4.w};
#pragma unroll
                                    for (int u = 0; u < 4; u++) {
                                        const int o = 4 * o4 + u;
                                        const float g = ex2_mufu(fmaf(kc[o], rr, kl[o] * rr)) * rinv;
                                        part[o] = fmaf(g, SS ? fmaf(-fi[o], wk, qv[u]) : qv[u], part[o]);
                                    }
                                }
                            }
                        }
                        idx += n1;
                    }
#pragma unroll
                    for (int o = 0; o < OG; o++) kahan_add(sum[o], cmp[o], part[o]);
                }
            }
            if (v) {
#pragma unroll
                for (int o = 0; o < OG; o++)
                    if (g0 + o < a.norb) a.out[(long)(g0 + o) * a.nt + i] = (double)sum[o] - (double)cmp[o];
            }
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
__global__ void __launch_bounds__(FT) near_f64(const __grid_constant__ Work w) {
    constexpr int T64 = 256;
    __shared__ double s_x[T64], s_y[T64], s_z[T64], s_f[T64], s_w[T64];
    __shared__ int s_item;
    const int tid = threadIdx.x;
    for (;;) {
        const int item = next_item(w.queue, &s_item);
        if (item >= w.nitems) break;
        const int2 it = w.items[item];
        const Fields &a = w.sys[it.y >> 16];
        const int b = it.x, orb = it.y & 0xffff;
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
                for (int t0 = range_begin(r); t0 < r.y; t0 += T64) {
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
__global__ void __launch_bounds__(FT) far_f64(const __grid_constant__ Work w) {
    constexpr int MAXP = MAXN1 * MAXN1 * MAXN1;
    __shared__ double s_q[MAXP], s_wh[MAXP];
    __shared__ double s_p[3][MAXN1];
    __shared__ int s_item;
    const int tid = threadIdx.x;
    for (;;) {
        const int item = next_item(w.queue, &s_item);
        if (item >= w.nitems) break;
        const int2 it = w.items[item];
        const Fields &a = w.sys[it.y >> 16];
        const int b = it.x, orb = it.y & 0xffff;
        const int n1 = a.n1, P = a.P;
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

// phi_i = near + far + f_i * SS factor, scattered back to caller order.  The
// SS term uses the same f_i the pair sums used (FP32-rounded in mixed mode):
// sum_j w_j (f_j - c) G + c * int G is exact for any constant c, while mixing
// two roundings of f_i would leave delta * f_i * sum_j w_j G in the result.
template <typename TF>
__global__ void epilogue(const double *__restrict__ nearv, const double *__restrict__ near2v,
                         const double *__restrict__ farv, const TF *__restrict__ fsorted,
                         const int *__restrict__ perm, int nt, const double *__restrict__ ss,
                         double *__restrict__ out) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    int orb = blockIdx.y;
    if (i >= nt) return;
    long si = (long)orb * nt + i;
    out[(long)orb * nt + perm[i]] = (nearv[si] + near2v[si]) + farv[si] + ss[orb] * (double)fsorted[si];
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
int launch_persistent(K kern, const Work &w, cudaStream_t s) {
    if (w.nitems == 0) return TAGI_OK;
    int grid = 0;
    TAGI_TRY(occupancy_grid(kern, &grid));
    if (grid > w.nitems) grid = w.nitems;
    if (grid < 1) grid = 1;
    launch(kern, grid, FT, 0, s, w);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

// ---------------------------------------------------------------------------
// Pair-throughput ceiling: the near/far inner loops' arithmetic with operands
// already in shared memory and registers and no global traffic.  The field
// kernels' roofline fraction is measured against this, live, on the same GPU.
// ---------------------------------------------------------------------------
template <int KERN, bool SS>
__global__ void __launch_bounds__(FT) pair_peak_near(int reps, float *out) {
    __shared__ float4 s_a[NTILE];
    __shared__ float4 s_b[NTILE];
    for (int j = threadIdx.x; j < NTILE; j += FT) {
        float v = (float)((j * 37) % 101) * 0.01f - 0.5f;
        s_a[j] = make_float4(v, 0.3f * v + 0.1f, 0.7f - v, 0.5f + 0.001f * j);
        s_b[j] = make_float4(0.f, 0.f, 0.f, 0.25f);
    }
    __syncthreads();
    float tx[2], ty[2], tz[2], fi[2];
    float sum[2] = {0.f, 0.f}, cmp[2] = {0.f, 0.f};
    for (int k = 0; k < 2; k++) {
        tx[k] = 0.01f * (threadIdx.x & 31) + 0.003f * k;
        ty[k] = 0.02f;
        tz[k] = -0.03f * (threadIdx.x >> 5);
        fi[k] = 0.3f;
    }
    for (int r = 0; r < reps; r++)
        near_tile<KERN, SS, false, false, 2>(s_a, s_b, NTILE, tx, ty, tz, nullptr, 1.f, fi, sum, cmp);
    out[blockIdx.x * FT + threadIdx.x] = sum[0] + sum[1] - cmp[0] - cmp[1];
}

template <int KERN, bool SS>
__global__ void __launch_bounds__(FT) pair_peak_far(int reps, float *out) {
    constexpr int N1 = 8;
    __shared__ float2 s_qw[N1 * N1 * N1];
    __shared__ float s_p[3][N1];
    for (int k = threadIdx.x; k < N1 * N1 * N1; k += FT) s_qw[k] = make_float2(0.5f + 0.001f * k, 0.25f);
    if (threadIdx.x < 3 * N1) s_p[threadIdx.x / N1][threadIdx.x % N1] = 1.0f + 0.1f * threadIdx.x;
    __syncthreads();
    float tx[2], ty[2], tz[2], fi[2], sum[2] = {0.f, 0.f}, cmp[2] = {0.f, 0.f};
    for (int k = 0; k < 2; k++) {
        tx[k] = 0.01f * (threadIdx.x & 31) + 0.003f * k;
        ty[k] = 0.02f;
        tz[k] = -0.03f * (threadIdx.x >> 5);
        fi[k] = 0.3f;
    }
    for (int r = 0; r < reps; r++) far_cluster<KERN, SS, true, N1, 2>(s_qw, s_p, N1, tx, ty, tz, fi, sum, cmp);
    out[blockIdx.x * FT + threadIdx.x] = sum[0] + sum[1] - cmp[0] - cmp[1];
}

// Yukawa orbital groups: group_tile over one staged tile, 8 orbitals per
// pair geometry; counted per (pair, orbital).
template <bool SS>
__global__ void __launch_bounds__(FT, 2) pair_peak_near_group(int reps, float *out) {
    constexpr int OG = 8;
    __shared__ float4 s_xyzw[GTILE];
    __shared__ float4 s_lo[GTILE];
    __shared__ float4 s_q4[GTILE * OG / 4];
    for (int j = threadIdx.x; j < GTILE; j += FT) {
        const float v = (float)((j * 37) % 101) * 0.01f - 0.5f;
        s_xyzw[j] = make_float4(v, 0.3f * v + 0.1f, 0.7f - v, 0.25f);
        s_lo[j] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    for (int k = threadIdx.x; k < GTILE * OG; k += FT) reinterpret_cast<float *>(s_q4)[k] = 0.5f + 0.001f * k;
    __syncthreads();
    const float tx = 0.01f * (threadIdx.x & 31), ty = 0.02f, tz = -0.03f * (threadIdx.x >> 5);
    float fi[OG], kc[OG], kl[OG], sum[OG], cmp[OG];
#pragma unroll
    for (int o = 0; o < OG; o++) {
        fi[o] = 0.3f;
        split_f32(-(0.5 + 0.3 * o) * LOG2E, kc[o], kl[o]);
        sum[o] = cmp[o] = 0.f;
    }
    for (int r = 0; r < reps; r++)
        group_tile<SS, false, false, OG>(s_xyzw, s_lo, s_q4, GTILE, tx, ty, tz, 0.f, 0.f, 0.f, fi, kc, kl, sum, cmp);
    float acc = 0.f;
#pragma unroll
    for (int o = 0; o < OG; o++) acc += sum[o] - cmp[o];
    out[blockIdx.x * FT + threadIdx.x] = acc;
}

template <int KERN, bool SS>
int launch_pair_peak(int variant, int grid, int reps, float *out, cudaStream_t s) {
    if (variant == 0) launch(pair_peak_near<KERN, SS>, grid, FT, 0, s, reps, out);
    else if (variant == 1) launch(pair_peak_far<KERN, SS>, grid, FT, 0, s, reps, out);
    else launch(pair_peak_near_group<SS>, grid, FT, 0, s, reps, out);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

template <int KERN, bool SS>
int run_pair_peak(int variant, double *pairs_per_s, cudaStream_t s) {
    if (variant < 0 || variant > 2) return set_error(TAGI_ERR_ARG, "pair peak variant %d (0 near, 1 far, 2 near group)", variant);
    if (variant == 2 && KERN != KERNEL_YUKAWA)
        return set_error(TAGI_ERR_UNSUPPORTED, "orbital-group kernels are Yukawa only");
    int grid = 0;
    if (variant == 0) TAGI_TRY(occupancy_grid(pair_peak_near<KERN, SS>, &grid));
    else if (variant == 1) TAGI_TRY(occupancy_grid(pair_peak_far<KERN, SS>, &grid));
    else TAGI_TRY(occupancy_grid(pair_peak_near_group<SS>, &grid));
    Arena tmp;
    tmp.stream = s;
    float *out = nullptr;
    TAGI_TRY(tmp.alloc(&out, (size_t)grid * FT));
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    // pairs per repetition per thread: two targets x a tile, or one target x a tile x 8 orbitals
    const int per_rep = variant == 0 ? 2 * NTILE : (variant == 1 ? 2 * 512 : GTILE * 8);
    int reps = 16;
    float ms = 0.f;
    int rc = TAGI_OK;
    for (int attempt = 0; attempt < 6; attempt++) {  // grow until the timed launch lasts >= 20 ms
        if ((rc = launch_pair_peak<KERN, SS>(variant, grid, reps, out, s))) break;
        cudaEventRecord(a, s);
        if ((rc = launch_pair_peak<KERN, SS>(variant, grid, reps, out, s))) break;
        cudaEventRecord(b, s);
        if (cudaEventSynchronize(b) != cudaSuccess) { rc = set_error(TAGI_ERR_CUDA, "pair peak launch failed"); break; }
        cudaEventElapsedTime(&ms, a, b);
        if (ms >= 20.f) break;
        reps *= 4;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    tmp.release();
    if (rc) return rc;
    *pairs_per_s = (double)grid * FT * per_rep * reps / (ms * 1e-3);
    return TAGI_OK;
}

// Kernel shape shared by every system of one field launch.
struct LaunchShape {
    int og = 1;     // orbitals per item (orbital-group kernels) or 1
    int nt = 1;     // targets per thread: 2 when some batch holds more than FT targets
    int maxn1 = 1;  // largest proxy-grid edge n + 1
};

template <int KERN, bool SS>
int launch_fields(const SysCall *calls, const Fields *f, int nsys, const Schedule &sc, const LaunchShape &sh,
                  int precision, int *queue, cudaStream_t s) {
    Work wn{};
    wn.queue = queue;
    for (int i = 0; i < nsys; i++) wn.sys[i] = f[i];
    Work wc = wn, wf = wn;
    for (int i = 0; i < nsys; i++) {
        wn.sys[i].out = calls[i].p->near_out;
        wc.sys[i].out = calls[i].p->near2_out;
        wf.sys[i].out = calls[i].p->far_out;
    }
    wn.items = sc.items + sc.off[0];
    wn.nitems = sc.count[0];
    wc.items = sc.items + sc.off[1];
    wc.nitems = sc.count[1];
    wc.queue = queue + 2;
    wf.items = sc.items + sc.off[2];
    wf.nitems = sc.count[2];
    wf.queue = queue + 1;
    const bool one = sh.nt == 1;
    phase_mark(PH_NEAR, true, s);
    if (precision == PREC_MIXED && KERN == KERNEL_YUKAWA && sh.og > 1) {
        // orbital groups share the geometry of each pair across og orbitals
        const bool g8 = sh.og == 8;
        if (g8) TAGI_TRY(launch_persistent(near_group<SS, 8, 0>, wn, s));
        else TAGI_TRY(launch_persistent(near_group<SS, 4, 0>, wn, s));
        phase_mark(PH_NEAR, false, s);
        phase_mark(PH_NEAR_CLOSE, true, s);
        if (g8) TAGI_TRY(launch_persistent(near_group<SS, 8, 1>, wc, s));
        else TAGI_TRY(launch_persistent(near_group<SS, 4, 1>, wc, s));
        phase_mark(PH_NEAR_CLOSE, false, s);
        phase_mark(PH_FAR, true, s);
        if (sh.maxn1 <= 4) {
            if (g8) TAGI_TRY(launch_persistent(far_group<SS, 4, 8>, wf, s));
            else TAGI_TRY(launch_persistent(far_group<SS, 4, 4>, wf, s));
        } else if (sh.maxn1 <= 8) {
            if (g8) TAGI_TRY(launch_persistent(far_group<SS, 8, 8>, wf, s));
            else TAGI_TRY(launch_persistent(far_group<SS, 8, 4>, wf, s));
        } else {
            if (g8) TAGI_TRY(launch_persistent(far_group<SS, MAX_DEGREE + 1, 8>, wf, s));
            else TAGI_TRY(launch_persistent(far_group<SS, MAX_DEGREE + 1, 4>, wf, s));
        }
        phase_mark(PH_FAR, false, s);
        return TAGI_OK;
    }
    if (precision == PREC_MIXED) {
        if (one) TAGI_TRY(launch_persistent(near_mixed<KERN, SS, 1, 0>, wn, s));
        else TAGI_TRY(launch_persistent(near_mixed<KERN, SS, 2, 0>, wn, s));
        phase_mark(PH_NEAR, false, s);
        phase_mark(PH_NEAR_CLOSE, true, s);
        if (one) TAGI_TRY(launch_persistent(near_mixed<KERN, SS, 1, 1>, wc, s));
        else TAGI_TRY(launch_persistent(near_mixed<KERN, SS, 2, 1>, wc, s));
        phase_mark(PH_NEAR_CLOSE, false, s);
    } else {
        // one FP64 pass over all near ranges, close ones included
        TAGI_TRY(launch_persistent(near_f64<KERN, SS>, wn, s));
        phase_mark(PH_NEAR, false, s);
    }
    phase_mark(PH_FAR, true, s);
    if (precision == PREC_MIXED) {
        if (one) {
            if (sh.maxn1 <= 4) TAGI_TRY(launch_persistent(far_mixed<KERN, SS, 4, 1>, wf, s));
            else if (sh.maxn1 <= 8) TAGI_TRY(launch_persistent(far_mixed<KERN, SS, 8, 1>, wf, s));
            else TAGI_TRY(launch_persistent(far_mixed<KERN, SS, MAX_DEGREE + 1, 1>, wf, s));
        } else {
            if (sh.maxn1 <= 4) TAGI_TRY(launch_persistent(far_mixed<KERN, SS, 4, 2>, wf, s));
            else if (sh.maxn1 <= 8) TAGI_TRY(launch_persistent(far_mixed<KERN, SS, 8, 2>, wf, s));
            else TAGI_TRY(launch_persistent(far_mixed<KERN, SS, MAX_DEGREE + 1, 2>, wf, s));
        }
    } else {
        if (sh.maxn1 <= 4) TAGI_TRY(launch_persistent(far_f64<KERN, SS, 4>, wf, s));
        else if (sh.maxn1 <= 8) TAGI_TRY(launch_persistent(far_f64<KERN, SS, 8>, wf, s));
        else TAGI_TRY(launch_persistent(far_f64<KERN, SS, MAX_DEGREE + 1>, wf, s));
    }
    phase_mark(PH_FAR, false, s);
    return TAGI_OK;
}

// Per-orbital constants from kernel parameter kp[o * nkp] (host-copied or
// caller's device array): d_kp = k (or a), d_kc = coordinate scale sc,
// d_ss = subtraction factor 4 pi/k^2 (Yukawa) or 2 pi/a^2 (Coulomb), 0
// without subtraction.  A parameter the kernel cannot use sets bit 0 of err
// and makes the orbital's subtraction factor NaN, so all its outputs are NaN.
__global__ void orbital_constants(const double *__restrict__ kp, int nkp, int norb, int kernel, int sing,
                                  double *__restrict__ kpo, float *__restrict__ kc, double *__restrict__ ss,
                                  int *__restrict__ err) {
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= norb) return;
    const double k = kp[(long)o * nkp];
    const bool used = kernel == KERNEL_YUKAWA || sing == SING_SUBTRACTION;
    const bool bad = !isfinite(k) || (used && !(k > 0.0));
    if (bad) atomicOr(err, 1);
    kpo[o] = k;
    float c = 1.0f;
    if (kernel == KERNEL_YUKAWA) c = (float)(k * LOG2E);
    else if (sing == SING_SUBTRACTION) c = (float)(k * sqrt(LOG2E));
    kc[o] = c;
    double f = 0.0;
    if (sing == SING_SUBTRACTION) f = (kernel == KERNEL_YUKAWA ? 4.0 : 2.0) * M_PI / (k * k);
    ss[o] = bad ? __longlong_as_double(0x7ff8000000000000LL) : f;  // NaN marks every output of the orbital
}

Fields make_fields(const Plan &p, int norb) {
    Fields a{};
    a.tx = p.tgt.x;
    a.ty = p.tgt.y;
    a.tz = p.tgt.z;
    a.tbegin = p.tgt.begin;
    a.tend = p.tgt.end;
    a.tcenter = p.tgt.center;
    a.tradius = p.tgt.radius;
    a.batch_node = p.batch_node;
    a.nbatch = p.nbatch;
    a.nt = p.tgt.n;
    a.norb = norb;
    a.rng_off = p.rng_off;
    a.rng = p.rng;
    a.rng_dmin = p.rng_dmin;
    a.sx = p.src.x;
    a.sy = p.src.y;
    a.sz = p.src.z;
    a.shi = p.src_hi;
    a.slo = p.src_lo;
    a.thi = p.tgt_hi;
    a.tlo = p.tgt_lo;
    a.ns = p.src.n;
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
    return a;
}

}  // namespace

bool stream_capturing(cudaStream_t s) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &st) != cudaSuccess) return false;
    return st == cudaStreamCaptureStatusActive;
}

// Per-call scratch for norb orbitals.  Growing it is rare (a larger orbital
// count than any earlier call) and synchronizes the device first: the old
// buffers may still be in use by calls on any stream.  Plain cudaMalloc keeps
// the new buffers valid on every stream.
int ensure_scratch(Plan &p, int norb) {
    if ((size_t)norb <= p.scratch_orbitals) return TAGI_OK;
    TAGI_CUDA(cudaDeviceSynchronize());
    for (void *v : p.scratch) cudaFree(v);
    p.scratch.clear();
    p.scratch_orbitals = 0;
    const size_t ns = p.src.n, nt = p.tgt.n, no = norb;
    auto alloc = [&](auto **ptr, size_t count) -> int {
        void *v = nullptr;
        const size_t bytes = (count ? count : 1) * sizeof(**ptr);
        cudaError_t e = cudaMalloc(&v, bytes);
        if (e != cudaSuccess)
            return set_error(TAGI_ERR_CUDA, "device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
        p.scratch.push_back(v);
        *ptr = static_cast<std::remove_reference_t<decltype(**ptr)> *>(v);
        return TAGI_OK;
    };
    TAGI_TRY(alloc(&p.q32, no * ns));
    TAGI_TRY(alloc(&p.ft32, no * nt));
    TAGI_TRY(alloc(&p.q64, no * ns));
    TAGI_TRY(alloc(&p.f64s, no * ns));
    TAGI_TRY(alloc(&p.ft64, no * nt));
    TAGI_TRY(alloc(&p.part, no * p.nitems * p.P));
    TAGI_TRY(alloc(&p.qhat32, no * p.nslots * p.P));
    TAGI_TRY(alloc(&p.qhat64, no * p.nslots * p.P));
    TAGI_TRY(alloc(&p.near_out, no * nt));
    TAGI_TRY(alloc(&p.near2_out, no * nt));
    TAGI_TRY(alloc(&p.far_out, no * nt));
    TAGI_TRY(alloc(&p.d_kc, no));
    TAGI_TRY(alloc(&p.d_kp, no));
    TAGI_TRY(alloc(&p.d_ss, no));
    p.scratch_orbitals = no;
    return TAGI_OK;
}

// Orbitals per work item: Yukawa in mixed precision shares each pair's
// geometry across a group of 8 (or 4) orbitals once the largest system has
// that many; everything else runs one orbital per item.  requested > 0
// (1, 4 or 8) overrides the choice where the kernel supports it.
int orbitals_per_item(int kernel, int precision, int max_norb, int requested) {
    if (kernel != KERNEL_YUKAWA || precision != PREC_MIXED) return 1;
    if (requested == 1 || requested == 4 || requested == 8) return requested;
    return max_norb >= 8 ? 8 : (max_norb >= 4 ? 4 : 1);
}

bool schedule_matches(const Schedule &sc, const int *norb, int nsys, int og) {
    if (sc.og != og || (int)sc.norb.size() != nsys) return false;
    for (int i = 0; i < nsys; i++)
        if (sc.norb[i] != norb[i]) return false;
    return true;
}

// Work lists for one launch over nsys systems: one item per (system, batch,
// group of og orbitals), ordered by pair count times orbitals in the item,
// heaviest first (ties in system, batch, group order).  Passes that have
// nothing to do for a batch (no close ranges, no far entries) get no item:
// their outputs are cleared before the launch.
int build_schedule(Plan *const *plans, const int *norb, int nsys, int og, Schedule &sc, cudaStream_t s) {
    if (nsys < 1 || nsys > MAX_SYSTEMS) return set_error(TAGI_ERR_ARG, "%d systems (1..%d per launch)", nsys, MAX_SYSTEMS);
    struct It {
        long long cost;
        int2 v;
    };
    std::vector<It> lists[3];
    for (int i = 0; i < nsys; i++) {
        const Plan &p = *plans[i];
        if (norb[i] < 1 || norb[i] > 0xffff) return set_error(TAGI_ERR_ARG, "system %d: %d orbitals", i, norb[i]);
        if ((int)p.cost_near.size() != p.nbatch) return set_error(TAGI_ERR_STATE, "plan without batch costs");
        for (int b = 0; b < p.nbatch; b++)
            for (int g0 = 0; g0 < norb[i]; g0 += og) {
                const long long lanes = og;
                const int2 v = make_int2(b, (i << 16) | g0);
                lists[0].push_back({p.cost_near[b] * lanes, v});
                if (p.cost_close[b] > 0) lists[1].push_back({p.cost_close[b] * lanes, v});
                if (p.cost_far[b] > 0) lists[2].push_back({p.cost_far[b] * lanes, v});
            }
    }
    std::vector<int2> all;
    for (int k = 0; k < 3; k++) {
        std::stable_sort(lists[k].begin(), lists[k].end(), [](const It &a, const It &b) { return a.cost > b.cost; });
        sc.off[k] = (long)all.size();
        sc.count[k] = (int)lists[k].size();
        for (const It &it : lists[k]) all.push_back(it.v);
    }
    // the old list may be in use on any stream: wait, then replace it
    TAGI_CUDA(cudaDeviceSynchronize());
    sc.release();
    if (all.empty()) all.push_back(make_int2(0, 0));
    void *v = nullptr;
    TAGI_CUDA(cudaMalloc(&v, sizeof(int2) * all.size()));
    sc.items = static_cast<int2 *>(v);
    // pageable source: the copy has read it when the call returns
    TAGI_CUDA(cudaMemcpyAsync(sc.items, all.data(), sizeof(int2) * all.size(), cudaMemcpyHostToDevice, s));
    sc.og = og;
    sc.norb.assign(norb, norb + nsys);
    return TAGI_OK;
}

// Per-orbital constants of one system into p.d_kp / d_kc / d_ss.
static int orbital_setup(Plan &p, const SysCall &c, int kernel, int singularity, cudaStream_t s) {
    const double *src = c.kp;
    int stride = c.nkp;
    if (!c.kp_device) {
        p.h_kp.resize(c.norb);
        for (int o = 0; o < c.norb; o++) p.h_kp[o] = c.kp[(long)o * c.nkp];
        TAGI_CUDA(cudaMemcpyAsync(p.d_kp, p.h_kp.data(), sizeof(double) * c.norb, cudaMemcpyHostToDevice, s));
        src = p.d_kp;
        stride = 1;
    }
    launch(orbital_constants, (c.norb + 127) / 128, 128, 0, s, src, stride, c.norb, kernel, singularity, p.d_kp,
           p.d_kc, p.d_ss, p.err_flag + 1);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

// One convolution call over nsys systems (1..MAX_SYSTEMS) sharing kernel,
// singularity handling and precision: per-system glue and upward pass, then
// ONE persistent launch per field pass across all systems, then per-system
// epilogues.  Under stream capture nothing may allocate or copy from host
// memory: scratch, schedule and FP64 weight charges must exist already, and
// kernel parameters must be on the device.
int convolve_systems(SysCall *calls, int nsys, int kernel, int singularity, int precision, const Schedule &sc,
                     int *queue, cudaStream_t s, int nt_request) {
    if (nsys < 1 || nsys > MAX_SYSTEMS) return set_error(TAGI_ERR_ARG, "%d systems (1..%d per launch)", nsys, MAX_SYSTEMS);
    const bool mixed = precision == PREC_MIXED;
    const bool ss = singularity == SING_SUBTRACTION;
    const bool capturing = stream_capturing(s);
    Fields f[MAX_SYSTEMS];
    LaunchShape sh;
    sh.og = sc.og;
    for (int i = 0; i < nsys; i++) {
        SysCall &c = calls[i];
        Plan &p = *c.p;
        if (capturing) {
            if ((size_t)c.norb > p.scratch_orbitals || (!mixed && p.nslots && !p.what64_ready) || !c.kp_device)
                return set_error(TAGI_ERR_STATE,
                                 "graph capture needs a prior uncaptured call with the same orbital counts and "
                                 "precision, and kernel parameters on the device");
        }
        TAGI_TRY(ensure_scratch(p, c.norb));
        TAGI_TRY(orbital_setup(p, c, kernel, singularity, s));
        const int ns = p.src.n, nt = p.tgt.n;
        dim3 gs((ns + 255) / 256, c.norb), gt((nt + 255) / 256, c.norb);
        phase_mark(PH_GLUE, true, s);
        launch(prep_sources, gs, 256, 0, s, c.sv, p.src.perm, p.sw64, ns, c.norb, p.q32, p.q64, p.f64s);
        launch(prep_targets, gt, 256, 0, s, c.tv, p.tgt.perm, nt, p.ft32, p.ft64);
        phase_mark(PH_GLUE, false, s);
        TAGI_LAUNCH_CHECK();
        phase_mark(PH_UPWARD, true, s);
        TAGI_TRY(modified_charges(p, mixed ? PREC_MIXED : PREC_FP64, c.norb, s));
        if (!mixed) TAGI_TRY(ensure_weight_charges64(p, s));  // before what64 is read below
        phase_mark(PH_UPWARD, false, s);
        if (!mixed && p.nslots && !p.what64) return set_error(TAGI_ERR_DEVICE, "FP64 weight charges missing");
        f[i] = make_fields(p, c.norb);
        if (p.max_batch > FT) sh.nt = 2;  // automatic: two targets per thread for batches above FT
        if (p.n1 > sh.maxn1) sh.maxn1 = p.n1;
        // the far and close-range passes write only the batches they visit
        TAGI_CUDA(cudaMemsetAsync(p.far_out, 0, sizeof(double) * (size_t)c.norb * nt, s));
        TAGI_CUDA(cudaMemsetAsync(p.near2_out, 0, sizeof(double) * (size_t)c.norb * nt, s));
    }
    if (nt_request == 1 || nt_request == 2) sh.nt = nt_request;
    TAGI_CUDA(cudaMemsetAsync(queue, 0, 3 * sizeof(int), s));
    if (kernel == KERNEL_YUKAWA) {
        if (ss) TAGI_TRY((launch_fields<KERNEL_YUKAWA, true>(calls, f, nsys, sc, sh, precision, queue, s)));
        else TAGI_TRY((launch_fields<KERNEL_YUKAWA, false>(calls, f, nsys, sc, sh, precision, queue, s)));
    } else {
        if (ss) TAGI_TRY((launch_fields<KERNEL_COULOMB, true>(calls, f, nsys, sc, sh, precision, queue, s)));
        else TAGI_TRY((launch_fields<KERNEL_COULOMB, false>(calls, f, nsys, sc, sh, precision, queue, s)));
    }
    phase_mark(PH_GLUE, true, s);
    for (int i = 0; i < nsys; i++) {
        const SysCall &c = calls[i];
        const Plan &p = *c.p;
        const int nt = p.tgt.n;
        dim3 gt((nt + 255) / 256, c.norb);
        if (mixed)
            launch(epilogue<float>, gt, 256, 0, s, p.near_out, p.near2_out, p.far_out, p.ft32, p.tgt.perm, nt,
                   p.d_ss, c.out);
        else
            launch(epilogue<double>, gt, 256, 0, s, p.near_out, p.near2_out, p.far_out, p.ft64, p.tgt.perm, nt,
                   p.d_ss, c.out);
    }
    phase_mark(PH_GLUE, false, s);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

// Single-plan call (norb orbitals over one mesh) with the plan's cached
// work list.
int convolve(Plan &p, const double *tv, const double *sv, double *out, int norb, int kernel,
             const double *kparams, int nkp, int singularity, int precision, cudaStream_t s, bool kp_device,
             int og_request, int nt_request) {
    const int og = orbitals_per_item(kernel, precision, norb, og_request);
    const Schedule *sc = nullptr;
    for (const Schedule &c : p.scheds)
        if (schedule_matches(c, &norb, 1, og)) sc = &c;
    if (!sc) {
        if (stream_capturing(s))
            return set_error(TAGI_ERR_STATE, "graph capture needs a prior uncaptured call with the same orbital count");
        constexpr size_t KEEP = 4;  // work lists kept per plan (e.g. Hartree + orbital batch)
        if (p.scheds.size() >= KEEP) {
            TAGI_CUDA(cudaDeviceSynchronize());
            p.scheds.front().release();
            p.scheds.erase(p.scheds.begin());
        }
        p.scheds.emplace_back();
        Plan *pp = &p;
        const int rc = build_schedule(&pp, &norb, 1, og, p.scheds.back(), s);
        if (rc) {
            p.scheds.back().release();
            p.scheds.pop_back();
            return rc;
        }
        sc = &p.scheds.back();
    }
    SysCall c;
    c.p = &p;
    c.tv = tv;
    c.sv = sv;
    c.out = out;
    c.norb = norb;
    c.kp = kparams;
    c.nkp = nkp;
    c.kp_device = kp_device;
    return convolve_systems(&c, 1, kernel, singularity, precision, *sc, p.queue, s, nt_request);
}

int pair_peak(int kernel, int singularity, int variant, double kp, double *pairs_per_s, cudaStream_t s) {
    (void)kp;
    const bool ss = singularity == SING_SUBTRACTION;
    if (kernel == KERNEL_YUKAWA)
        return ss ? run_pair_peak<KERNEL_YUKAWA, true>(variant, pairs_per_s, s)
                  : run_pair_peak<KERNEL_YUKAWA, false>(variant, pairs_per_s, s);
    return ss ? run_pair_peak<KERNEL_COULOMB, true>(variant, pairs_per_s, s)
              : run_pair_peak<KERNEL_COULOMB, false>(variant, pairs_per_s, s);
}

}  // namespace tagi
