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
__device__ __forceinline__ float lg2_mufu(float x) {
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
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

// Packed FP32 pairs.  On the sm_100 family one FADD2 / FMUL2 / FFMA2
// instruction applies the same round-to-nearest IEEE operation to two lanes
// held in a register pair, so the pair arithmetic takes half the issue slots
// of its scalar form with bit-identical per-lane results.  The field kernels
// pack two SOURCES (near field) or two proxy points (far field) per
// operation; a target's own values are duplicated once into both lanes.
__device__ __forceinline__ float2 dup2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 rsqrt2(float2 a) { return make_float2(rsqrt_mufu(a.x), rsqrt_mufu(a.y)); }
// 2^{-a} per lane
__device__ __forceinline__ float2 ex2neg2(float2 a) { return make_float2(ex2_mufu(-a.x), ex2_mufu(-a.y)); }
// 2^{a} per lane
__device__ __forceinline__ float2 ex2pos2(float2 a) { return make_float2(ex2_mufu(a.x), ex2_mufu(a.y)); }
// -log2(r) = -log2(r^2) / 2 per lane
__device__ __forceinline__ float2 nlog2r2(float2 r2) {
    return mul2(dup2(-0.5f), make_float2(lg2_mufu(r2.x), lg2_mufu(r2.y)));
}

// Two pairs (one target, two sources) from their squared scaled distances
// r2 = r'^2; q, w the two sources' charges and weights, nfi = -f_i in both
// lanes.  Per lane:
//   Yukawa   acc += 2^{-r'} / r' * (SS ? q - f_i w : q)
//   Coulomb  acc += (SS ? q - f_i 2^{-r'^2} w : q) / r'
// MASK zeroes a coincident (r = 0) pair.
template <int KERN, bool SS, bool MASK>
__device__ __forceinline__ float2 pair2(float2 r2, float2 q, float2 w, float2 nfi, float2 acc) {
    float2 rinv = rsqrt2(r2);
    if (MASK) {
        rinv.x = r2.x > 0.f ? rinv.x : 0.f;
        rinv.y = r2.y > 0.f ? rinv.y : 0.f;
    }
    if (KERN == KERNEL_YUKAWA) {
        const float2 g = mul2(ex2neg2(mul2(r2, rinv)), rinv);
        return fma2(g, SS ? fma2(nfi, w, q) : q, acc);
    } else if (SS) {
        return fma2(rinv, fma2(mul2(nfi, ex2neg2(r2)), w, q), acc);
    } else {
        return fma2(rinv, q, acc);
    }
}

// Compensated (Kahan) addition of an FP32 partial into (sum, cmp).
__device__ __forceinline__ void kahan_add(float &sum, float &cmp, float part) {
    const float y = part - cmp;
    const float t = sum + y;
    cmp = (t - sum) - y;
    sum = t;
}

__device__ __forceinline__ float4 lds4(const float *p) { return *reinterpret_cast<const float4 *>(p); }
__device__ __forceinline__ float2 lds2(const float *p) { return *reinterpret_cast<const float2 *>(p); }

// Near-field source tile in shared memory, structure of arrays, NEGATED
// coordinates so that one FADD2 forms t - s for two sources:
//   row 0..2  -x, -y, -z   (ordinary tiles: scaled batch-relative FP32;
//                           PRECISE tiles: hi parts of the absolute FP64
//                           coordinates' FP32 splits)
//   row 3, 4  charge q = f w, weight w
//   row 5..7  -lo parts of the splits (PRECISE tiles only)
// A tile of cnt sources is padded to cnt4 = a multiple of 4 with copies of
// its first source carrying q = w = 0: their terms are exactly +-0.
//
// One tile against NT targets, two sources per packed operation.  Pairs are
// summed in FP32 per lane over chunks of KCHUNK sources; each chunk's two
// lane sums are added and the result enters the target's Kahan sum: a long
// FP32 run loses ~sqrt(n) u of its total, and singularity subtraction
// multiplies that loss by |f_i int G| / |phi_i| (often 10-100).
// PRECISE tiles (close ranges): each difference is (t_hi - s_hi) +
// (t_lo - s_lo) -- exact hi differences for nearby points -- and the
// unscaled r^2 is multiplied by sc2 = sc^2, so the shortest pairs keep FP32
// relative precision in r whatever the batch size.
constexpr int KCHUNK = 64;
constexpr int NROWS_PRECISE = 8;
template <int KERN, bool SS, bool MASK, bool PRECISE, int NT>
__device__ __forceinline__ void near_tile(const float (*__restrict__ s)[NTILE], int cnt4, const float2 (&tx)[NT],
                                          const float2 (&ty)[NT], const float2 (&tz)[NT], const float2 (&lx)[NT],
                                          const float2 (&ly)[NT], const float2 (&lz)[NT], float2 sc2,
                                          const float2 (&nfi)[NT], float (&sum)[NT], float (&cmp)[NT]) {
    for (int j0 = 0; j0 < cnt4; j0 += KCHUNK) {
        const int j1 = min(j0 + KCHUNK, cnt4);
        float2 part[NT];
#pragma unroll
        for (int k = 0; k < NT; k++) part[k] = make_float2(0.f, 0.f);
#pragma unroll 2
        for (int j = j0; j < j1; j += 4) {
            const float4 X = lds4(s[0] + j), Y = lds4(s[1] + j), Z = lds4(s[2] + j);
            const float4 Q = lds4(s[3] + j), W = lds4(s[4] + j);
            float4 XL = make_float4(0.f, 0.f, 0.f, 0.f), YL = XL, ZL = XL;
            if constexpr (PRECISE) {
                XL = lds4(s[5] + j);
                YL = lds4(s[6] + j);
                ZL = lds4(s[7] + j);
            }
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const float2 sx = h ? make_float2(X.z, X.w) : make_float2(X.x, X.y);
                const float2 sy = h ? make_float2(Y.z, Y.w) : make_float2(Y.x, Y.y);
                const float2 sz = h ? make_float2(Z.z, Z.w) : make_float2(Z.x, Z.y);
                const float2 q = h ? make_float2(Q.z, Q.w) : make_float2(Q.x, Q.y);
                const float2 w = h ? make_float2(W.z, W.w) : make_float2(W.x, W.y);
                const float2 sxl = h ? make_float2(XL.z, XL.w) : make_float2(XL.x, XL.y);
                const float2 syl = h ? make_float2(YL.z, YL.w) : make_float2(YL.x, YL.y);
                const float2 szl = h ? make_float2(ZL.z, ZL.w) : make_float2(ZL.x, ZL.y);
#pragma unroll
                for (int k = 0; k < NT; k++) {
                    float2 dx = add2(tx[k], sx), dy = add2(ty[k], sy), dz = add2(tz[k], sz);
                    if (PRECISE) {
                        dx = add2(dx, add2(lx[k], sxl));
                        dy = add2(dy, add2(ly[k], syl));
                        dz = add2(dz, add2(lz[k], szl));
                    }
                    float2 r2 = fma2(dx, dx, fma2(dy, dy, mul2(dz, dz)));
                    if (PRECISE) r2 = mul2(r2, sc2);
                    part[k] = pair2<KERN, SS, MASK>(r2, q, w, nfi[k], part[k]);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < NT; k++) kahan_add(sum[k], cmp[k], part[k].x + part[k].y);
    }
}


// ---------------------------------------------------------------------------
// Near field, mixed precision.
// ---------------------------------------------------------------------------
// PASS 0 handles the ordinary near ranges, PASS 1 the close ones (double-float
// coordinates, r = 0 mask) into a second output; two passes keep each
// kernel's register footprint at one tile variant's.
#ifndef TAGI_NEAR_MINB
#define TAGI_NEAR_MINB 3   // resident CTAs per SM the near kernel is compiled for
#endif
template <int KERN, bool SS, int NT, int PASS>
__global__ void __launch_bounds__(FT, TAGI_NEAR_MINB) near_mixed(const __grid_constant__ Work w) {
    constexpr int NR = PASS == 1 ? NROWS_PRECISE : 5;
    __shared__ __align__(16) float s_src[NR][NTILE];
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
        const double cbx = a.tcenter[3L * bn], cby = a.tcenter[3L * bn + 1],
                     cbz = a.tcenter[3L * bn + 2];
        const float scf = a.kc32[orb];
        const double sc = (double)scf;
        const float2 sc2 = dup2((float)(sc * sc));
        const float *q = a.q32 + (long)orb * a.ns;
        const float *ft = a.ft32 + (long)orb * a.nt;
        const int r0 = a.rng_off[b], r1 = a.rng_off[b + 1];
        for (int base = tb; base < te; base += FT * NT) {
            // consecutive targets per thread: the threads with targets form a
            // prefix, so whole warps past it have none and skip the pair loops
            const bool warp_busy = base + NT * (tid & ~31) < te;
            float2 tx[NT], ty[NT], tz[NT], lx[NT], ly[NT], lz[NT], nfi[NT];
            float sum[NT], cmp[NT];
#pragma unroll
            for (int k = 0; k < NT; k++) {
                const int i = base + NT * tid + k;
                const bool v = i < te;
                if (PASS == 1) {
                    const float4 h = v ? a.thi[i] : make_float4(0.f, 0.f, 0.f, 0.f);
                    const float4 l = v ? a.tlo[i] : make_float4(0.f, 0.f, 0.f, 0.f);
                    tx[k] = dup2(h.x);
                    ty[k] = dup2(h.y);
                    tz[k] = dup2(h.z);
                    lx[k] = dup2(l.x);
                    ly[k] = dup2(l.y);
                    lz[k] = dup2(l.z);
                } else {
                    tx[k] = dup2(v ? (float)((a.tx[i] - cbx) * sc) : 0.f);
                    ty[k] = dup2(v ? (float)((a.ty[i] - cby) * sc) : 0.f);
                    tz[k] = dup2(v ? (float)((a.tz[i] - cbz) * sc) : 0.f);
                    lx[k] = ly[k] = lz[k] = dup2(0.f);
                }
                nfi[k] = dup2(v ? -ft[i] : 0.f);
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
                    const int cnt4 = (cnt + 3) & ~3;
                    __syncthreads();
                    for (int j = tid; j < cnt4; j += FT) {
                        const bool real = j < cnt;
                        const int jj = t0 + (real ? j : 0);   // padding: a copy of the first source
                        if constexpr (PASS == 1) {
                            const float4 h = a.shi[jj], l = a.slo[jj];
                            s_src[0][j] = -h.x;
                            s_src[1][j] = -h.y;
                            s_src[2][j] = -h.z;
                            s_src[5][j] = -l.x;
                            s_src[6][j] = -l.y;
                            s_src[7][j] = -l.z;
                        } else {
                            s_src[0][j] = -(float)((a.sx[jj] - cbx) * sc);
                            s_src[1][j] = -(float)((a.sy[jj] - cby) * sc);
                            s_src[2][j] = -(float)((a.sz[jj] - cbz) * sc);
                        }
                        s_src[3][j] = real ? q[jj] : 0.f;
                        s_src[4][j] = real ? a.w32[jj] : 0.f;
                    }
                    __syncthreads();
                    if (!warp_busy) continue;
                    if (PASS == 1)
                        near_tile<KERN, SS, true, true, NT>(s_src, cnt4, tx, ty, tz, lx, ly, lz, sc2, nfi, sum, cmp);
                    else if (noexp)
                        near_tile<KERN, false, false, false, NT>(s_src, cnt4, tx, ty, tz, lx, ly, lz, sc2, nfi, sum,
                                                                 cmp);
                    else
                        near_tile<KERN, SS, false, false, NT>(s_src, cnt4, tx, ty, tz, lx, ly, lz, sc2, nfi, sum,
                                                              cmp);
                }
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
// Far field, mixed precision.  The proxy grid is a tensor product, so r'^2
// is assembled from per-axis squares: one packed add per two proxy points.
// Two proxy points along the innermost axis share each packed operation; the
// staged charges and weights have that axis padded to an even length n1p
// (padding: charge and weight 0, the distance of the first point).  Coulomb
// subtraction: when the whole cluster lies so far that r'^2 > 40 for every
// proxy point, the Gaussian term f_i what_k 2^{-r'^2} is below 2^-40 of
// f_i what_k and is dropped (one MUFU op less per pair); Yukawa clusters
// with r' > 127 everywhere add exactly 0 in FP32 (2^{-r'} flushes to zero)
// and are skipped.
// ---------------------------------------------------------------------------
template <int MAXN1>
__host__ __device__ constexpr int even_up() { return MAXN1 + (MAXN1 & 1); }

template <int KERN, bool SS, bool EXPTERM, int MAXN1, int NT, bool EXACT = false>
__device__ __forceinline__ void far_cluster(const float *__restrict__ s_q, const float *__restrict__ s_w,
                                            const float (*s_p)[MAXN1], int n1_in, const float (&tx)[NT],
                                            const float (&ty)[NT], const float (&tz)[NT],
                                            const float2 (&nfi)[NT], float (&sum)[NT], float (&cmp)[NT]) {
    constexpr int MH = even_up<MAXN1>() / 2;
    constexpr bool PSS = KERN == KERNEL_YUKAWA ? SS : (SS && EXPTERM);
    const int n1 = EXACT ? MAXN1 : n1_in;   // EXACT: every loop bound known at compile time
    const int n1p = n1 + (n1 & 1);
    float2 dz2[NT][MH];
#pragma unroll
    for (int k = 0; k < NT; k++)
#pragma unroll
        for (int m = 0; m < MH; m++) {
            const float d0 = tz[k] - s_p[2][2 * m < n1 ? 2 * m : 0];
            const float d1 = tz[k] - s_p[2][2 * m + 1 < n1 ? 2 * m + 1 : 0];
            dz2[k][m] = make_float2(d0 * d0, d1 * d1);
        }
    int idx = 0;
    for (int k1 = 0; k1 < n1; k1++) {  // one (n+1)^2 slab per FP32 partial, then Kahan
        float2 part[NT];
        float dx2[NT];
#pragma unroll
        for (int k = 0; k < NT; k++) {
            part[k] = make_float2(0.f, 0.f);
            const float dx = tx[k] - s_p[0][k1];
            dx2[k] = dx * dx;
        }
        for (int k2 = 0; k2 < n1; k2++) {
            float2 rxy[NT];
#pragma unroll
            for (int k = 0; k < NT; k++) {
                const float dy = ty[k] - s_p[1][k2];
                rxy[k] = dup2(fmaf(dy, dy, dx2[k]));
            }
#pragma unroll
            for (int m = 0; m < MH; m++) {
                if (2 * m < n1) {
                    const float2 q = lds2(s_q + idx + 2 * m), wv = lds2(s_w + idx + 2 * m);
#pragma unroll
                    for (int k = 0; k < NT; k++)
                        part[k] = pair2<KERN, PSS, false>(add2(rxy[k], dz2[k][m]), q, wv, nfi[k], part[k]);
                }
            }
            idx += n1p;
        }
#pragma unroll
        for (int k = 0; k < NT; k++) kahan_add(sum[k], cmp[k], part[k].x + part[k].y);
    }
}

// EXACT: every system of the launch has n + 1 = MAXN1 (the loops over the
// proxy grid are then fully known at compile time).
template <int KERN, bool SS, int MAXN1, int NT, bool EXACT = false>
__global__ void __launch_bounds__(FT, 2) far_mixed(const __grid_constant__ Work w) {
    constexpr int MAXPP = MAXN1 * MAXN1 * even_up<MAXN1>();
    __shared__ __align__(16) float s_q[MAXPP];
    __shared__ __align__(16) float s_w[MAXPP];
    __shared__ float s_p[3][MAXN1];
    __shared__ int s_item, s_mode;
    const int tid = threadIdx.x;
    for (;;) {
        const int item = next_item(w.queue, &s_item);
        if (item >= w.nitems) break;
        const int2 it = w.items[item];
        const Fields &a = w.sys[it.y >> 16];
        const int b = it.x, orb = it.y & 0xffff;
        const int n1 = EXACT ? MAXN1 : a.n1, P = EXACT ? MAXN1 * MAXN1 * MAXN1 : a.P;
        const int n1p = n1 + (n1 & 1), Pp = n1 * n1 * n1p;
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
            float tx[NT], ty[NT], tz[NT], sum[NT], cmp[NT];
            float2 nfi[NT];
#pragma unroll
            for (int k = 0; k < NT; k++) {
                const int i = base + NT * tid + k;
                const bool v = i < te;
                tx[k] = v ? (float)(a.tx[i] - cb[0]) * scf : 0.f;
                ty[k] = v ? (float)(a.ty[i] - cb[1]) * scf : 0.f;
                tz[k] = v ? (float)(a.tz[i] - cb[2]) * scf : 0.f;
                nfi[k] = dup2(v ? -ft[i] : 0.f);
                sum[k] = 0.f;
                cmp[k] = 0.f;
            }
            for (int e = f0; e < f1; e++) {
                const int slot = a.node_slot[a.far_list[e]];
                const double *g = a.geom + 6L * slot;
                __syncthreads();
                const float *qs = qh + (long)slot * P;
                const float *ws = a.what32 + (long)slot * P;
                for (int k = tid; k < Pp; k += FT) {
                    const int row = k / n1p, k3 = k - row * n1p;
                    const bool real = k3 < n1;
                    const int src = row * n1 + (real ? k3 : 0);
                    s_q[k] = real ? qs[src] : 0.f;
                    s_w[k] = real ? ws[src] : 0.f;
                }
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
                if (mode == 1)
                    far_cluster<KERN, SS, false, MAXN1, NT, EXACT>(s_q, s_w, s_p, n1, tx, ty, tz, nfi, sum, cmp);
                else
                    far_cluster<KERN, SS, true, MAXN1, NT, EXACT>(s_q, s_w, s_p, n1, tx, ty, tz, nfi, sum, cmp);
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
// OG orbitals).  Per two sources (or two proxy points) the differences, r^2,
// r (via rsqrt) and -log2 r (via lg2) are formed once for the group in packed
// operations; each orbital then adds 2^{-k_o log2(e) r - log2 r} * c, which is
// e^{-k_o r} / r * c with the 1/r folded into the exponent.  -k_o log2(e) is
// the orbital's FP32 constant sc (orbital_constants), and the subtraction term
// uses the k that sc represents, so one FP32 constant suffices.  Coordinates
// are translated to the batch center but not scaled (each orbital has its own
// k).  Charges are staged as float4
// {q(o, j), q(o, j+1), q(o+1, j), q(o+1, j+1)} per (pair of sources, pair of
// orbitals), so one 16-byte shared read serves four (pair, orbital) terms.
// Orbitals past the last one of the request have zero charges and are not
// written.
// ---------------------------------------------------------------------------
constexpr int GTILE = 512;   // sources per group tile

__device__ __forceinline__ int q4_pos(int j, int o, int og) {   // float index of q(o, j) in the staged layout
    return (((j >> 1) * (og >> 1) + (o >> 1)) << 2) + ((o & 1) << 1) + (j & 1);
}

// Group tile rows: 0..2 negated coordinates (batch-relative, or hi parts of
// the absolute splits), 3 weight, 4..6 negated lo parts (PRECISE).
template <bool SS, bool MASK, bool PRECISE, int OG>
__device__ __forceinline__ void group_tile(const float (*__restrict__ s)[GTILE], const float4 *__restrict__ s_q4,
                                           int cnt2, float2 tx, float2 ty, float2 tz, float2 lx, float2 ly,
                                           float2 lz, const float2 (&nfi)[OG], const float2 (&kc)[OG],
                                           float (&sum)[OG], float (&cmp)[OG]) {
    for (int j0 = 0; j0 < cnt2; j0 += KCHUNK) {
        const int j1 = min(j0 + KCHUNK, cnt2);
        float2 part[OG];
#pragma unroll
        for (int o = 0; o < OG; o++) part[o] = make_float2(0.f, 0.f);
#pragma unroll 1   // measured: unrolling the source loop slows the group kernels
        for (int j = j0; j < j1; j += 2) {
            float2 dx = add2(tx, lds2(s[0] + j)), dy = add2(ty, lds2(s[1] + j)), dz = add2(tz, lds2(s[2] + j));
            if constexpr (PRECISE) {
                dx = add2(dx, add2(lx, lds2(s[4] + j)));
                dy = add2(dy, add2(ly, lds2(s[5] + j)));
                dz = add2(dz, add2(lz, lds2(s[6] + j)));
            }
            const float2 wv = lds2(s[3] + j);
            const float2 r2 = fma2(dx, dx, fma2(dy, dy, mul2(dz, dz)));
            float2 rinv = rsqrt2(r2);
            float2 nl = nlog2r2(r2);
            if (MASK) {   // r = 0: r = 0 and 2^{-inf} = 0, so the pair adds exactly 0
                rinv.x = r2.x > 0.f ? rinv.x : 0.f;
                rinv.y = r2.y > 0.f ? rinv.y : 0.f;
                nl.x = r2.x > 0.f ? nl.x : -INFINITY;
                nl.y = r2.y > 0.f ? nl.y : -INFINITY;
            }
            const float2 r = mul2(r2, rinv);
#pragma unroll
            for (int o2 = 0; o2 < OG / 2; o2++) {
                const float4 q4 = s_q4[(j >> 1) * (OG / 2) + o2];
#pragma unroll
                for (int u = 0; u < 2; u++) {
                    const int o = 2 * o2 + u;
                    const float2 q = u ? make_float2(q4.z, q4.w) : make_float2(q4.x, q4.y);
                    // e^{-k r} / r = 2^{-k log2(e) r - log2 r}
                    const float2 g = ex2pos2(fma2(kc[o], r, nl));
                    part[o] = fma2(g, SS ? fma2(nfi[o], wv, q) : q, part[o]);
                }
            }
        }
#pragma unroll
        for (int o = 0; o < OG; o++) kahan_add(sum[o], cmp[o], part[o].x + part[o].y);
    }
}

template <bool SS, int OG, int PASS>
__global__ void __launch_bounds__(FT, 2) near_group(const __grid_constant__ Work w) {
    constexpr int NR = PASS == 1 ? 7 : 4;
    __shared__ __align__(16) float s_src[NR][GTILE];
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
        float2 kc[OG];
        float kmin = 3.4e38f;
#pragma unroll
        for (int o = 0; o < OG; o++) {
            const int orb = g0 + o;
            kc[o] = dup2(orb < a.norb ? -a.kc32[orb] : 0.f);   // -k log2(e) as one FP32 constant
            if (orb < a.norb) kmin = fminf(kmin, a.kc32[orb]);
        }
        const int r0 = a.rng_off[b], r1 = a.rng_off[b + 1];
        for (int base = tb; base < te; base += FT) {
            const int i = base + tid;
            const bool v = i < te;
            const bool warp_busy = base + (tid & ~31) < te;
            float2 tx, ty, tz, lx = dup2(0.f), ly = dup2(0.f), lz = dup2(0.f);
            if (PASS == 1) {  // absolute hi/lo splits (see near_tile)
                const float4 h = v ? a.thi[i] : make_float4(0.f, 0.f, 0.f, 0.f);
                const float4 l = v ? a.tlo[i] : make_float4(0.f, 0.f, 0.f, 0.f);
                tx = dup2(h.x);
                ty = dup2(h.y);
                tz = dup2(h.z);
                lx = dup2(l.x);
                ly = dup2(l.y);
                lz = dup2(l.z);
            } else {
                tx = dup2(v ? (float)(a.tx[i] - cbx) : 0.f);
                ty = dup2(v ? (float)(a.ty[i] - cby) : 0.f);
                tz = dup2(v ? (float)(a.tz[i] - cbz) : 0.f);
            }
            float2 nfi[OG];
            float sum[OG], cmp[OG];
#pragma unroll
            for (int o = 0; o < OG; o++) {
                const int orb = g0 + o;
                nfi[o] = dup2((v && orb < a.norb) ? -a.ft32[(long)orb * a.nt + i] : 0.f);
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
                    const int cnt2 = (cnt + 1) & ~1;
                    __syncthreads();
                    for (int j = tid; j < cnt2; j += FT) {
                        const bool real = j < cnt;
                        const int jj = t0 + (real ? j : 0);   // padding: a copy of the first source
                        if constexpr (PASS == 1) {
                            const float4 h = a.shi[jj], l = a.slo[jj];
                            s_src[0][j] = -h.x;
                            s_src[1][j] = -h.y;
                            s_src[2][j] = -h.z;
                            s_src[4][j] = -l.x;
                            s_src[5][j] = -l.y;
                            s_src[6][j] = -l.z;
                        } else {
                            s_src[0][j] = -(float)(a.sx[jj] - cbx);
                            s_src[1][j] = -(float)(a.sy[jj] - cby);
                            s_src[2][j] = -(float)(a.sz[jj] - cbz);
                        }
                        s_src[3][j] = real ? a.w32[jj] : 0.f;
                    }
                    for (int k = tid; k < cnt2 * OG; k += FT) {   // orbital-major: coalesced global reads
                        const int o = k / cnt2, j = k - o * cnt2;
                        const int orb = g0 + o;
                        reinterpret_cast<float *>(s_q4)[q4_pos(j, o, OG)] =
                            (j < cnt && orb < a.norb) ? a.q32[(long)orb * a.ns + t0 + j] : 0.f;
                    }
                    __syncthreads();
                    if (!warp_busy) continue;
                    if (PASS == 1)
                        group_tile<SS, true, true, OG>(s_src, s_q4, cnt2, tx, ty, tz, lx, ly, lz, nfi, kc, sum,
                                                       cmp);
                    else
                        group_tile<SS, false, false, OG>(s_src, s_q4, cnt2, tx, ty, tz, lx, ly, lz, nfi, kc, sum,
                                                         cmp);
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

// One staged proxy grid against one target for a group of orbitals (see
// far_cluster for the padded innermost axis).
template <bool SS, int MAXN1, int OG, bool EXACT = false>
__device__ __forceinline__ void far_group_cluster(const float4 *__restrict__ s_q4, const float *__restrict__ s_w,
                                                  const float (*s_p)[MAXN1], int n1_in, float tx, float ty, float tz,
                                                  const float2 (&nfi)[OG], const float2 (&kc)[OG],
                                                  float (&sum)[OG], float (&cmp)[OG]) {
    constexpr int MH = even_up<MAXN1>() / 2;
    const int n1 = EXACT ? MAXN1 : n1_in;
    const int n1p = n1 + (n1 & 1);
    float2 dz2[MH];
#pragma unroll
    for (int m = 0; m < MH; m++) {
        const float d0 = tz - s_p[2][2 * m < n1 ? 2 * m : 0];
        const float d1 = tz - s_p[2][2 * m + 1 < n1 ? 2 * m + 1 : 0];
        dz2[m] = make_float2(d0 * d0, d1 * d1);
    }
    int idx = 0;
    for (int k1 = 0; k1 < n1; k1++) {
        float2 part[OG];
#pragma unroll
        for (int o = 0; o < OG; o++) part[o] = make_float2(0.f, 0.f);
        const float dx = tx - s_p[0][k1];
        const float dx2 = dx * dx;
        for (int k2 = 0; k2 < n1; k2++) {
            const float dy = ty - s_p[1][k2];
            const float2 rxy = dup2(fmaf(dy, dy, dx2));
#pragma unroll
            for (int m = 0; m < MH; m++) {
                if (2 * m < n1) {
                    const float2 r2 = add2(rxy, dz2[m]);
                    const float2 rr = mul2(r2, rsqrt2(r2));
                    const float2 nl = nlog2r2(r2);
                    const float2 wk = lds2(s_w + idx + 2 * m);
#pragma unroll
                    for (int o2 = 0; o2 < OG / 2; o2++) {
                        const float4 q4 = s_q4[((idx >> 1) + m) * (OG / 2) + o2];
#pragma unroll
                        for (int u = 0; u < 2; u++) {
                            const int o = 2 * o2 + u;
                            const float2 q = u ? make_float2(q4.z, q4.w) : make_float2(q4.x, q4.y);
                            const float2 g = ex2pos2(fma2(kc[o], rr, nl));
                            part[o] = fma2(g, SS ? fma2(nfi[o], wk, q) : q, part[o]);
                        }
                    }
                }
            }
            idx += n1p;
        }
#pragma unroll
        for (int o = 0; o < OG; o++) kahan_add(sum[o], cmp[o], part[o].x + part[o].y);
    }
}

// Dynamic shared memory of far_group: the staged charges (Pp * OG floats,
// Pp = n1 * n1 * n1p) then the weights (Pp floats), for the largest grid of
// the launch's systems (above 48 KB at degree 10 with 8 orbitals).
__host__ __device__ constexpr size_t far_group_smem(int n1, int og) {
    return sizeof(float) * (size_t)n1 * n1 * (n1 + (n1 & 1)) * (og + 1);
}

template <bool SS, int MAXN1, int OG, bool EXACT = false>
__global__ void __launch_bounds__(FT, 2) far_group(const __grid_constant__ Work w) {
    extern __shared__ __align__(16) float s_dyn[];
    __shared__ float s_p[3][MAXN1];
    __shared__ int s_item;
    float4 *s_q4 = reinterpret_cast<float4 *>(s_dyn);
    const int tid = threadIdx.x;
    for (;;) {
        const int item = next_item(w.queue, &s_item);
        if (item >= w.nitems) break;
        const int2 it = w.items[item];
        const Fields &a = w.sys[it.y >> 16];
        const int b = it.x, g0 = it.y & 0xffff;
        const int n1 = EXACT ? MAXN1 : a.n1, P = EXACT ? MAXN1 * MAXN1 * MAXN1 : a.P;
        const int n1p = n1 + (n1 & 1), Pp = n1 * n1 * n1p;
        const float *s_w = s_dyn + (size_t)Pp * OG;   // Pp * OG is a multiple of 4: float4 aligned
        const int f0 = a.far_off[b], f1 = a.far_off[b + 1];
        if (f0 == f1) continue;
        const int bn = a.batch_node[b];
        const int tb = a.tbegin[bn], te = a.tend[bn];
        const double cb[3] = {a.tcenter[3L * bn], a.tcenter[3L * bn + 1], a.tcenter[3L * bn + 2]};
        float2 kc[OG];
#pragma unroll
        for (int o = 0; o < OG; o++) kc[o] = dup2((g0 + o) < a.norb ? -a.kc32[g0 + o] : 0.f);
        for (int base = tb; base < te; base += FT) {
            const int i = base + tid;
            const bool v = i < te;
            const bool warp_busy = base + (tid & ~31) < te;
            const float tx = v ? (float)(a.tx[i] - cb[0]) : 0.f;
            const float ty = v ? (float)(a.ty[i] - cb[1]) : 0.f;
            const float tz = v ? (float)(a.tz[i] - cb[2]) : 0.f;
            float2 nfi[OG];
            float sum[OG], cmp[OG];
#pragma unroll
            for (int o = 0; o < OG; o++) {
                const int orb = g0 + o;
                nfi[o] = dup2((v && orb < a.norb) ? -a.ft32[(long)orb * a.nt + i] : 0.f);
                sum[o] = 0.f;
                cmp[o] = 0.f;
            }
            for (int e = f0; e < f1; e++) {
                const int slot = a.node_slot[a.far_list[e]];
                const double *gm = a.geom + 6L * slot;
                __syncthreads();
                for (int k = tid; k < Pp * OG; k += FT) {   // orbital-major: coalesced global reads
                    const int o = k / Pp, kk = k - o * Pp;
                    const int row = kk / n1p, k3 = kk - row * n1p;
                    const int orb = g0 + o;
                    reinterpret_cast<float *>(s_q4)[q4_pos(kk, o, OG)] =
                        (k3 < n1 && orb < a.norb) ? a.qhat32[((long)orb * a.nslots + slot) * P + row * n1 + k3] : 0.f;
                }
                for (int k = tid; k < Pp; k += FT) {
                    const int row = k / n1p, k3 = k - row * n1p;
                    s_dyn[(size_t)Pp * OG + k] = k3 < n1 ? a.what32[(long)slot * P + row * n1 + k3] : 0.f;
                }
                if (tid < 3 * n1) {
                    const int d = tid / n1, m = tid - d * n1;
                    const double cbd = d == 0 ? cb[0] : (d == 1 ? cb[1] : cb[2]);
                    s_p[d][m] = (float)((gm[d] + gm[3 + d] * a.tn[m]) - cbd);
                }
                __syncthreads();
                if (!warp_busy) continue;
                far_group_cluster<SS, MAXN1, OG, EXACT>(s_q4, s_w, s_p, n1, tx, ty, tz, nfi, kc, sum, cmp);
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
// far_group at degree 7 with the next cluster's charges in flight: cp.async
// copies global -> shared without registers, so the charges and weight
// charges of far cluster e+1 load while cluster e is computed, and one
// barrier per cluster separates the two buffers.  Charges are copied 8 bytes
// at a time ({q(o, j), q(o, j+1)} is contiguous both in global memory and in
// the staged layout); orbitals past the request's last get zero-filled copies.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem, bool valid) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    const int n = valid ? 8 : 0;   // source bytes; the rest of the 8 are zero-filled
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(sa), "l"(gmem), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

constexpr int DB_N1 = 8, DB_P = DB_N1 * DB_N1 * DB_N1;   // degree 7
__host__ __device__ constexpr size_t far_group_db_smem(int og) { return sizeof(float) * 2 * (size_t)DB_P * (og + 1); }

template <bool SS, int OG>
__global__ void __launch_bounds__(FT, 2) far_group_db(const __grid_constant__ Work w) {
    constexpr int BUF = DB_P * OG + DB_P;   // floats per buffer: charges, then weight charges
    extern __shared__ __align__(16) float s_dyn[];
    __shared__ float s_p[2][3][DB_N1];
    __shared__ int s_item;
    const int tid = threadIdx.x;
    for (;;) {
        const int item = next_item(w.queue, &s_item);
        if (item >= w.nitems) break;
        const int2 it = w.items[item];
        const Fields &a = w.sys[it.y >> 16];
        const int b = it.x, g0 = it.y & 0xffff;
        const int f0 = a.far_off[b], f1 = a.far_off[b + 1];
        if (f0 == f1) continue;
        const int bn = a.batch_node[b];
        const int tb = a.tbegin[bn], te = a.tend[bn];
        const double cb[3] = {a.tcenter[3L * bn], a.tcenter[3L * bn + 1], a.tcenter[3L * bn + 2]};
        float2 kc[OG];
#pragma unroll
        for (int o = 0; o < OG; o++) kc[o] = dup2((g0 + o) < a.norb ? -a.kc32[g0 + o] : 0.f);
        // issue the copies of far cluster e into buffer buf (completes at the next wait + barrier)
        auto stage = [&](int e, int buf) {
            const int slot = a.node_slot[a.far_list[e]];
            float *q = s_dyn + (size_t)buf * BUF;
            for (int k = tid; k < DB_P * OG / 2; k += FT) {
                const int o = k / (DB_P / 2), kk = 2 * (k - o * (DB_P / 2));
                const int orb = g0 + o;
                const bool valid = orb < a.norb;
                const float *src = a.qhat32 + ((long)(valid ? orb : g0) * a.nslots + slot) * DB_P + kk;
                cp_async8(q + q4_pos(kk, o, OG), src, valid);
            }
            for (int k = tid; k < DB_P / 4; k += FT) cp_async16(q + DB_P * OG + 4 * k, a.what32 + (long)slot * DB_P + 4 * k);
            cp_async_commit();
            if (tid < 3 * DB_N1) {
                const double *gm = a.geom + 6L * slot;
                const int d = tid / DB_N1, m = tid - d * DB_N1;
                const double cbd = d == 0 ? cb[0] : (d == 1 ? cb[1] : cb[2]);
                s_p[buf][d][m] = (float)((gm[d] + gm[3 + d] * a.tn[m]) - cbd);
            }
        };
        for (int base = tb; base < te; base += FT) {
            const int i = base + tid;
            const bool v = i < te;
            const bool warp_busy = base + (tid & ~31) < te;
            const float tx = v ? (float)(a.tx[i] - cb[0]) : 0.f;
            const float ty = v ? (float)(a.ty[i] - cb[1]) : 0.f;
            const float tz = v ? (float)(a.tz[i] - cb[2]) : 0.f;
            float2 nfi[OG];
            float sum[OG], cmp[OG];
#pragma unroll
            for (int o = 0; o < OG; o++) {
                const int orb = g0 + o;
                nfi[o] = dup2((v && orb < a.norb) ? -a.ft32[(long)orb * a.nt + i] : 0.f);
                sum[o] = 0.f;
                cmp[o] = 0.f;
            }
            __syncthreads();   // every thread is done with both buffers of the previous target chunk
            stage(f0, 0);
            for (int e = f0; e < f1; e++) {
                const int cur = (e - f0) & 1;
                cp_async_wait_all();   // this thread's copies of cluster e
                __syncthreads();       // everyone's copies visible; everyone done reading the other buffer
                if (e + 1 < f1) stage(e + 1, cur ^ 1);
                if (!warp_busy) continue;
                const float *q = s_dyn + (size_t)cur * BUF;
                far_group_cluster<SS, DB_N1, OG, true>(reinterpret_cast<const float4 *>(q), q + DB_P * OG, s_p[cur],
                                                       DB_N1, tx, ty, tz, nfi, kc, sum, cmp);
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
// Orbital-group kernels with 16 orbitals per item, packed by ORBITAL: the two
// lanes of every packed operation are orbitals (2p, 2p+1) of one source (or
// proxy point).  The per-orbital constants -k log2(e) and -f_i are then
// natural float2 pairs -- 8 pairs of registers each for 16 orbitals, where
// the source-packed layout needs 16 duplicated pairs -- and only the
// source's r, -log2 r and weight are duplicated, once per source for all 16
// orbitals.  The geometry (differences, r^2, rsqrt, lg2) of two sources is
// still formed in packed operations and is shared by 16 orbitals: MUFU work
// per pair-orbital is 1 ex2 + (rsqrt + lg2)/16.
// Charges are staged orbital-fastest, QS16 floats per source (16 used + 4 of
// padding, which spreads the staging writes over all banks); a thread reads
// one source's 16 charges as four float4.  Each lane sums KCHUNK16 sources of
// one orbital before the Kahan step, the same run length per lane as the
// source-packed kernels.
// ---------------------------------------------------------------------------
constexpr int QS16 = 20;
constexpr int KCHUNK16 = 32;

// One tile of cnt4 sources (a multiple of 4) for 16 orbitals.  Four sources
// per iteration (two packed pairs), software pipelined: the next four
// sources' geometry (loads, rsqrt, lg2) is issued before this iteration's
// 64 orbital-pair updates, which hides its latency.  The per-orbital Kahan
// sums live in shared memory (s_k[o][FT] sums, s_k[16 + o][FT]
// compensations, touched once per KCHUNK16 sources), which leaves the
// registers for the pipelined geometry.  NP: orbital pairs of the item that
// hold orbitals (the last group of a request may be partly filled); the
// pairs past NP are not computed.
template <bool SS, bool MASK, bool PRECISE, int NP = 8>
__device__ __forceinline__ void group16_tile(const float (*__restrict__ s)[GTILE], const float *__restrict__ s_q,
                                             int cnt4, float2 tx, float2 ty, float2 tz, float2 lx, float2 ly,
                                             float2 lz, const float2 (&nfi)[8], const float2 (&kc)[8],
                                             float *__restrict__ s_k) {
    // r, -log2 r and w of the source pair at j (packed over the two sources)
    auto geometry = [&](int j, float2 &r, float2 &nl, float2 &wv) {
        float2 dx = add2(tx, lds2(s[0] + j)), dy = add2(ty, lds2(s[1] + j)), dz = add2(tz, lds2(s[2] + j));
        if constexpr (PRECISE) {
            dx = add2(dx, add2(lx, lds2(s[4] + j)));
            dy = add2(dy, add2(ly, lds2(s[5] + j)));
            dz = add2(dz, add2(lz, lds2(s[6] + j)));
        }
        wv = lds2(s[3] + j);
        const float2 r2 = fma2(dx, dx, fma2(dy, dy, mul2(dz, dz)));
        float2 rinv = rsqrt2(r2);
        nl = nlog2r2(r2);
        if (MASK) {   // r = 0: r = 0 and 2^{-inf} = 0, so the pair adds exactly 0
            rinv.x = r2.x > 0.f ? rinv.x : 0.f;
            rinv.y = r2.y > 0.f ? rinv.y : 0.f;
            nl.x = r2.x > 0.f ? nl.x : -INFINITY;
            nl.y = r2.y > 0.f ? nl.y : -INFINITY;
        }
        r = mul2(r2, rinv);
    };
    const int tid = threadIdx.x;
    float2 part[8];
#pragma unroll
    for (int p = 0; p < 8; p++) part[p] = make_float2(0.f, 0.f);
    float2 rc[2], nc[2], wc[2];
    geometry(0, rc[0], nc[0], wc[0]);
    geometry(2, rc[1], nc[1], wc[1]);
#pragma unroll 1
    for (int j = 0; j < cnt4; j += 4) {
        const int jn = j + 4 < cnt4 ? j + 4 : j;
        float2 rn[2], nn[2], wn[2];
        geometry(jn, rn[0], nn[0], wn[0]);
        geometry(jn + 2, rn[1], nn[1], wn[1]);
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const float ru = (u & 1) ? rc[u >> 1].y : rc[u >> 1].x;
            const float nu = (u & 1) ? nc[u >> 1].y : nc[u >> 1].x;
            const float wu = (u & 1) ? wc[u >> 1].y : wc[u >> 1].x;
            const float2 rd = dup2(ru), nd = dup2(nu), wd = dup2(wu);
            const float *qj = s_q + (j + u) * QS16;
#pragma unroll
            for (int o4 = 0; o4 < (NP + 1) / 2; o4++) {
                const float4 q4 = lds4(qj + 4 * o4);
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int p = 2 * o4 + h;   // orbitals 2p, 2p+1
                    if (p < NP) {
                        const float2 q = h ? make_float2(q4.z, q4.w) : make_float2(q4.x, q4.y);
                        const float2 g = ex2pos2(fma2(kc[p], rd, nd));
                        part[p] = fma2(g, SS ? fma2(nfi[p], wd, q) : q, part[p]);
                    }
                }
            }
        }
        if ((j + 4) % KCHUNK16 == 0 || j + 4 >= cnt4) {   // end of a run of KCHUNK16 sources
#pragma unroll
            for (int p = 0; p < NP; p++) {
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int o = 2 * p + h;
                    float sm = s_k[o * FT + tid], cm = s_k[(16 + o) * FT + tid];
                    kahan_add(sm, cm, h ? part[p].y : part[p].x);
                    s_k[o * FT + tid] = sm;
                    s_k[(16 + o) * FT + tid] = cm;
                }
                part[p] = make_float2(0.f, 0.f);
            }
        }
#pragma unroll
        for (int v = 0; v < 2; v++) {
            rc[v] = rn[v];
            nc[v] = nn[v];
            wc[v] = wn[v];
        }
    }
}

// group16_tile for the item's np filled orbital pairs (1..8).
template <bool SS, bool MASK, bool PRECISE>
__device__ __forceinline__ void group16_tile_np(int np, const float (*__restrict__ s)[GTILE],
                                                const float *__restrict__ s_q, int cnt4, float2 tx, float2 ty,
                                                float2 tz, float2 lx, float2 ly, float2 lz, const float2 (&nfi)[8],
                                                const float2 (&kc)[8], float *__restrict__ s_k) {
#define TAGI_G16(N) group16_tile<SS, MASK, PRECISE, N>(s, s_q, cnt4, tx, ty, tz, lx, ly, lz, nfi, kc, s_k)
    switch (np) {
    case 1: TAGI_G16(1); break;
    case 2: TAGI_G16(2); break;
    case 3: TAGI_G16(3); break;
    case 4: TAGI_G16(4); break;
    case 5: TAGI_G16(5); break;
    case 6: TAGI_G16(6); break;
    case 7: TAGI_G16(7); break;
    default: TAGI_G16(8); break;
    }
#undef TAGI_G16
}

// Filled orbital pairs of a 16-orbital item starting at orbital g0.
__device__ __forceinline__ int group16_pairs(int norb, int g0) { return min(8, (norb - g0 + 1) >> 1); }

// Per-orbital constants of a 16-orbital item, as orbital pairs.
__device__ __forceinline__ void group16_constants(const Fields &a, int g0, float2 (&kc)[8], float *kmin) {
    float km = 3.4e38f;
#pragma unroll
    for (int p = 0; p < 8; p++) {
        const int o0 = g0 + 2 * p, o1 = o0 + 1;
        kc[p] = make_float2(o0 < a.norb ? -a.kc32[o0] : 0.f, o1 < a.norb ? -a.kc32[o1] : 0.f);   // -k log2(e)
        if (o0 < a.norb) km = fminf(km, a.kc32[o0]);
        if (o1 < a.norb) km = fminf(km, a.kc32[o1]);
    }
    if (kmin) *kmin = km;
}

// Dynamic shared memory of near_group16: the source rows, the charges, then
// the per-thread Kahan sums and compensations of 16 orbitals.
__host__ __device__ constexpr size_t near_group16_smem(int pass) {
    return sizeof(float) * ((size_t)GTILE * ((pass == 1 ? 7 : 4) + QS16) + 32 * FT);
}

template <bool SS, int PASS>
__global__ void __launch_bounds__(FT, 2) near_group16(const __grid_constant__ Work w) {
    constexpr int NR = PASS == 1 ? 7 : 4;
    extern __shared__ __align__(16) float s_dyn[];
    float(*s_src)[GTILE] = reinterpret_cast<float(*)[GTILE]>(s_dyn);
    float *s_q = s_dyn + NR * GTILE;
    float *s_k = s_q + GTILE * QS16;
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
        float2 kc[8];
        float kmin;
        group16_constants(a, g0, kc, &kmin);
        const int r0 = a.rng_off[b], r1 = a.rng_off[b + 1];
        for (int base = tb; base < te; base += FT) {
            const int i = base + tid;
            const bool v = i < te;
            const bool warp_busy = base + (tid & ~31) < te;
            float2 tx, ty, tz, lx = dup2(0.f), ly = dup2(0.f), lz = dup2(0.f);
            if (PASS == 1) {  // absolute hi/lo splits (see near_tile)
                const float4 h = v ? a.thi[i] : make_float4(0.f, 0.f, 0.f, 0.f);
                const float4 l = v ? a.tlo[i] : make_float4(0.f, 0.f, 0.f, 0.f);
                tx = dup2(h.x);
                ty = dup2(h.y);
                tz = dup2(h.z);
                lx = dup2(l.x);
                ly = dup2(l.y);
                lz = dup2(l.z);
            } else {
                tx = dup2(v ? (float)(a.tx[i] - cbx) : 0.f);
                ty = dup2(v ? (float)(a.ty[i] - cby) : 0.f);
                tz = dup2(v ? (float)(a.tz[i] - cbz) : 0.f);
            }
            float2 nfi[8];
#pragma unroll
            for (int p = 0; p < 8; p++) {
                const int o0 = g0 + 2 * p, o1 = o0 + 1;
                nfi[p] = make_float2((v && o0 < a.norb) ? -a.ft32[(long)o0 * a.nt + i] : 0.f,
                                     (v && o1 < a.norb) ? -a.ft32[(long)o1 * a.nt + i] : 0.f);
            }
#pragma unroll
            for (int o = 0; o < 32; o++) s_k[o * FT + tid] = 0.f;   // this thread's own sums
            for (int e = r0; e < r1; e++) {
                const int2 r = a.rng[e];
                if (a.rng_dmin[e] * kmin > 127.f) continue;  // every orbital's term is exactly 0
                const bool close = range_is_close(r);
                if (close != (PASS == 1)) continue;
                const int rb = range_begin(r);
                for (int t0 = rb; t0 < r.y; t0 += GTILE) {
                    const int cnt = min(GTILE, r.y - t0);
                    const int cnt4 = (cnt + 3) & ~3;
                    __syncthreads();
                    for (int j = tid; j < cnt4; j += FT) {
                        const bool real = j < cnt;
                        const int jj = t0 + (real ? j : 0);   // padding: a copy of the first source
                        if constexpr (PASS == 1) {
                            const float4 h = a.shi[jj], l = a.slo[jj];
                            s_src[0][j] = -h.x;
                            s_src[1][j] = -h.y;
                            s_src[2][j] = -h.z;
                            s_src[4][j] = -l.x;
                            s_src[5][j] = -l.y;
                            s_src[6][j] = -l.z;
                        } else {
                            s_src[0][j] = -(float)(a.sx[jj] - cbx);
                            s_src[1][j] = -(float)(a.sy[jj] - cby);
                            s_src[2][j] = -(float)(a.sz[jj] - cbz);
                        }
                        s_src[3][j] = real ? a.w32[jj] : 0.f;
                    }
                    // a warp stages 8 sources x 4 orbitals: 32-byte global segments,
                    // conflict-free shared writes with the QS16 stride
                    for (int k = tid; k < ((cnt4 + 7) & ~7) * 16; k += FT) {
                        const int jb = k >> 7, rem = k & 127;
                        const int o = rem >> 3, j = (jb << 3) + (rem & 7);
                        if (j >= cnt4) continue;
                        const int orb = g0 + o;
                        s_q[j * QS16 + o] = (j < cnt && orb < a.norb) ? a.q32[(long)orb * a.ns + t0 + j] : 0.f;
                    }
                    __syncthreads();
                    if (!warp_busy) continue;
                    const int np = group16_pairs(a.norb, g0);
                    if (PASS == 1)
                        group16_tile_np<SS, true, true>(np, s_src, s_q, cnt4, tx, ty, tz, lx, ly, lz, nfi, kc, s_k);
                    else
                        group16_tile_np<SS, false, false>(np, s_src, s_q, cnt4, tx, ty, tz, lx, ly, lz, nfi, kc,
                                                          s_k);
                }
            }
            if (v) {
#pragma unroll
                for (int o = 0; o < 16; o++)
                    if (g0 + o < a.norb)
                        a.out[(long)(g0 + o) * a.nt + i] = (double)s_k[o * FT + tid] - (double)s_k[(16 + o) * FT + tid];
            }
        }
    }
}

// One staged proxy grid against one target for 16 orbitals (see far_cluster
// for the padded innermost axis; charges staged QS16 floats per proxy point).
// NP: filled orbital pairs, as in group16_tile.
template <bool SS, int MAXN1, bool EXACT, int NP = 8>
__device__ __forceinline__ void far_group16_cluster(const float *__restrict__ s_q, const float *__restrict__ s_w,
                                                    const float (*s_p)[MAXN1], int n1_in, float tx, float ty,
                                                    float tz, const float2 (&nfi)[8], const float2 (&kc)[8],
                                                    float (&sum)[16], float (&cmp)[16]) {
    constexpr int MH = even_up<MAXN1>() / 2;
    const int n1 = EXACT ? MAXN1 : n1_in;
    const int n1p = n1 + (n1 & 1);
    float2 dz2[MH];
#pragma unroll
    for (int m = 0; m < MH; m++) {
        const float d0 = tz - s_p[2][2 * m < n1 ? 2 * m : 0];
        const float d1 = tz - s_p[2][2 * m + 1 < n1 ? 2 * m + 1 : 0];
        dz2[m] = make_float2(d0 * d0, d1 * d1);
    }
    int idx = 0;
    for (int k1 = 0; k1 < n1; k1++) {
        float2 part[8];
#pragma unroll
        for (int p = 0; p < 8; p++) part[p] = make_float2(0.f, 0.f);
        const float dx = tx - s_p[0][k1];
        const float dx2 = dx * dx;
        for (int k2 = 0; k2 < n1; k2++) {
            const float dy = ty - s_p[1][k2];
            const float2 rxy = dup2(fmaf(dy, dy, dx2));
#pragma unroll
            for (int m = 0; m < MH; m++) {
                if (2 * m < n1) {
                    const float2 r2 = add2(rxy, dz2[m]);
                    const float2 rr = mul2(r2, rsqrt2(r2));
                    const float2 nl = nlog2r2(r2);
                    const float2 wk = lds2(s_w + idx + 2 * m);
#pragma unroll
                    for (int u = 0; u < 2; u++) {
                        const float2 rd = dup2(u ? rr.y : rr.x), nd = dup2(u ? nl.y : nl.x);
                        const float2 wd = dup2(u ? wk.y : wk.x);
                        const float *qk = s_q + (idx + 2 * m + u) * QS16;
#pragma unroll
                        for (int o4 = 0; o4 < (NP + 1) / 2; o4++) {
                            const float4 q4 = lds4(qk + 4 * o4);
#pragma unroll
                            for (int h = 0; h < 2; h++) {
                                const int p = 2 * o4 + h;
                                if (p < NP) {
                                    const float2 q = h ? make_float2(q4.z, q4.w) : make_float2(q4.x, q4.y);
                                    const float2 g = ex2pos2(fma2(kc[p], rd, nd));
                                    part[p] = fma2(g, SS ? fma2(nfi[p], wd, q) : q, part[p]);
                                }
                            }
                        }
                    }
                }
            }
            idx += n1p;
        }
#pragma unroll
        for (int p = 0; p < NP; p++) {
            kahan_add(sum[2 * p], cmp[2 * p], part[p].x);
            kahan_add(sum[2 * p + 1], cmp[2 * p + 1], part[p].y);
        }
    }
}

template <bool SS, int MAXN1, bool EXACT>
__device__ __forceinline__ void far_group16_cluster_np(int np, const float *__restrict__ s_q,
                                                       const float *__restrict__ s_w, const float (*s_p)[MAXN1],
                                                       int n1, float tx, float ty, float tz, const float2 (&nfi)[8],
                                                       const float2 (&kc)[8], float (&sum)[16],
                                                       float (&cmp)[16]) {
#define TAGI_F16(N) far_group16_cluster<SS, MAXN1, EXACT, N>(s_q, s_w, s_p, n1, tx, ty, tz, nfi, kc, sum, cmp)
    switch (np) {
    case 1: TAGI_F16(1); break;
    case 2: TAGI_F16(2); break;
    case 3: TAGI_F16(3); break;
    case 4: TAGI_F16(4); break;
    case 5: TAGI_F16(5); break;
    case 6: TAGI_F16(6); break;
    case 7: TAGI_F16(7); break;
    default: TAGI_F16(8); break;
    }
#undef TAGI_F16
}

// Dynamic shared memory of far_group16: charges (Pp * QS16 floats) then the
// weight charges (Pp floats), Pp = n1 * n1 * n1p.
__host__ __device__ constexpr size_t far_group16_smem(int n1) {
    return sizeof(float) * (size_t)n1 * n1 * (n1 + (n1 & 1)) * (QS16 + 1);
}

template <bool SS, int MAXN1, bool EXACT>
__global__ void __launch_bounds__(FT, 2) far_group16(const __grid_constant__ Work w) {
    extern __shared__ __align__(16) float s_dyn[];
    __shared__ float s_p[3][MAXN1];
    __shared__ int s_item;
    const int tid = threadIdx.x;
    for (;;) {
        const int item = next_item(w.queue, &s_item);
        if (item >= w.nitems) break;
        const int2 it = w.items[item];
        const Fields &a = w.sys[it.y >> 16];
        const int b = it.x, g0 = it.y & 0xffff;
        const int n1 = EXACT ? MAXN1 : a.n1, P = EXACT ? MAXN1 * MAXN1 * MAXN1 : a.P;
        const int n1p = n1 + (n1 & 1), Pp = n1 * n1 * n1p;
        float *s_q = s_dyn;
        float *s_w = s_dyn + (size_t)Pp * QS16;
        const int f0 = a.far_off[b], f1 = a.far_off[b + 1];
        if (f0 == f1) continue;
        const int bn = a.batch_node[b];
        const int tb = a.tbegin[bn], te = a.tend[bn];
        const double cb[3] = {a.tcenter[3L * bn], a.tcenter[3L * bn + 1], a.tcenter[3L * bn + 2]};
        float2 kc[8];
        group16_constants(a, g0, kc, nullptr);
        for (int base = tb; base < te; base += FT) {
            const int i = base + tid;
            const bool v = i < te;
            const bool warp_busy = base + (tid & ~31) < te;
            const float tx = v ? (float)(a.tx[i] - cb[0]) : 0.f;
            const float ty = v ? (float)(a.ty[i] - cb[1]) : 0.f;
            const float tz = v ? (float)(a.tz[i] - cb[2]) : 0.f;
            float2 nfi[8];
            float sum[16], cmp[16];
#pragma unroll
            for (int p = 0; p < 8; p++) {
                const int o0 = g0 + 2 * p, o1 = o0 + 1;
                nfi[p] = make_float2((v && o0 < a.norb) ? -a.ft32[(long)o0 * a.nt + i] : 0.f,
                                     (v && o1 < a.norb) ? -a.ft32[(long)o1 * a.nt + i] : 0.f);
            }
#pragma unroll
            for (int o = 0; o < 16; o++) {
                sum[o] = 0.f;
                cmp[o] = 0.f;
            }
            for (int e = f0; e < f1; e++) {
                const int slot = a.node_slot[a.far_list[e]];
                const double *gm = a.geom + 6L * slot;
                __syncthreads();
                // a warp stages 8 proxy points x 4 orbitals (see near_group16)
                for (int k = tid; k < ((Pp + 7) & ~7) * 16; k += FT) {
                    const int kb = k >> 7, rem = k & 127;
                    const int o = rem >> 3, kk = (kb << 3) + (rem & 7);
                    if (kk >= Pp) continue;
                    const int row = kk / n1p, k3 = kk - row * n1p;
                    const int orb = g0 + o;
                    s_q[kk * QS16 + o] =
                        (k3 < n1 && orb < a.norb) ? a.qhat32[((long)orb * a.nslots + slot) * P + row * n1 + k3] : 0.f;
                }
                for (int k = tid; k < Pp; k += FT) {
                    const int row = k / n1p, k3 = k - row * n1p;
                    s_w[k] = k3 < n1 ? a.what32[(long)slot * P + row * n1 + k3] : 0.f;
                }
                if (tid < 3 * n1) {
                    const int d = tid / n1, m = tid - d * n1;
                    const double cbd = d == 0 ? cb[0] : (d == 1 ? cb[1] : cb[2]);
                    s_p[d][m] = (float)((gm[d] + gm[3 + d] * a.tn[m]) - cbd);
                }
                __syncthreads();
                if (!warp_busy) continue;
                far_group16_cluster_np<SS, MAXN1, EXACT>(group16_pairs(a.norb, g0), s_q, s_w, s_p, n1, tx, ty, tz,
                                                         nfi, kc, sum, cmp);
            }
            if (v) {
#pragma unroll
                for (int o = 0; o < 16; o++)
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
int occupancy_grid(K kern, int *grid, size_t smem = 0) {
    int dev = 0, sms = 0, per = 0;
    TAGI_CUDA(cudaGetDevice(&dev));
    TAGI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    TAGI_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, FT, smem));
    *grid = sms * (per > 0 ? per : 1);
    return TAGI_OK;
}

// Persistent launch: grid = resident CTAs (at most one per work item).  smem
// bytes of dynamic shared memory; for large requests the kernel's limit is
// raised first.
template <typename K>
int launch_persistent(K kern, const Work &w, cudaStream_t s, size_t smem = 0) {
    if (w.nitems == 0) return TAGI_OK;
    if (smem > 32 * 1024)   // dynamic + static above the 48 KB default needs the opt-in
        TAGI_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int grid = 0;
    TAGI_TRY(occupancy_grid(kern, &grid, smem));
    if (grid > w.nitems) grid = w.nitems;
    if (grid < 1) grid = 1;
    launch(kern, grid, FT, smem, s, w);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

// ---------------------------------------------------------------------------
// Loop ceilings: the near/far inner loops' arithmetic with operands already
// in shared memory and registers and no global traffic, measured live on the
// same GPU.  The ratio of a field kernel's pair rate to its loop's ceiling is
// its loop efficiency (staging, scheduling and tails); the hardware roofline
// is the per-pipe rate (tagi_pipe_rates).
// ---------------------------------------------------------------------------
template <int KERN, bool SS>
__global__ void __launch_bounds__(FT) pair_peak_near(int reps, float *out) {
    __shared__ __align__(16) float s[5][NTILE];
    for (int j = threadIdx.x; j < NTILE; j += FT) {
        const float v = (float)((j * 37) % 101) * 0.01f - 0.5f;
        s[0][j] = -v;
        s[1][j] = -(0.3f * v + 0.1f);
        s[2][j] = -(0.7f - v);
        s[3][j] = 0.5f + 0.001f * j;
        s[4][j] = 0.25f;
    }
    __syncthreads();
    float2 tx[2], ty[2], tz[2], z2[2], nfi[2];
    float sum[2] = {0.f, 0.f}, cmp[2] = {0.f, 0.f};
    for (int k = 0; k < 2; k++) {
        tx[k] = dup2(0.01f * (threadIdx.x & 31) + 0.003f * k);
        ty[k] = dup2(0.02f);
        tz[k] = dup2(-0.03f * (threadIdx.x >> 5));
        z2[k] = dup2(0.f);
        nfi[k] = dup2(-0.3f);
    }
    for (int r = 0; r < reps; r++)
        near_tile<KERN, SS, false, false, 2>(s, NTILE, tx, ty, tz, z2, z2, z2, dup2(1.f), nfi, sum, cmp);
    out[blockIdx.x * FT + threadIdx.x] = sum[0] + sum[1] - cmp[0] - cmp[1];
}

template <int KERN, bool SS>
__global__ void __launch_bounds__(FT) pair_peak_far(int reps, float *out) {
    constexpr int N1 = 8;
    __shared__ __align__(16) float s_q[N1 * N1 * N1];
    __shared__ __align__(16) float s_w[N1 * N1 * N1];
    __shared__ float s_p[3][N1];
    for (int k = threadIdx.x; k < N1 * N1 * N1; k += FT) {
        s_q[k] = 0.5f + 0.001f * k;
        s_w[k] = 0.25f;
    }
    if (threadIdx.x < 3 * N1) s_p[threadIdx.x / N1][threadIdx.x % N1] = 1.0f + 0.1f * threadIdx.x;
    __syncthreads();
    float tx[2], ty[2], tz[2], sum[2] = {0.f, 0.f}, cmp[2] = {0.f, 0.f};
    float2 nfi[2];
    for (int k = 0; k < 2; k++) {
        tx[k] = 0.01f * (threadIdx.x & 31) + 0.003f * k;
        ty[k] = 0.02f;
        tz[k] = -0.03f * (threadIdx.x >> 5);
        nfi[k] = dup2(-0.3f);
    }
    for (int r = 0; r < reps; r++)
        far_cluster<KERN, SS, true, N1, 2, true>(s_q, s_w, s_p, N1, tx, ty, tz, nfi, sum, cmp);
    out[blockIdx.x * FT + threadIdx.x] = sum[0] + sum[1] - cmp[0] - cmp[1];
}

// Yukawa orbital groups, 8 orbitals per pair geometry; counted per (pair, orbital).
template <bool SS>
__global__ void __launch_bounds__(FT, 2) pair_peak_near_group(int reps, float *out) {
    constexpr int OG = 8;
    __shared__ __align__(16) float s[4][GTILE];
    __shared__ float4 s_q4[GTILE * OG / 4];
    for (int j = threadIdx.x; j < GTILE; j += FT) {
        const float v = (float)((j * 37) % 101) * 0.01f - 0.5f;
        s[0][j] = -v;
        s[1][j] = -(0.3f * v + 0.1f);
        s[2][j] = -(0.7f - v);
        s[3][j] = 0.25f;
    }
    for (int k = threadIdx.x; k < GTILE * OG; k += FT) reinterpret_cast<float *>(s_q4)[k] = 0.5f + 0.001f * k;
    __syncthreads();
    const float2 tx = dup2(0.01f * (threadIdx.x & 31)), ty = dup2(0.02f), tz = dup2(-0.03f * (threadIdx.x >> 5));
    float2 nfi[OG], kc[OG];
    float sum[OG], cmp[OG];
#pragma unroll
    for (int o = 0; o < OG; o++) {
        kc[o] = dup2((float)(-(0.5 + 0.3 * o) * LOG2E));
        nfi[o] = dup2(-0.3f);
        sum[o] = cmp[o] = 0.f;
    }
    const float2 z = dup2(0.f);
    for (int r = 0; r < reps; r++)
        group_tile<SS, false, false, OG>(s, s_q4, GTILE, tx, ty, tz, z, z, z, nfi, kc, sum, cmp);
    float acc = 0.f;
#pragma unroll
    for (int o = 0; o < OG; o++) acc += sum[o] - cmp[o];
    out[blockIdx.x * FT + threadIdx.x] = acc;
}

// Yukawa orbital groups in the far field: one degree-7 proxy grid, 8 orbitals.
template <bool SS>
__global__ void __launch_bounds__(FT, 2) pair_peak_far_group(int reps, float *out) {
    constexpr int OG = 8, N1 = 8, PP = N1 * N1 * N1;
    __shared__ float4 s_q4[PP * OG / 4];
    __shared__ __align__(16) float s_w[PP];
    __shared__ float s_p[3][N1];
    for (int k = threadIdx.x; k < PP * OG; k += FT) reinterpret_cast<float *>(s_q4)[k] = 0.5f + 0.001f * k;
    for (int k = threadIdx.x; k < PP; k += FT) s_w[k] = 0.25f;
    if (threadIdx.x < 3 * N1) s_p[threadIdx.x / N1][threadIdx.x % N1] = 1.0f + 0.1f * threadIdx.x;
    __syncthreads();
    const float tx = 0.01f * (threadIdx.x & 31), ty = 0.02f, tz = -0.03f * (threadIdx.x >> 5);
    float2 nfi[OG], kc[OG];
    float sum[OG], cmp[OG];
#pragma unroll
    for (int o = 0; o < OG; o++) {
        kc[o] = dup2((float)(-(0.5 + 0.3 * o) * LOG2E));
        nfi[o] = dup2(-0.3f);
        sum[o] = cmp[o] = 0.f;
    }
    for (int r = 0; r < reps; r++)
        far_group_cluster<SS, N1, OG, true>(s_q4, s_w, s_p, N1, tx, ty, tz, nfi, kc, sum, cmp);
    float acc = 0.f;
#pragma unroll
    for (int o = 0; o < OG; o++) acc += sum[o] - cmp[o];
    out[blockIdx.x * FT + threadIdx.x] = acc;
}

// The same two loops with 16 orbitals packed by orbital (near: shared memory
// laid out as near_group16's, dynamic).
constexpr int PEAK16_TILE = GTILE;
template <bool SS>
__global__ void __launch_bounds__(FT, 2) pair_peak_near_group16(int reps, float *out) {
    extern __shared__ __align__(16) float s_dyn[];
    float(*s)[GTILE] = reinterpret_cast<float(*)[GTILE]>(s_dyn);
    float *s_q = s_dyn + 4 * GTILE;
    float *s_k = s_q + GTILE * QS16;
    for (int j = threadIdx.x; j < PEAK16_TILE; j += FT) {
        const float v = (float)((j * 37) % 101) * 0.01f - 0.5f;
        s[0][j] = -v;
        s[1][j] = -(0.3f * v + 0.1f);
        s[2][j] = -(0.7f - v);
        s[3][j] = 0.25f;
    }
    for (int k = threadIdx.x; k < PEAK16_TILE * QS16; k += FT) s_q[k] = 0.5f + 0.001f * k;
    __syncthreads();
    const float2 tx = dup2(0.01f * (threadIdx.x & 31)), ty = dup2(0.02f), tz = dup2(-0.03f * (threadIdx.x >> 5));
    float2 nfi[8], kc[8];
#pragma unroll
    for (int p = 0; p < 8; p++) {
        kc[p] = make_float2((float)(-(0.5 + 0.3 * (2 * p)) * LOG2E), (float)(-(0.5 + 0.3 * (2 * p + 1)) * LOG2E));
        nfi[p] = dup2(-0.3f);
    }
    for (int o = 0; o < 32; o++) s_k[o * FT + threadIdx.x] = 0.f;
    const float2 z = dup2(0.f);
    for (int r = 0; r < reps; r++)
        group16_tile<SS, false, false>(s, s_q, PEAK16_TILE, tx, ty, tz, z, z, z, nfi, kc, s_k);
    float acc = 0.f;
    for (int o = 0; o < 16; o++) acc += s_k[o * FT + threadIdx.x] - s_k[(16 + o) * FT + threadIdx.x];
    out[blockIdx.x * FT + threadIdx.x] = acc;
}

template <bool SS>
__global__ void __launch_bounds__(FT, 2) pair_peak_far_group16(int reps, float *out) {
    constexpr int N1 = 8, PP = N1 * N1 * N1;
    __shared__ __align__(16) float s_q[PP * QS16];
    __shared__ __align__(16) float s_w[PP];
    __shared__ float s_p[3][N1];
    for (int k = threadIdx.x; k < PP * QS16; k += FT) s_q[k] = 0.5f + 0.001f * k;
    for (int k = threadIdx.x; k < PP; k += FT) s_w[k] = 0.25f;
    if (threadIdx.x < 3 * N1) s_p[threadIdx.x / N1][threadIdx.x % N1] = 1.0f + 0.1f * threadIdx.x;
    __syncthreads();
    const float tx = 0.01f * (threadIdx.x & 31), ty = 0.02f, tz = -0.03f * (threadIdx.x >> 5);
    float2 nfi[8], kc[8];
    float sum[16], cmp[16];
#pragma unroll
    for (int p = 0; p < 8; p++) {
        kc[p] = make_float2((float)(-(0.5 + 0.3 * (2 * p)) * LOG2E), (float)(-(0.5 + 0.3 * (2 * p + 1)) * LOG2E));
        nfi[p] = dup2(-0.3f);
    }
#pragma unroll
    for (int o = 0; o < 16; o++) sum[o] = cmp[o] = 0.f;
    for (int r = 0; r < reps; r++)
        far_group16_cluster<SS, N1, true>(s_q, s_w, s_p, N1, tx, ty, tz, nfi, kc, sum, cmp);
    float acc = 0.f;
#pragma unroll
    for (int o = 0; o < 16; o++) acc += sum[o] - cmp[o];
    out[blockIdx.x * FT + threadIdx.x] = acc;
}

template <int KERN, bool SS>
int launch_pair_peak(int variant, int grid, int reps, float *out, cudaStream_t s) {
    if (variant == 0) launch(pair_peak_near<KERN, SS>, grid, FT, 0, s, reps, out);
    else if (variant == 1) launch(pair_peak_far<KERN, SS>, grid, FT, 0, s, reps, out);
    else if (variant == 2) launch(pair_peak_near_group<SS>, grid, FT, 0, s, reps, out);
    else if (variant == 3) launch(pair_peak_far_group<SS>, grid, FT, 0, s, reps, out);
    else if (variant == 4) launch(pair_peak_near_group16<SS>, grid, FT, near_group16_smem(0), s, reps, out);
    else launch(pair_peak_far_group16<SS>, grid, FT, 0, s, reps, out);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

template <int KERN, bool SS>
int run_pair_peak(int variant, double *pairs_per_s, cudaStream_t s) {
    if (variant < 0 || variant > 5)
        return set_error(TAGI_ERR_ARG,
                         "pair peak variant %d (0 near, 1 far, 2 near group, 3 far group, 4 near group of 16, "
                         "5 far group of 16)", variant);
    if (variant >= 2 && KERN != KERNEL_YUKAWA)
        return set_error(TAGI_ERR_UNSUPPORTED, "orbital-group kernels are Yukawa only");
    int grid = 0;
    if (variant == 0) TAGI_TRY(occupancy_grid(pair_peak_near<KERN, SS>, &grid));
    else if (variant == 1) TAGI_TRY(occupancy_grid(pair_peak_far<KERN, SS>, &grid));
    else if (variant == 2) TAGI_TRY(occupancy_grid(pair_peak_near_group<SS>, &grid));
    else if (variant == 3) TAGI_TRY(occupancy_grid(pair_peak_far_group<SS>, &grid));
    else if (variant == 4) {
        TAGI_CUDA(cudaFuncSetAttribute(pair_peak_near_group16<SS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)near_group16_smem(0)));
        TAGI_TRY(occupancy_grid(pair_peak_near_group16<SS>, &grid, near_group16_smem(0)));
    }
    else TAGI_TRY(occupancy_grid(pair_peak_far_group16<SS>, &grid));
    Arena tmp;
    tmp.stream = s;
    float *out = nullptr;
    TAGI_TRY(tmp.alloc(&out, (size_t)grid * FT));
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    // pairs per repetition per thread: two targets x a tile, or one target x a tile x 8 (16) orbitals
    const int per_rep_of[6] = {2 * NTILE, 2 * 512, GTILE * 8, 512 * 8, PEAK16_TILE * 16, 512 * 16};
    const int per_rep = per_rep_of[variant];
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
    int maxn1 = 1;        // largest proxy-grid edge n + 1
    int minn1 = 1 << 20;  // smallest proxy-grid edge n + 1
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
    if (precision == PREC_MIXED && KERN == KERNEL_YUKAWA && sh.og == 16) {
        TAGI_TRY(launch_persistent(near_group16<SS, 0>, wn, s, near_group16_smem(0)));
        phase_mark(PH_NEAR, false, s);
        phase_mark(PH_NEAR_CLOSE, true, s);
        TAGI_TRY(launch_persistent(near_group16<SS, 1>, wc, s, near_group16_smem(1)));
        phase_mark(PH_NEAR_CLOSE, false, s);
        phase_mark(PH_FAR, true, s);
        if (sh.maxn1 <= 4)
            TAGI_TRY(launch_persistent(far_group16<SS, 4, false>, wf, s, far_group16_smem(sh.maxn1)));
        else if (sh.maxn1 == 8 && sh.minn1 == 8)   // degree 7 everywhere: fixed loops
            TAGI_TRY(launch_persistent(far_group16<SS, 8, true>, wf, s, far_group16_smem(8)));
        else if (sh.maxn1 <= 8)
            TAGI_TRY(launch_persistent(far_group16<SS, 8, false>, wf, s, far_group16_smem(sh.maxn1)));
        else
            TAGI_TRY(launch_persistent(far_group16<SS, MAX_DEGREE + 1, false>, wf, s, far_group16_smem(sh.maxn1)));
        phase_mark(PH_FAR, false, s);
        return TAGI_OK;
    }
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
        const size_t fsm = far_group_smem(sh.maxn1, sh.og);
        if (sh.maxn1 <= 4) {
            if (g8) TAGI_TRY(launch_persistent(far_group<SS, 4, 8>, wf, s, fsm));
            else TAGI_TRY(launch_persistent(far_group<SS, 4, 4>, wf, s, fsm));
        } else if (sh.maxn1 == 8 && sh.minn1 == 8) {   // degree 7 everywhere: pipelined staging, fixed loops
            if (g8) TAGI_TRY(launch_persistent(far_group_db<SS, 8>, wf, s, far_group_db_smem(8)));
            else TAGI_TRY(launch_persistent(far_group_db<SS, 4>, wf, s, far_group_db_smem(4)));
        } else if (sh.maxn1 <= 8) {
            if (g8) TAGI_TRY(launch_persistent(far_group<SS, 8, 8>, wf, s, fsm));
            else TAGI_TRY(launch_persistent(far_group<SS, 8, 4>, wf, s, fsm));
        } else {
            if (g8) TAGI_TRY(launch_persistent(far_group<SS, MAX_DEGREE + 1, 8>, wf, s, fsm));
            else TAGI_TRY(launch_persistent(far_group<SS, MAX_DEGREE + 1, 4>, wf, s, fsm));
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
        const bool deg7 = sh.maxn1 == 8 && sh.minn1 == 8;
        if (one) {
            if (sh.maxn1 <= 4) TAGI_TRY(launch_persistent(far_mixed<KERN, SS, 4, 1>, wf, s));
            else if (deg7) TAGI_TRY(launch_persistent(far_mixed<KERN, SS, 8, 1, true>, wf, s));
            else if (sh.maxn1 <= 8) TAGI_TRY(launch_persistent(far_mixed<KERN, SS, 8, 1>, wf, s));
            else TAGI_TRY(launch_persistent(far_mixed<KERN, SS, MAX_DEGREE + 1, 1>, wf, s));
        } else {
            if (sh.maxn1 <= 4) TAGI_TRY(launch_persistent(far_mixed<KERN, SS, 4, 2>, wf, s));
            else if (deg7) TAGI_TRY(launch_persistent(far_mixed<KERN, SS, 8, 2, true>, wf, s));
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
// Mixed precision: the field kernels see k only through the FP32 constant sc
// (k log2(e), or a sqrt(log2(e))), so the subtraction factor uses the k that
// sc represents exactly, k' = sc / log2(e) (a' = sc / sqrt(log2(e))): sums and
// subtraction term then belong to one kernel parameter, k' = k (1 + O(2^-24)),
// and the rounding of k moves the result by about twice that, smoothly,
// instead of entering the cancellation of the subtraction.
__global__ void orbital_constants(const double *__restrict__ kp, int nkp, int norb, int kernel, int sing,
                                  int mixed, double *__restrict__ kpo, float *__restrict__ kc,
                                  double *__restrict__ ss, int *__restrict__ err) {
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
    double ke = k;
    if (mixed && kernel == KERNEL_YUKAWA) ke = (double)c / LOG2E;
    else if (mixed && sing == SING_SUBTRACTION) ke = (double)c / sqrt(LOG2E);
    if (sing == SING_SUBTRACTION) f = (kernel == KERNEL_YUKAWA ? 4.0 : 2.0) * M_PI / (ke * ke);
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
// geometry across a group of 4, 8 or 16 orbitals; everything else (and fewer
// than 4 orbitals) runs one orbital per item.  The choice minimises a cost
// model measured on GB300 (1M-point mesh, degree 7): a pass over all batches
// costs 1.0 per group of 8 (padded slots cost as much as filled ones), 0.59
// per group of 4, and 0.345 + 0.18 np per group of 16 with np filled orbital
// pairs (its kernels skip empty pairs); systems weigh by their point counts.
// Groups of 16 only up to degree 7: above it a 16-orbital proxy grid no
// longer fits two CTAs per SM.  requested > 0 (1, 4, 8 or 16) overrides the
// choice where the kernel supports it.
double group_cost(int og, int norb) {
    if (og == 16) {
        const int full = norb / 16, rem = norb % 16;
        return full * (0.345 + 0.18 * 8) + (rem ? 0.345 + 0.18 * ((rem + 1) / 2) : 0.0);
    }
    if (og == 8) return 1.0 * ((norb + 7) / 8);
    return 0.59 * ((norb + 3) / 4);
}

int orbitals_per_item(int kernel, int precision, const int *norb, const double *weight, int nsys, int requested,
                      int max_n1) {
    if (kernel != KERNEL_YUKAWA || precision != PREC_MIXED) return 1;
    if (requested == 1 || requested == 4 || requested == 8 || requested == 16) return requested;
    int maxo = 0;
    for (int i = 0; i < nsys; i++) maxo = norb[i] > maxo ? norb[i] : maxo;
    if (maxo < 4) return 1;
    int best = 0;
    double best_cost = 0.0;
    for (int og : {4, 8, 16}) {
        if (og == 16 && max_n1 > 8) continue;
        double c = 0.0;
        for (int i = 0; i < nsys; i++) c += (weight ? weight[i] : 1.0) * group_cost(og, norb[i]);
        if (!best || c < best_cost) {
            best = og;
            best_cost = c;
        }
    }
    return best;
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
static int orbital_setup(Plan &p, const SysCall &c, int kernel, int singularity, int mixed, cudaStream_t s) {
    const double *src = c.kp;
    int stride = c.nkp;
    if (!c.kp_device) {
        p.h_kp.resize(c.norb);
        for (int o = 0; o < c.norb; o++) p.h_kp[o] = c.kp[(long)o * c.nkp];
        TAGI_CUDA(cudaMemcpyAsync(p.d_kp, p.h_kp.data(), sizeof(double) * c.norb, cudaMemcpyHostToDevice, s));
        src = p.d_kp;
        stride = 1;
    }
    launch(orbital_constants, (c.norb + 127) / 128, 128, 0, s, src, stride, c.norb, kernel, singularity, mixed,
           p.d_kp, p.d_kc, p.d_ss, p.err_flag + 1);
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
        TAGI_TRY(orbital_setup(p, c, kernel, singularity, mixed ? 1 : 0, s));
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
        if (p.n1 < sh.minn1) sh.minn1 = p.n1;
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
    const int og = orbitals_per_item(kernel, precision, &norb, nullptr, 1, og_request, p.n1);
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
