// Learned extrapolation of Green iteration: a small MLP on per-cell patches,
// trained on the device by this file's kernels.  No counterpart in the
// reference (its closest relative is the Anderson mixing of orbitals,
// scfFixedPoint.py:491-597); the plain Green-iteration residual checks every
// proposal, so the plain method stays the fallback.
//
// Rows are (orbital, cell) patches of P = (order+1)^3 mesh points (the mesh
// stores each cell's points contiguously).  Features of a row, in BF16:
//   [ psi / s_psi (P), d / s_d (P), eps, 0 padding ]   d = psi_t - psi_{t-1}
// with s_psi, s_d the patch RMS values (s_d floored by a fraction of the
// orbital's RMS update).  The network predicts the next update of the patch
// in units of s_d:  d_next / s_d ~ alpha * d / s_d + MLP(features).
// MLP: Linear(Din -> H) ReLU Linear(H -> H) ReLU Linear(H -> P), weights BF16
// (FP32 master copies for Adam), every product accumulated in FP32.
//
// GEMMs run on the tensor cores with warp-level mma.sync (m16n8k16, BF16
// in, FP32 accumulate): C[M x N] = A[M x K] B[K x N] with arbitrary strides,
// so the transposes of the backward pass need no copies.  Weight gradients
// split K across blocks into partial sums that a second kernel adds in a
// fixed order: results do not depend on scheduling.
#include "tagi_internal.h"

#include <cuda_bf16.h>

namespace tagi {

namespace {

constexpr int BM = 64, BN = 64, BK = 32;
constexpr int GEMM_THREADS = 128;  // 4 warps, 2 x 2, 32 x 32 each

enum { EPI_F32 = 0, EPI_BIAS_RELU_BF16 = 1, EPI_MASK_BF16 = 2, EPI_BIAS_F32 = 3 };

struct GemmArgs {
    const __nv_bfloat16 *A, *B;
    long sAm, sAk, sBk, sBn;
    int M, N, K;
    int k_per_split;     // K range of one blockIdx.z
    float *C32;          // f32 output (or partials [split][M][N])
    __nv_bfloat16 *C16;  // bf16 output
    long sCm;            // output row stride (elements)
    const float *bias;   // [N]
    const __nv_bfloat16 *mask;  // [M][sCm]: multiply by (mask > 0)
    int epi;
};

__device__ __forceinline__ unsigned pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return (unsigned)__bfloat16_as_ushort(lo) | ((unsigned)__bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], unsigned a0, unsigned a1, unsigned a2, unsigned a3,
                                         unsigned b0, unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__global__ void __launch_bounds__(GEMM_THREADS) gemm_bf16(const GemmArgs g) {
    __shared__ __nv_bfloat16 As[BM][BK + 8];
    __shared__ __nv_bfloat16 Bs[BK][BN + 8];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const int kb = blockIdx.z * g.k_per_split;
    const int ke = min(g.K, kb + g.k_per_split);
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int e = 0; e < 4; e++) acc[i][j][e] = 0.f;
    for (int k0 = kb; k0 < ke; k0 += BK) {
        // stage A[m0..m0+63][k0..k0+31] and B[k0..k0+31][n0..n0+63], zero outside
        for (int e = tid; e < BM * BK; e += GEMM_THREADS) {
            const int r = e / BK, c = e - r * BK;
            const int m = m0 + r, k = k0 + c;
            As[r][c] = (m < g.M && k < ke) ? g.A[(long)m * g.sAm + (long)k * g.sAk] : zero;
        }
        for (int e = tid; e < BK * BN; e += GEMM_THREADS) {
            const int r = e / BN, c = e - r * BN;
            const int k = k0 + r, n = n0 + c;
            Bs[r][c] = (k < ke && n < g.N) ? g.B[(long)k * g.sBk + (long)n * g.sBn] : zero;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; kk += 16) {
            unsigned af[2][4], bfr[4][2];
            const int ar = lane >> 2, ac = kk + 2 * (lane & 3);
#pragma unroll
            for (int i = 0; i < 2; i++) {
                const int r = wm + i * 16 + ar;
                af[i][0] = pack2(As[r][ac], As[r][ac + 1]);
                af[i][1] = pack2(As[r + 8][ac], As[r + 8][ac + 1]);
                af[i][2] = pack2(As[r][ac + 8], As[r][ac + 9]);
                af[i][3] = pack2(As[r + 8][ac + 8], As[r + 8][ac + 9]);
            }
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int n = wn + j * 8 + (lane >> 2);
                bfr[j][0] = pack2(Bs[ac][n], Bs[ac + 1][n]);
                bfr[j][1] = pack2(Bs[ac + 8][n], Bs[ac + 9][n]);
            }
#pragma unroll
            for (int i = 0; i < 2; i++)
#pragma unroll
                for (int j = 0; j < 4; j++)
                    mma_bf16(acc[i][j], af[i][0], af[i][1], af[i][2], af[i][3], bfr[j][0], bfr[j][1]);
        }
        __syncthreads();
    }
    // epilogue: fragment element e -> row (lane/4) + 8 (e >= 2), col 2 (lane%4) + (e & 1)
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int m = m0 + wm + i * 16 + (lane >> 2) + (e >= 2 ? 8 : 0);
                const int n = n0 + wn + j * 8 + 2 * (lane & 3) + (e & 1);
                if (m >= g.M || n >= g.N) continue;
                float v = acc[i][j][e];
                const long o = (long)m * g.sCm + n;
                if (g.epi == EPI_F32) {
                    g.C32[(long)blockIdx.z * g.M * g.sCm + o] = v;
                } else if (g.epi == EPI_BIAS_F32) {
                    g.C32[o] = v + g.bias[n];
                } else if (g.epi == EPI_BIAS_RELU_BF16) {
                    v += g.bias[n];
                    g.C16[o] = __float2bfloat16_rn(v > 0.f ? v : 0.f);
                } else {  // EPI_MASK_BF16
                    const float keep = __bfloat162float(g.mask[o]) > 0.f ? 1.f : 0.f;
                    g.C16[o] = __float2bfloat16_rn(v * keep);
                }
            }
}

// out[m][n] = sum over splits of part[s][m][n] (fixed order)
__global__ void splitk_reduce(const float *__restrict__ part, int splits, long mn, float *__restrict__ out) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= mn) return;
    float s = 0.f;
    for (int k = 0; k < splits; k++) s += part[(long)k * mn + i];
    out[i] = s;
}

// ---------------------------------------------------------------------------
// Patch features.  One block per row (orbital m, cell c).
// ---------------------------------------------------------------------------
constexpr int PT = 128;

__device__ __forceinline__ float block_sum_f(float v, float *sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    float s = 0.f;
    for (int w = 0; w < PT / 32; w++) s += sh[w];
    return s;  // every thread
}

// X[row] = [psi/s_psi, d/s_d, eps, 0...]; scale[row] = s_d; dn[row] = d/s_d (f32, for the skip term)
__global__ void __launch_bounds__(PT) patch_features(const double *__restrict__ psi, const double *__restrict__ d,
                                                     const double *__restrict__ eps, const double *__restrict__ dfloor,
                                                     int ncell, int P, long n, int ldx,
                                                     __nv_bfloat16 *__restrict__ X, float *__restrict__ scale,
                                                     float *__restrict__ dn) {
    __shared__ float sh[PT / 32];
    const int row = blockIdx.x;
    const int m = row / ncell, c = row - m * ncell;
    const double *pp = psi + (long)m * n + (long)c * P;
    const double *dd = d + (long)m * n + (long)c * P;
    float sp = 0.f, sd = 0.f;
    for (int i = threadIdx.x; i < P; i += PT) {
        const float a = (float)pp[i], b = (float)dd[i];
        sp += a * a;
        sd += b * b;
    }
    sp = block_sum_f(sp, sh);
    sd = block_sum_f(sd, sh);
    const float rp = sqrtf(sp / P) + 1e-30f;
    const float rd = fmaxf(sqrtf(sd / P), (float)dfloor[m]) + 1e-30f;
    __nv_bfloat16 *x = X + (long)row * ldx;
    for (int i = threadIdx.x; i < P; i += PT) {
        const float b = (float)dd[i] / rd;
        x[i] = __float2bfloat16_rn((float)pp[i] / rp);
        x[P + i] = __float2bfloat16_rn(b);
        dn[(long)row * P + i] = b;
    }
    for (int i = 2 * P + threadIdx.x; i < ldx; i += PT) x[i] = __float2bfloat16_rn(i == 2 * P ? (float)eps[m] : 0.f);
    if (threadIdx.x == 0) scale[row] = rd;
}

// target T = d_next / s_d (per row, from the same scale as the inputs)
__global__ void patch_target(const double *__restrict__ dnext, const float *__restrict__ scale, int ncell, int P,
                             long n, float *__restrict__ T) {
    const int row = blockIdx.x;
    const int m = row / ncell, c = row - m * ncell;
    const double *dd = dnext + (long)m * n + (long)c * P;
    const float s = scale[row];
    for (int i = threadIdx.x; i < P; i += blockDim.x) T[(long)row * P + i] = (float)dd[i] / s;
}

// Residual of the prediction and its gradient:
//   r = alpha dn + Y - T;  loss partial = sum r^2;  dY = 2 r / (rows P);  dalpha partial = sum dY dn
__global__ void __launch_bounds__(PT) mse_grad(const float *__restrict__ Y, const float *__restrict__ dn,
                                               const float *__restrict__ T, const float *__restrict__ alpha, int P,
                                               float inv_count, float *__restrict__ dY, __nv_bfloat16 *__restrict__ dY16,
                                               float *__restrict__ part) {
    __shared__ float sh[PT / 32];
    const int row = blockIdx.x;
    const float a = *alpha;
    float l = 0.f, ga = 0.f;
    for (int i = threadIdx.x; i < P; i += PT) {
        const long o = (long)row * P + i;
        const float r = a * dn[o] + Y[o] - T[o];
        const float g = 2.f * r * inv_count;
        dY[o] = g;
        dY16[o] = __float2bfloat16_rn(g);
        l += r * r;
        ga += g * dn[o];
    }
    l = block_sum_f(l, sh);
    ga = block_sum_f(ga, sh);
    if (threadIdx.x == 0) {
        part[2L * row] = l;
        part[2L * row + 1] = ga;
    }
}

// Column sums of a [rows x N] matrix (bias gradients; f32, or bf16 for the
// hidden layers' gradients): chunk b of COL_ROWS rows -> part[b][N], then the
// chunks are added in order.
constexpr int COL_ROWS = 1024;

template <typename T>
__device__ __forceinline__ float to_f(T v);
template <>
__device__ __forceinline__ float to_f<float>(float v) { return v; }
template <>
__device__ __forceinline__ float to_f<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }

template <typename T>
__global__ void colsum_partial(const T *__restrict__ G, long rows, int N, float *__restrict__ part) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    const long r0 = (long)blockIdx.y * COL_ROWS, r1 = min(rows, r0 + COL_ROWS);
    float s = 0.f;
    for (long r = r0; r < r1; r++) s += to_f(G[r * N + j]);
    part[(long)blockIdx.y * N + j] = s;
}

__global__ void colsum_final(const float *__restrict__ part, int chunks, int N, float *__restrict__ out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    float s = 0.f;
    for (int b = 0; b < chunks; b++) s += part[(long)b * N + j];
    out[j] = s;
}

// loss and dalpha from the per-row partials: thread t adds rows t, t + 256,
// ..., then a fixed tree over the threads
__global__ void __launch_bounds__(256) rows_reduce2(const float *__restrict__ part, int rows,
                                                   float *__restrict__ out) {
    __shared__ float sa[256], sb[256];
    float a = 0.f, b = 0.f;
    for (int r = threadIdx.x; r < rows; r += 256) {
        a += part[2L * r];
        b += part[2L * r + 1];
    }
    sa[threadIdx.x] = a;
    sb[threadIdx.x] = b;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if (threadIdx.x < h) {
            sa[threadIdx.x] += sa[threadIdx.x + h];
            sb[threadIdx.x] += sb[threadIdx.x + h];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = sa[0];
        out[1] = sb[0];
    }
}

// Adam on FP32 master weights; the BF16 copy the GEMMs read is refreshed.
__global__ void adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m1,
                     float *__restrict__ m2, long n, float lr, float b1, float b2, float eps, float c1, float c2,
                     __nv_bfloat16 *__restrict__ w16) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float a = b1 * m1[i] + (1.f - b1) * gi;
    const float b = b2 * m2[i] + (1.f - b2) * gi * gi;
    m1[i] = a;
    m2[i] = b;
    const float v = w[i] - lr * (a / c1) / (sqrtf(b / c2) + eps);
    w[i] = v;
    if (w16) w16[i] = __float2bfloat16_rn(v);
}

// psi_next = psi + s_d (alpha dn + Y) per patch; d_next = the same increment
__global__ void patch_apply(const double *__restrict__ psi, const float *__restrict__ Y,
                            const float *__restrict__ dn, const float *__restrict__ scale,
                            const float *__restrict__ alpha, int ncell, int P, long n, double *__restrict__ psi_out,
                            double *__restrict__ d_out) {
    const int row = blockIdx.x;
    const int m = row / ncell, c = row - m * ncell;
    const long base = (long)m * n + (long)c * P;
    const float s = scale[row], a = *alpha;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        const long o = (long)row * P + i;
        const double inc = (double)s * (double)(a * dn[o] + Y[o]);
        psi_out[base + i] = psi[base + i] + inc;
        d_out[base + i] = inc;
    }
}

__global__ void f32_to_bf16(const float *__restrict__ a, long n, __nv_bfloat16 *__restrict__ b) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = __float2bfloat16_rn(a[i]);
}

}  // namespace

}  // namespace tagi

using namespace tagi;

extern "C" {

// C[M x N] = A[M x K] B[K x N] (+ epilogue), BF16 operands, FP32 accumulation;
// element (m, k) of A at A[m sAm + k sAk], (k, n) of B at B[k sBk + n sBn].
// epilogue 0: f32 C; 1: bf16 relu(C + bias); 2: bf16 C * (mask > 0);
// 3: f32 C + bias.
int tagi_mlp_gemm(const void *A, long long sAm, long long sAk, const void *B, long long sBk, long long sBn, int M,
                  int N, int K, int epilogue, float *C32, void *C16, long long ldc, const float *bias,
                  const void *mask, void *stream) {
    if (!A || !B || M <= 0 || N <= 0 || K <= 0) return set_error(TAGI_ERR_ARG, "bad GEMM arguments");
    if (epilogue < 0 || epilogue > 3) return set_error(TAGI_ERR_ARG, "epilogue %d", epilogue);
    if ((epilogue == 0 || epilogue == 3) && !C32) return set_error(TAGI_ERR_ARG, "null f32 output");
    if ((epilogue == 1 || epilogue == 2) && !C16) return set_error(TAGI_ERR_ARG, "null bf16 output");
    if ((epilogue == 1 || epilogue == 3) && !bias) return set_error(TAGI_ERR_ARG, "null bias");
    if (epilogue == 2 && !mask) return set_error(TAGI_ERR_ARG, "null mask");
    if (ldc < N) return set_error(TAGI_ERR_ARG, "ldc < N");
    GemmArgs g;
    g.A = static_cast<const __nv_bfloat16 *>(A);
    g.B = static_cast<const __nv_bfloat16 *>(B);
    g.sAm = sAm;
    g.sAk = sAk;
    g.sBk = sBk;
    g.sBn = sBn;
    g.M = M;
    g.N = N;
    g.K = K;
    g.k_per_split = ((K + BK - 1) / BK) * BK;
    g.C32 = C32;
    g.C16 = static_cast<__nv_bfloat16 *>(C16);
    g.sCm = ldc;
    g.bias = bias;
    g.mask = static_cast<const __nv_bfloat16 *>(mask);
    g.epi = epilogue;
    dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, 1);
    launch(gemm_bf16, grid, GEMM_THREADS, 0, (cudaStream_t)stream, g);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

// f32 C = A B with K split over `splits` blocks; `partial` holds
// splits * M * N floats; C = sum of the partials in split order.
int tagi_mlp_gemm_splitk(const void *A, long long sAm, long long sAk, const void *B, long long sBk, long long sBn,
                         int M, int N, int K, int splits, float *partial, float *C, void *stream) {
    if (!A || !B || !partial || !C || M <= 0 || N <= 0 || K <= 0 || splits < 1)
        return set_error(TAGI_ERR_ARG, "bad split-K GEMM arguments");
    GemmArgs g;
    g.A = static_cast<const __nv_bfloat16 *>(A);
    g.B = static_cast<const __nv_bfloat16 *>(B);
    g.sAm = sAm;
    g.sAk = sAk;
    g.sBk = sBk;
    g.sBn = sBn;
    g.M = M;
    g.N = N;
    g.K = K;
    int kps = (K + splits - 1) / splits;
    kps = ((kps + BK - 1) / BK) * BK;
    splits = (K + kps - 1) / kps;
    g.k_per_split = kps;
    g.C32 = partial;
    g.C16 = nullptr;
    g.sCm = N;
    g.bias = nullptr;
    g.mask = nullptr;
    g.epi = EPI_F32;
    cudaStream_t s = (cudaStream_t)stream;
    dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, splits);
    launch(gemm_bf16, grid, GEMM_THREADS, 0, s, g);
    const long mn = (long)M * N;
    launch(splitk_reduce, (unsigned)((mn + 255) / 256), 256, 0, s, partial, splits, mn, C);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

int tagi_mlp_patch_features(const double *psi, const double *d, const double *eps, const double *dfloor,
                            int numOrbitals, int numCells, int P, long long numPoints, int ldx, void *X,
                            float *scale, float *dn, void *stream) {
    if (!psi || !d || !eps || !dfloor || !X || !scale || !dn) return set_error(TAGI_ERR_ARG, "null pointer");
    if ((long long)numCells * P != numPoints) return set_error(TAGI_ERR_ARG, "cells x P != points");
    if (ldx < 2 * P + 1) return set_error(TAGI_ERR_ARG, "ldx < 2P + 1");
    launch(patch_features, numOrbitals * numCells, PT, 0, (cudaStream_t)stream, psi, d, eps, dfloor, numCells, P,
           (long)numPoints, ldx, static_cast<__nv_bfloat16 *>(X), scale, dn);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

int tagi_mlp_patch_target(const double *dnext, const float *scale, int numOrbitals, int numCells, int P,
                          long long numPoints, float *T, void *stream) {
    if (!dnext || !scale || !T) return set_error(TAGI_ERR_ARG, "null pointer");
    launch(patch_target, numOrbitals * numCells, PT, 0, (cudaStream_t)stream, dnext, scale, numCells, P,
           (long)numPoints, T);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

int tagi_mlp_mse_grad(const float *Y, const float *dn, const float *T, const float *alpha, int rows, int P,
                      float *dY, void *dY16, float *part, float *lossAndDalpha, void *stream) {
    if (!Y || !dn || !T || !alpha || !dY || !dY16 || !part || !lossAndDalpha)
        return set_error(TAGI_ERR_ARG, "null pointer");
    cudaStream_t s = (cudaStream_t)stream;
    launch(mse_grad, rows, PT, 0, s, Y, dn, T, alpha, P, 1.f / ((float)rows * (float)P), dY,
           static_cast<__nv_bfloat16 *>(dY16), part);
    launch(rows_reduce2, 1, 256, 0, s, part, rows, lossAndDalpha);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

long long tagi_mlp_colsum_workspace(long long rows, int N) {
    return ((rows + COL_ROWS - 1) / COL_ROWS) * (long long)N;
}

int tagi_mlp_colsum(const void *G, int isBf16, long long rows, int N, float *out, float *work, long long workFloats,
                    void *stream) {
    if (!G || !out || !work || rows <= 0 || N <= 0) return set_error(TAGI_ERR_ARG, "bad column-sum arguments");
    if (workFloats < tagi_mlp_colsum_workspace(rows, N)) return set_error(TAGI_ERR_ARG, "workspace too small");
    cudaStream_t s = (cudaStream_t)stream;
    const int chunks = (int)((rows + COL_ROWS - 1) / COL_ROWS);
    dim3 g((N + 127) / 128, chunks);
    if (isBf16)
        launch(colsum_partial<__nv_bfloat16>, g, 128, 0, s, static_cast<const __nv_bfloat16 *>(G), (long)rows, N,
               work);
    else
        launch(colsum_partial<float>, g, 128, 0, s, static_cast<const float *>(G), (long)rows, N, work);
    launch(colsum_final, (N + 127) / 128, 128, 0, s, work, chunks, N, out);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

int tagi_mlp_adam(float *w, const float *g, float *m1, float *m2, long long n, float lr, float beta1, float beta2,
                  float epsilon, int step, void *w16, void *stream) {
    if (!w || !g || !m1 || !m2 || n <= 0 || step < 1) return set_error(TAGI_ERR_ARG, "bad Adam arguments");
    const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
    launch(adam, (unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream, w, g, m1, m2, (long)n, lr, beta1, beta2,
           epsilon, c1, c2, static_cast<__nv_bfloat16 *>(w16));
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

int tagi_mlp_patch_apply(const double *psi, const float *Y, const float *dn, const float *scale, const float *alpha,
                         int numOrbitals, int numCells, int P, long long numPoints, double *psiOut, double *dOut,
                         void *stream) {
    if (!psi || !Y || !dn || !scale || !alpha || !psiOut || !dOut) return set_error(TAGI_ERR_ARG, "null pointer");
    launch(patch_apply, numOrbitals * numCells, PT, 0, (cudaStream_t)stream, psi, Y, dn, scale, alpha, numCells, P,
           (long)numPoints, psiOut, dOut);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

int tagi_mlp_to_bf16(const float *a, long long n, void *b, void *stream) {
    if (!a || !b || n <= 0) return set_error(TAGI_ERR_ARG, "bad arguments");
    launch(f32_to_bf16, (unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream, a, (long)n,
           static_cast<__nv_bfloat16 *>(b));
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

}  // extern "C"
