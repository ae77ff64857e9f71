// Subsystem (b): upward pass.  For every far-field cluster ("slot") the
// modified charges on its (n+1)^3 Chebyshev 2nd-kind proxy grid,
//     qhat_k = sum_{j in cluster} L_k1(u_jx) L_k2(u_jy) L_k3(u_jz) q_j ,
// with the barycentric Lagrange basis on nodes cos(m pi / n) and weights
// (-1)^m (halved at both ends), u = (y - c) / h in the slot's proxy box.
// k = (k1 * (n+1) + k2) * (n+1) + k3, x-major like the reference's cells.
//
// Work items are (slot, chunk of <= 2048 sorted sources); each item writes
// FP64 partial sums and a second kernel adds the partials of a slot in item
// order, so results do not depend on scheduling.  The weight charges (q = w)
// are built once per plan in FP64; charge vectors are done per call, in FP32
// products with FP64 accumulation across tiles (mixed) or all in FP64.
#include "tagi_internal.h"

namespace tagi {

namespace {

constexpr int P2M_THREADS = 256;
constexpr int P2M_TILE = 64;

template <typename T>
struct P2MArgs {
    const int *item_slot, *item_begin, *item_end;
    int nitems;
    const double *geom;          // [slot][6]
    const double *xs, *ys, *zs;  // sorted sources
    const T *q;                  // [norb][ns] sorted charges
    long q_stride;
    double *part;                // [norb][nitems][P]
    int n1, P;
    T tn[MAX_DEGREE + 1];
};

template <typename T>
__device__ __forceinline__ T bary_weight(int m, int n1) {
    T w = (m & 1) ? T(-1) : T(1);
    if (m == 0 || m == n1 - 1) w *= T(0.5);
    return w;
}

template <typename T, int MAXN1>
__global__ void __launch_bounds__(P2M_THREADS) p2m_kernel(P2MArgs<T> a) {
    extern __shared__ double red[];  // [G][P]
    __shared__ T sL[3][P2M_TILE][MAXN1];
    __shared__ T sq[P2M_TILE];
    const int item = blockIdx.x, orb = blockIdx.y;
    const int n1 = a.n1, pairs = n1 * n1, P = a.P;
    const int G = P2M_THREADS / pairs;
    const int tid = threadIdx.x;
    const int g = tid / pairs, pr = tid % pairs;
    const int k1 = pr / n1, k2 = pr % n1;
    const bool active = g < G;
    const int slot = a.item_slot[item];
    const int b = a.item_begin[item], e = a.item_end[item];
    const double *gm = a.geom + 6L * slot;
    const T *q = a.q + (long)orb * a.q_stride;

    double acc[MAXN1];
#pragma unroll
    for (int m = 0; m < MAXN1; m++) acc[m] = 0.0;

    for (int t0 = b; t0 < e; t0 += P2M_TILE) {
        const int cnt = min(P2M_TILE, e - t0);
        if (tid < 3 * cnt) {
            const int p = tid / 3, d = tid - 3 * (tid / 3);
            const double *src = d == 0 ? a.xs : (d == 1 ? a.ys : a.zs);
            T u = (T)((src[t0 + p] - gm[d]) / gm[3 + d]);
            int exact = -1;
            for (int m = 0; m < n1; m++)
                if (u - a.tn[m] == T(0)) exact = m;
            if (exact >= 0) {
                for (int m = 0; m < n1; m++) sL[d][p][m] = (m == exact) ? T(1) : T(0);
            } else {
                T s = T(0);
                for (int m = 0; m < n1; m++) {
                    T l = bary_weight<T>(m, n1) / (u - a.tn[m]);
                    sL[d][p][m] = l;
                    s += l;
                }
                for (int m = 0; m < n1; m++) sL[d][p][m] = sL[d][p][m] / s;
            }
        }
        if (tid < cnt) sq[tid] = q[t0 + tid];
        __syncthreads();
        if (active) {
            T tacc[MAXN1];
#pragma unroll
            for (int m = 0; m < MAXN1; m++) tacc[m] = T(0);
            for (int p = g; p < cnt; p += G) {
                T axy = sL[0][p][k1] * sL[1][p][k2] * sq[p];
#pragma unroll
                for (int m = 0; m < MAXN1; m++)
                    if (m < n1) tacc[m] += axy * sL[2][p][m];
            }
#pragma unroll
            for (int m = 0; m < MAXN1; m++) acc[m] += (double)tacc[m];
        }
        __syncthreads();
    }
    if (active) {
#pragma unroll
        for (int m = 0; m < MAXN1; m++)
            if (m < n1) red[(long)g * P + (k1 * n1 + k2) * n1 + m] = acc[m];
    }
    __syncthreads();
    double *out = a.part + ((long)orb * a.nitems + item) * P;
    for (int k = tid; k < P; k += P2M_THREADS) {
        double s = 0.0;
        for (int gg = 0; gg < G; gg++) s += red[(long)gg * P + k];
        out[k] = s;
    }
}

template <typename TO>
__global__ void p2m_reduce(const double *__restrict__ part, const int *__restrict__ slot_item_off,
                           int nslots, int nitems, int P, TO *__restrict__ out) {
    const int slot = blockIdx.x, orb = blockIdx.y;
    const int i0 = slot_item_off[slot], i1 = slot_item_off[slot + 1];
    const double *pp = part + (long)orb * nitems * P;
    TO *o = out + ((long)orb * nslots + slot) * P;
    for (int k = threadIdx.x; k < P; k += blockDim.x) {
        double s = 0.0;
        for (int it = i0; it < i1; it++) s += pp[(long)it * P + k];
        o[k] = (TO)s;
    }
}

template <typename T>
int launch_p2m(Plan &p, const T *q, long q_stride, int norb, double *part, cudaStream_t s) {
    P2MArgs<T> a;
    a.item_slot = p.item_slot;
    a.item_begin = p.item_begin;
    a.item_end = p.item_end;
    a.nitems = p.nitems;
    a.geom = p.slot_geom;
    a.xs = p.src.x;
    a.ys = p.src.y;
    a.zs = p.src.z;
    a.q = q;
    a.q_stride = q_stride;
    a.part = part;
    a.n1 = p.n1;
    a.P = p.P;
    for (int m = 0; m <= MAX_DEGREE; m++) a.tn[m] = (T)(m <= p.degree ? p.cheb[m] : 0.0);
    const int G = P2M_THREADS / (p.n1 * p.n1);
    const size_t smem = sizeof(double) * (size_t)G * p.P;
    dim3 grid(p.nitems, norb);
    if (p.n1 <= 8) {
        if (smem > 48 * 1024)
            cudaFuncSetAttribute(p2m_kernel<T, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        launch(p2m_kernel<T, 8>, grid, P2M_THREADS, smem, s, a);
    } else {
        if (smem > 48 * 1024)
            cudaFuncSetAttribute(p2m_kernel<T, MAX_DEGREE + 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
        launch(p2m_kernel<T, MAX_DEGREE + 1>, grid, P2M_THREADS, smem, s, a);
    }
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

}  // namespace

// Weight modified charges (q = w).  The mixed path uses charges built with
// the same FP32 products as its charge vectors, so qhat - f_i what keeps the
// subtraction's structure; the FP64 set is built on first use by an FP64 call.
int build_weight_charges(Plan &p, cudaStream_t s) {
    TAGI_TRY(p.arena.alloc(&p.what32, (size_t)p.nslots * p.P));
    p.what64_ready = false;
    if (p.nslots == 0) return TAGI_OK;
    Arena tmp;
    tmp.stream = s;
    double *part = nullptr;
    int rc = tmp.alloc(&part, (size_t)p.nitems * p.P);
    if (!rc) rc = launch_p2m<float>(p, p.sw32, p.src.n, 1, part, s);
    if (!rc) {
        launch(p2m_reduce<float>, dim3(p.nslots, 1), 256, 0, s, part, p.slot_item_off, p.nslots, p.nitems, p.P,
               p.what32);
        if (cudaGetLastError() != cudaSuccess) rc = set_error(TAGI_ERR_CUDA, "weight charge kernels");
    }
    tmp.release();
    return rc;
}

int ensure_weight_charges64(Plan &p, cudaStream_t s) {
    if (p.what64_ready) return TAGI_OK;
    if (!p.what64) {
        // plain cudaMalloc: the first FP64 call may run on another stream than the plan's
        void *v = nullptr;
        TAGI_CUDA(cudaMalloc(&v, sizeof(double) * ((size_t)p.nslots * p.P + 1)));
        p.arena.ptrs.push_back(v);
        p.what64 = static_cast<double *>(v);
    }
    if (p.nslots) {
        Arena tmp;
        tmp.stream = s;
        double *part = nullptr;
        int rc = tmp.alloc(&part, (size_t)p.nitems * p.P);
        if (!rc) rc = launch_p2m<double>(p, p.sw64, p.src.n, 1, part, s);
        if (!rc) {
            launch(p2m_reduce<double>, dim3(p.nslots, 1), 256, 0, s, part, p.slot_item_off, p.nslots, p.nitems,
                   p.P, p.what64);
            if (cudaGetLastError() != cudaSuccess) rc = set_error(TAGI_ERR_CUDA, "weight charge kernels");
        }
        tmp.release();
        if (rc) return rc;
    }
    p.what64_ready = true;
    return TAGI_OK;
}

// Charges for norb sorted charge vectors already in p.q32 / p.q64.
int modified_charges(Plan &p, int precision, int norb, cudaStream_t s) {
    if (p.nslots == 0) return TAGI_OK;
    if (precision == PREC_MIXED) {
        TAGI_TRY(launch_p2m<float>(p, p.q32, p.src.n, norb, p.part, s));
        launch(p2m_reduce<float>, dim3(p.nslots, norb), 256, 0, s, p.part, p.slot_item_off, p.nslots,
                                                               p.nitems, p.P, p.qhat32);
    } else {
        TAGI_TRY(launch_p2m<double>(p, p.q64, p.src.n, norb, p.part, s));
        launch(p2m_reduce<double>, dim3(p.nslots, norb), 256, 0, s, p.part, p.slot_item_off, p.nslots,
                                                                p.nitems, p.P, p.qhat64);
    }
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

}  // namespace tagi
