// Device-wide exclusive scan (int32) and stable LSD radix sort of 64-bit
// Morton codes with int32 payloads.  Integer work for the tree build: the
// sort fixes the point order every later kernel reads, so it must be stable
// (equal codes keep caller order) to give lists identical to the CPU oracle,
// which sorts by (code, index).
#include "tagi_internal.h"

namespace tagi {

namespace {

constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ int warp_incl_scan(int v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Exclusive scan of one tile per block; writes the tile total to sums[block].
__global__ void __launch_bounds__(SCAN_THREADS) scan_tiles(const int *__restrict__ in,
                                                           int *__restrict__ out, int n,
                                                           int *__restrict__ sums) {
    __shared__ int warp_tot[SCAN_THREADS / 32];
    const long base = (long)blockIdx.x * SCAN_TILE + (long)threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS];
    int tsum = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        long i = base + k;
        v[k] = (i < n) ? in[i] : 0;
        tsum += v[k];
    }
    int incl = warp_incl_scan(tsum);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        int w = warp_tot[lane];
        int wi = warp_incl_scan(w);
        warp_tot[lane] = wi - w;
        if (lane == 31) sums[blockIdx.x] = wi;
    }
    __syncthreads();
    int run = warp_tot[wid] + incl - tsum;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        long i = base + k;
        if (i < n) out[i] = run;
        run += v[k];
    }
}

__global__ void add_tile_offsets(int *__restrict__ out, int n, const int *__restrict__ offs) {
    const long base = (long)blockIdx.x * SCAN_TILE;
    const int add = offs[blockIdx.x];
    for (int k = threadIdx.x; k < SCAN_TILE; k += blockDim.x) {
        long i = base + k;
        if (i < n) out[i] += add;
    }
}

__global__ void copy_one(const int *src, int *dst) { *dst = *src; }

}  // namespace

int exclusive_scan(const int *in, int *out, int n, int *d_total, Arena &ar, cudaStream_t s) {
    if (n <= 0) {
        if (d_total) TAGI_CUDA(cudaMemsetAsync(d_total, 0, sizeof(int), s));
        return TAGI_OK;
    }
    int nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    int *sums = nullptr;
    TAGI_TRY(ar.alloc(&sums, nb + 1));
    launch(scan_tiles, nb, SCAN_THREADS, 0, s, in, out, n, sums);
    TAGI_LAUNCH_CHECK();
    if (nb == 1) {
        if (d_total) launch(copy_one, 1, 1, 0, s, sums, d_total);
        TAGI_LAUNCH_CHECK();
        return TAGI_OK;
    }
    int *offs = nullptr;
    TAGI_TRY(ar.alloc(&offs, nb));
    TAGI_TRY(exclusive_scan(sums, offs, nb, d_total, ar, s));
    launch(add_tile_offsets, nb, 256, 0, s, out, n, offs);
    TAGI_LAUNCH_CHECK();
    return TAGI_OK;
}

namespace {

constexpr int RS_THREADS = 256;
constexpr int RS_ROUNDS = 8;
constexpr int RS_TILE = RS_THREADS * RS_ROUNDS;
constexpr int RS_WARPS = RS_THREADS / 32;

__global__ void __launch_bounds__(RS_THREADS) rs_histogram(const uint64_t *__restrict__ keys,
                                                           int n, int shift,
                                                           int *__restrict__ hist, int nblocks) {
    __shared__ int cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const long base = (long)blockIdx.x * RS_TILE;
    for (int r = 0; r < RS_ROUNDS; r++) {
        long i = base + (long)r * RS_THREADS + threadIdx.x;
        if (i < n) atomicAdd(&cnt[(int)((keys[i] >> shift) & 255u)], 1);
    }
    __syncthreads();
    hist[(long)threadIdx.x * nblocks + blockIdx.x] = cnt[threadIdx.x];
}

// Stable scatter: elements of a tile are ranked in index order, warp by warp,
// round by round; ties between tiles follow block order via the scanned
// digit-major histogram.
__global__ void __launch_bounds__(RS_THREADS) rs_scatter(const uint64_t *__restrict__ kin,
                                                         const int *__restrict__ vin,
                                                         uint64_t *__restrict__ kout,
                                                         int *__restrict__ vout, int n, int shift,
                                                         const int *__restrict__ offs,
                                                         int nblocks) {
    __shared__ int base[256];
    __shared__ int wcnt[RS_WARPS][256];
    base[threadIdx.x] = offs[(long)threadIdx.x * nblocks + blockIdx.x];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    const long tile = (long)blockIdx.x * RS_TILE;
    for (int r = 0; r < RS_ROUNDS; r++) {
#pragma unroll
        for (int w = 0; w < RS_WARPS; w++) wcnt[w][threadIdx.x] = 0;
        __syncthreads();
        long i = tile + (long)r * RS_THREADS + threadIdx.x;
        bool valid = i < n;
        uint64_t k = valid ? kin[i] : 0;
        int v = valid ? vin[i] : 0;
        int d = valid ? (int)((k >> shift) & 255u) : 256 + lane;  // invalid lanes stay alone
        unsigned peers = __match_any_sync(0xffffffffu, d);
        int rank = __popc(peers & lt);
        if (valid && rank == 0) wcnt[wid][d] = __popc(peers);
        __syncthreads();
        {
            int dd = threadIdx.x;
            int run = base[dd];
#pragma unroll
            for (int w = 0; w < RS_WARPS; w++) {
                int c = wcnt[w][dd];
                wcnt[w][dd] = run;
                run += c;
            }
            base[dd] = run;
        }
        __syncthreads();
        if (valid) {
            int pos = wcnt[wid][d] + rank;
            kout[pos] = k;
            vout[pos] = v;
        }
        __syncthreads();
    }
}

}  // namespace

int radix_sort_u64(uint64_t *keys, int *vals, int n, Arena &ar, cudaStream_t s) {
    if (n <= 1) return TAGI_OK;
    int nb = (n + RS_TILE - 1) / RS_TILE;
    uint64_t *k2 = nullptr;
    int *v2 = nullptr, *hist = nullptr, *offs = nullptr;
    TAGI_TRY(ar.alloc(&k2, n));
    TAGI_TRY(ar.alloc(&v2, n));
    TAGI_TRY(ar.alloc(&hist, 256L * nb));
    TAGI_TRY(ar.alloc(&offs, 256L * nb));
    uint64_t *ka = keys, *kb = k2;
    int *va = vals, *vb = v2;
    for (int shift = 0; shift < 64; shift += 8) {
        launch(rs_histogram, nb, RS_THREADS, 0, s, ka, n, shift, hist, nb);
        TAGI_LAUNCH_CHECK();
        TAGI_TRY(exclusive_scan(hist, offs, 256 * nb, nullptr, ar, s));
        launch(rs_scatter, nb, RS_THREADS, 0, s, ka, va, kb, vb, n, shift, offs, nb);
        TAGI_LAUNCH_CHECK();
        uint64_t *kt = ka; ka = kb; kb = kt;
        int *vt = va; va = vb; vb = vt;
    }
    // 8 passes: the result is back in the caller's buffers.
    return TAGI_OK;
}

}  // namespace tagi
