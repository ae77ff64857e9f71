// Subsystem (a): source tree, target batches and interaction lists, on device.
//
// Rules (project-defined; BaryTree's own rules are not part of the reference,
// see 3D-GreenIteration/src/utilities/BaryTreeInterface.py:52-83):
//  * 63-bit Morton codes on the cubic box of the points' bounding box,
//    21 bits per axis, x above y above z in each 3-bit digit; stable sort.
//  * compressed octree: a node with more than `leaf` points splits at the
//    highest Morton digit in which its first and last codes differ; children
//    are the non-empty runs of that digit (2..8), numbered breadth first.
//  * tight FP64 bounding box per node; radius = half the box diagonal.
//  * batches = target-tree leaves in Morton order.
//  * per batch, pre-order DFS of the source tree:
//      (rB + rC) < theta * |cB - cC|  and  count > sizeCheck * (n+1)^3 -> far
//      (rB + rC) < theta * |cB - cC|  otherwise                       -> near
//      leaf                                                            -> near
//      else children in digit order.
// Every FP64 operation that feeds a decision uses an explicitly rounded
// intrinsic, so the lists equal the CPU oracle's integer for integer.
#include "tagi_internal.h"

#include <algorithm>
#include <numeric>

namespace tagi {

namespace {

__device__ __forceinline__ double dmin(double a, double b) { return a < b ? a : b; }
__device__ __forceinline__ double dmax(double a, double b) { return a > b ? a : b; }

__global__ void bbox_partial(const double *__restrict__ x, const double *__restrict__ y,
                             const double *__restrict__ z, int n, double *__restrict__ part) {
    double l[3] = {x[0], y[0], z[0]}, h[3] = {x[0], y[0], z[0]};
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x) {
        double p[3] = {x[i], y[i], z[i]};
#pragma unroll
        for (int d = 0; d < 3; d++) {
            l[d] = dmin(l[d], p[d]);
            h[d] = dmax(h[d], p[d]);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int d = 0; d < 3; d++) {
            l[d] = dmin(l[d], __shfl_xor_sync(0xffffffffu, l[d], o));
            h[d] = dmax(h[d], __shfl_xor_sync(0xffffffffu, h[d], o));
        }
    __shared__ double sl[32][6];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
        for (int d = 0; d < 3; d++) {
            sl[wid][d] = l[d];
            sl[wid][3 + d] = h[d];
        }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++)
            for (int d = 0; d < 3; d++) {
                sl[0][d] = dmin(sl[0][d], sl[w][d]);
                sl[0][3 + d] = dmax(sl[0][3 + d], sl[w][3 + d]);
            }
        for (int d = 0; d < 6; d++) part[blockIdx.x * 6 + d] = sl[0][d];
    }
}

// params[0..2] = lower corner, params[3] = 2^21 / cube edge.  One block
// reduces the per-block partials (min/max are exact in any order).
__global__ void __launch_bounds__(256) bbox_final(const double *__restrict__ part, int nb,
                                                  double *__restrict__ params) {
    double l[3] = {part[0], part[1], part[2]}, h[3] = {part[3], part[4], part[5]};
    for (int b = threadIdx.x; b < nb; b += blockDim.x)
        for (int d = 0; d < 3; d++) {
            l[d] = dmin(l[d], part[b * 6 + d]);
            h[d] = dmax(h[d], part[b * 6 + 3 + d]);
        }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int d = 0; d < 3; d++) {
            l[d] = dmin(l[d], __shfl_xor_sync(0xffffffffu, l[d], o));
            h[d] = dmax(h[d], __shfl_xor_sync(0xffffffffu, h[d], o));
        }
    __shared__ double sl[8][6];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
        for (int d = 0; d < 3; d++) {
            sl[wid][d] = l[d];
            sl[wid][3 + d] = h[d];
        }
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int w = 1; w < (int)(blockDim.x >> 5); w++)
        for (int d = 0; d < 3; d++) {
            l[d] = dmin(l[d], sl[w][d]);
            h[d] = dmax(h[d], sl[w][3 + d]);
        }
    double ext = __dsub_rn(h[0], l[0]);
    if (__dsub_rn(h[1], l[1]) > ext) ext = __dsub_rn(h[1], l[1]);
    if (__dsub_rn(h[2], l[2]) > ext) ext = __dsub_rn(h[2], l[2]);
    if (!(ext > 0.0)) ext = 1.0;
    params[0] = l[0];
    params[1] = l[1];
    params[2] = l[2];
    params[3] = __ddiv_rn(2097152.0, ext);
}

__device__ __forceinline__ uint64_t spread21(uint32_t v) {
    uint64_t r = 0;
#pragma unroll
    for (int b = 0; b < 21; b++) r |= (uint64_t)((v >> b) & 1u) << (3 * b);
    return r;
}

__device__ __forceinline__ uint32_t quantize(double p, double lo, double scale) {
    double s = __dmul_rn(__dsub_rn(p, lo), scale);
    uint32_t v = __double2uint_rz(s);
    return v > 2097151u ? 2097151u : v;
}

__global__ void morton_codes(const double *__restrict__ x, const double *__restrict__ y,
                             const double *__restrict__ z, int n,
                             const double *__restrict__ params, uint64_t *__restrict__ codes,
                             int *__restrict__ idx) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double sc = params[3];
    uint32_t qx = quantize(x[i], params[0], sc);
    uint32_t qy = quantize(y[i], params[1], sc);
    uint32_t qz = quantize(z[i], params[2], sc);
    codes[i] = (spread21(qx) << 2) | (spread21(qy) << 1) | spread21(qz);
    idx[i] = (int)i;
}

__global__ void gather3(const double *__restrict__ x, const double *__restrict__ y,
                        const double *__restrict__ z, const int *__restrict__ perm, int n,
                        double *__restrict__ xs, double *__restrict__ ys,
                        double *__restrict__ zs) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int o = perm[i];
    xs[i] = x[o];
    ys[i] = y[o];
    zs[i] = z[o];
}

// First index in [lo, hi) whose code >> sh exceeds key (codes are sorted).
__device__ __forceinline__ int run_end(const uint64_t *__restrict__ codes, int lo, int hi,
                                       uint64_t key, int sh) {
    while (lo < hi) {
        int mid = lo + ((hi - lo) >> 1);
        if ((codes[mid] >> sh) > key) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

__device__ __forceinline__ int split_shift(const uint64_t *__restrict__ codes, int b, int e) {
    uint64_t x = codes[b] ^ codes[e - 1];
    if (x == 0) return -1;
    int hb = 63 - __clzll((long long)x);
    return 3 * (hb / 3);
}

__global__ void count_children(const uint64_t *__restrict__ codes, const int *__restrict__ begin,
                               const int *__restrict__ end, int ls, int le, int leaf,
                               int *__restrict__ cc) {
    int v = ls + blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= le) return;
    int b = begin[v], e = end[v];
    int c = 0;
    if (e - b > leaf) {
        int sh = split_shift(codes, b, e);
        if (sh >= 0) {
            int pos = b;
            while (pos < e) {
                pos = run_end(codes, pos, e, codes[pos] >> sh, sh);
                c++;
            }
        }
    }
    cc[v - ls] = c;
}

__global__ void fill_children(const uint64_t *__restrict__ codes, int *__restrict__ begin,
                              int *__restrict__ end, int *__restrict__ parent,
                              int *__restrict__ first_child, int *__restrict__ nchild, int ls,
                              int le, const int *__restrict__ cc, const int *__restrict__ off) {
    int v = ls + blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= le) return;
    int c = cc[v - ls];
    nchild[v] = c;
    if (c == 0) {
        first_child[v] = -1;
        return;
    }
    int first = le + off[v - ls];
    first_child[v] = first;
    int b = begin[v], e = end[v];
    int sh = split_shift(codes, b, e);
    int pos = b, k = 0;
    while (pos < e) {
        int nx = run_end(codes, pos, e, codes[pos] >> sh, sh);
        begin[first + k] = pos;
        end[first + k] = nx;
        parent[first + k] = v;
        pos = nx;
        k++;
    }
}

// One warp per node of a level; children (deeper level) are already done.
__global__ void node_boxes(int ls, int le, const int *__restrict__ begin,
                           const int *__restrict__ end, const int *__restrict__ first_child,
                           const int *__restrict__ nchild, const double *__restrict__ x,
                           const double *__restrict__ y, const double *__restrict__ z,
                           double *__restrict__ box, double *__restrict__ center,
                           double *__restrict__ half, double *__restrict__ radius) {
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    int v = ls + warp;
    if (v >= le) return;
    double l[3] = {INFINITY, INFINITY, INFINITY}, h[3] = {-INFINITY, -INFINITY, -INFINITY};
    int nc = nchild[v];
    if (nc == 0) {
        for (int i = begin[v] + lane; i < end[v]; i += 32) {
            double p[3] = {x[i], y[i], z[i]};
#pragma unroll
            for (int d = 0; d < 3; d++) {
                l[d] = dmin(l[d], p[d]);
                h[d] = dmax(h[d], p[d]);
            }
        }
    } else if (lane < nc) {
        const double *cb = box + 6L * (first_child[v] + lane);
#pragma unroll
        for (int d = 0; d < 3; d++) {
            l[d] = cb[d];
            h[d] = cb[3 + d];
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int d = 0; d < 3; d++) {
            l[d] = dmin(l[d], __shfl_xor_sync(0xffffffffu, l[d], o));
            h[d] = dmax(h[d], __shfl_xor_sync(0xffffffffu, h[d], o));
        }
    if (lane == 0) {
        double hh[3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
            box[6L * v + d] = l[d];
            box[6L * v + 3 + d] = h[d];
            center[3L * v + d] = __dmul_rn(__dadd_rn(l[d], h[d]), 0.5);
            hh[d] = __dmul_rn(__dsub_rn(h[d], l[d]), 0.5);
            half[3L * v + d] = hh[d];
        }
        double s = __dmul_rn(hh[0], hh[0]);
        s = __dadd_rn(s, __dmul_rn(hh[1], hh[1]));
        s = __dadd_rn(s, __dmul_rn(hh[2], hh[2]));
        radius[v] = __dsqrt_rn(s);
    }
}

__global__ void init_root(int *begin, int *end, int *parent, int n) {
    begin[0] = 0;
    end[0] = n;
    parent[0] = -1;
}

}  // namespace

int build_tree(Tree &t, const double *x, const double *y, const double *z, int n, int leaf,
               Arena &ar, int *err_flag, cudaStream_t s) {
    (void)err_flag;
    t.n = n;
    Arena tmp;
    tmp.stream = s;
    int rc = TAGI_OK;
    do {
        const int nbb = std::min(1024, (n + 255) / 256);
        double *part = nullptr, *params = nullptr;
        if ((rc = tmp.alloc(&part, 6L * nbb))) break;
        if ((rc = tmp.alloc(&params, 4))) break;
        launch(bbox_partial, nbb, 256, 0, s, x, y, z, n, part);
        launch(bbox_final, 1, 256, 0, s, part, nbb, params);
        if ((rc = ar.alloc(&t.codes, n))) break;
        if ((rc = ar.alloc(&t.perm, n))) break;
        launch(morton_codes, (n + 255) / 256, 256, 0, s, x, y, z, n, params, t.codes, t.perm);
        if (cudaGetLastError() != cudaSuccess) { rc = set_error(TAGI_ERR_CUDA, "morton launch"); break; }
        if ((rc = radix_sort_u64(t.codes, t.perm, n, tmp, s))) break;
        if ((rc = ar.alloc(&t.x, n)) || (rc = ar.alloc(&t.y, n)) || (rc = ar.alloc(&t.z, n))) break;
        launch(gather3, (n + 255) / 256, 256, 0, s, x, y, z, t.perm, n, t.x, t.y, t.z);

        const long cap = 2L * n + 1;
        if ((rc = ar.alloc(&t.begin, cap)) || (rc = ar.alloc(&t.end, cap)) ||
            (rc = ar.alloc(&t.parent, cap)) || (rc = ar.alloc(&t.first_child, cap)) ||
            (rc = ar.alloc(&t.nchild, cap)))
            break;
        int *cc = nullptr, *off = nullptr, *total = nullptr;
        if ((rc = tmp.alloc(&cc, cap)) || (rc = tmp.alloc(&off, cap)) || (rc = tmp.alloc(&total, 1)))
            break;
        launch(init_root, 1, 1, 0, s, t.begin, t.end, t.parent, n);
        t.level_start.assign(1, 0);
        int ls = 0, le = 1;
        while (ls < le) {
            int m = le - ls;
            launch(count_children, (m + 127) / 128, 128, 0, s, t.codes, t.begin, t.end, ls, le, leaf, cc);
            if ((rc = exclusive_scan(cc, off, m, total, tmp, s))) break;
            launch(fill_children, (m + 127) / 128, 128, 0, s, t.codes, t.begin, t.end, t.parent,
                                                          t.first_child, t.nchild, ls, le, cc, off);
            int h_total = 0;
            if (cudaMemcpyAsync(&h_total, total, sizeof(int), cudaMemcpyDeviceToHost, s) !=
                    cudaSuccess ||
                cudaStreamSynchronize(s) != cudaSuccess) {
                rc = set_error(TAGI_ERR_CUDA, "tree level build: %s",
                               cudaGetErrorString(cudaGetLastError()));
                break;
            }
            if (le + (long)h_total > cap) { rc = set_error(TAGI_ERR_DEVICE, "tree node capacity exceeded"); break; }
            ls = le;
            le += h_total;
            t.level_start.push_back(ls);
        }
        if (rc) break;
        t.nnodes = le;
        t.nlevels = (int)t.level_start.size() - 1;
        double *box = nullptr;
        if ((rc = tmp.alloc(&box, 6L * t.nnodes))) break;
        if ((rc = ar.alloc(&t.center, 3L * t.nnodes)) || (rc = ar.alloc(&t.half, 3L * t.nnodes)) ||
            (rc = ar.alloc(&t.radius, t.nnodes)))
            break;
        for (int lv = t.nlevels - 1; lv >= 0; lv--) {
            int a = t.level_start[lv], b = t.level_start[lv + 1];
            int warps = b - a;
            launch(node_boxes, (warps * 32 + 255) / 256, 256, 0, s, a, b, t.begin, t.end, t.first_child,
                                                                t.nchild, t.x, t.y, t.z, box,
                                                                t.center, t.half, t.radius);
        }
        if (cudaGetLastError() != cudaSuccess) { rc = set_error(TAGI_ERR_CUDA, "node box launch"); break; }
    } while (0);
    tmp.release();
    return rc;
}

// ---------------------------------------------------------------------------
// Batches, lists, slots, upward-pass items.
// ---------------------------------------------------------------------------
namespace {

__global__ void mark_leaves(int nn, const int *__restrict__ nchild, const int *__restrict__ begin,
                            int *__restrict__ mark) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < nn && nchild[v] == 0) mark[begin[v]] = v + 1;
}

__global__ void nonzero_flags(const int *__restrict__ a, int n, int *__restrict__ f) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) f[i] = a[i] != 0;
}

__global__ void compact_leaves(const int *__restrict__ mark, const int *__restrict__ idx, int n,
                               int *__restrict__ batch_node) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && mark[i]) batch_node[idx[i]] = mark[i] - 1;
}

struct TravArgs {
    int nbatch;
    const int *batch_node;
    const double *tc, *tr;                 // target centers / radii
    const double *sc, *sr;                 // source centers / radii
    const int *sbegin, *send, *snchild, *sfirst;
    double theta, thresh;
    int *near_cnt, *far_cnt;
    const int *near_off, *far_off;
    int *near_list, *far_list;
    int *node_flag;
    int *err;
};

template <bool FILL>
__global__ void traverse(TravArgs a) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= a.nbatch) return;
    int bn = a.batch_node[b];
    const double cbx = a.tc[3L * bn], cby = a.tc[3L * bn + 1], cbz = a.tc[3L * bn + 2];
    const double rb = a.tr[bn];
    int stack[TRAVERSAL_STACK];
    int sp = 0;
    stack[sp++] = 0;
    int cn = 0, cf = 0;
    int *nl = FILL ? a.near_list + a.near_off[b] : nullptr;
    int *fl = FILL ? a.far_list + a.far_off[b] : nullptr;
    while (sp > 0) {
        int c = stack[--sp];
        double dx = __dsub_rn(cbx, a.sc[3L * c]);
        double dy = __dsub_rn(cby, a.sc[3L * c + 1]);
        double dz = __dsub_rn(cbz, a.sc[3L * c + 2]);
        double d2 = __dmul_rn(dx, dx);
        d2 = __dadd_rn(d2, __dmul_rn(dy, dy));
        d2 = __dadd_rn(d2, __dmul_rn(dz, dz));
        double dist = __dsqrt_rn(d2);
        bool mac = __dadd_rn(rb, a.sr[c]) < __dmul_rn(a.theta, dist);
        int nc = a.snchild[c];
        if (mac) {
            if ((double)(a.send[c] - a.sbegin[c]) > a.thresh) {
                if (FILL) {
                    fl[cf] = c;
                    a.node_flag[c] = 1;
                }
                cf++;
            } else {
                if (FILL) nl[cn] = c;
                cn++;
            }
        } else if (nc == 0) {
            if (FILL) nl[cn] = c;
            cn++;
        } else {
            if (sp + nc > TRAVERSAL_STACK) {
                atomicOr(a.err, 1);
                break;
            }
            int f = a.sfirst[c];
            for (int k = nc - 1; k >= 0; k--) stack[sp++] = f + k;
        }
    }
    if (!FILL) {
        a.near_cnt[b] = cn;
        a.far_cnt[b] = cf;
    }
}

__global__ void assign_slots(int nn, const int *__restrict__ flag, const int *__restrict__ idx,
                             int *__restrict__ node_slot, int *__restrict__ slot_node) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nn) return;
    if (flag[v]) {
        node_slot[v] = idx[v];
        slot_node[idx[v]] = v;
    } else {
        node_slot[v] = -1;
    }
}

// Gap between the batch box (center cb, half widths hb) and a node box: the
// Euclidean distance between the closed boxes, reduced by a relative margin so
// that touching boxes give 0.
__device__ __forceinline__ double box_gap(const double *cb, const double *hb, const double *cc,
                                          const double *hc) {
    double g2 = 0.0;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        double gap = fabs(cb[d] - cc[d]) - (hb[d] + hc[d]);
        gap -= 1e-12 * (fabs(cb[d]) + fabs(cc[d]) + hb[d] + hc[d]) + 1e-300;
        if (gap > 0.0) g2 += gap * gap;
    }
    return sqrt(g2);
}

// Merge consecutive near entries whose source ranges touch and whose nodes
// are of the same class: a node is CLOSE when its box lies within
// CLOSE_RANGE_FRACTION batch radii of the batch's box (touching included).
// Close ranges are stored with bit 31 of their begin set (range_is_close).
// rng_dmin = smallest node gap of the range, rounded down: a lower bound of
// every pair distance in it.
template <bool FILL>
__global__ void merge_ranges(int nbatch, const int *__restrict__ near_off,
                             const int *__restrict__ near_list, const int *__restrict__ sbegin,
                             const int *__restrict__ send, const double *__restrict__ scenter,
                             const double *__restrict__ shalf, const int *__restrict__ batch_node,
                             const double *__restrict__ tcenter, const double *__restrict__ thalf,
                             const double *__restrict__ tradius,
                             int *__restrict__ cnt, const int *__restrict__ rng_off,
                             int2 *__restrict__ rng, float *__restrict__ rng_dmin) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbatch) return;
    const int bn = batch_node[b];
    const double cb[3] = {tcenter[3L * bn], tcenter[3L * bn + 1], tcenter[3L * bn + 2]};
    const double hb[3] = {thalf[3L * bn], thalf[3L * bn + 1], thalf[3L * bn + 2]};
    const double close_gap = CLOSE_RANGE_FRACTION * tradius[bn];
    int k = 0;
    int cb0 = -1, ce = -1;
    bool cclose = false;
    double cmin = INFINITY;
    for (int e = near_off[b]; e <= near_off[b + 1]; e++) {
        int c = -1, nb = -1, ne = -1;
        bool nclose = false;
        double gap = 0.0;
        if (e < near_off[b + 1]) {
            c = near_list[e];
            nb = sbegin[c];
            ne = send[c];
            const double cc[3] = {scenter[3L * c], scenter[3L * c + 1], scenter[3L * c + 2]};
            const double hc[3] = {shalf[3L * c], shalf[3L * c + 1], shalf[3L * c + 2]};
            gap = box_gap(cb, hb, cc, hc);
            nclose = gap <= close_gap;
        }
        if (c >= 0 && cb0 >= 0 && nb == ce && nclose == cclose) {
            ce = ne;
            cmin = fmin(cmin, gap);
            continue;
        }
        if (cb0 >= 0) {
            if (FILL) {
                rng[rng_off[b] + k] = make_int2(cb0 | (cclose ? (int)0x80000000u : 0), ce);
                rng_dmin[rng_off[b] + k] = (float)(cmin * (1.0 - 1e-6));
            }
            k++;
        }
        if (c < 0) break;
        cb0 = nb;
        ce = ne;
        cclose = nclose;
        cmin = gap;
    }
    if (!FILL) cnt[b] = k;
}

__global__ void batch_costs(int nbatch, const int *__restrict__ batch_node,
                            const int *__restrict__ tbegin, const int *__restrict__ tend,
                            const int *__restrict__ rng_off, const int2 *__restrict__ rng,
                            const int *__restrict__ far_off, long long *__restrict__ cost_near,
                            long long *__restrict__ cost_far, int *__restrict__ bsize,
                            long long *__restrict__ cost_close) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbatch) return;
    int bn = batch_node[b];
    long long nb = tend[bn] - tbegin[bn];
    long long s = 0, sc = 0;
    for (int e = rng_off[b]; e < rng_off[b + 1]; e++) {
        const long long len = rng[e].y - range_begin(rng[e]);
        s += len;
        if (range_is_close(rng[e])) sc += len;
    }
    cost_near[b] = nb * s;
    cost_close[b] = nb * sc;
    cost_far[b] = nb * (long long)(far_off[b + 1] - far_off[b]);
    bsize[b] = (int)nb;
}

__global__ void slot_chunks(int nslots, const int *__restrict__ slot_node,
                            const int *__restrict__ sbegin, const int *__restrict__ send,
                            int chunk, int *__restrict__ nch) {
    int sl = blockIdx.x * blockDim.x + threadIdx.x;
    if (sl >= nslots) return;
    int c = slot_node[sl];
    int cnt = send[c] - sbegin[c];
    nch[sl] = (cnt + chunk - 1) / chunk;
}

__global__ void fill_items(int nslots, const int *__restrict__ slot_node,
                           const int *__restrict__ sbegin, const int *__restrict__ send,
                           int chunk, const int *__restrict__ off, int *__restrict__ item_slot,
                           int *__restrict__ item_begin, int *__restrict__ item_end) {
    int sl = blockIdx.x * blockDim.x + threadIdx.x;
    if (sl >= nslots) return;
    int c = slot_node[sl];
    int b = sbegin[c], e = send[c];
    int k = off[sl];
    for (int p = b; p < e; p += chunk, k++) {
        item_slot[k] = sl;
        item_begin[k] = p;
        item_end[k] = min(p + chunk, e);
    }
}

// Proxy box of each slot: node center and half widths; a zero width gets a
// small one (1e-3 of the largest, or 1) so the barycentric map stays finite.
__global__ void slot_geometry(int nslots, const int *__restrict__ slot_node,
                              const double *__restrict__ center, const double *__restrict__ half,
                              double *__restrict__ geom) {
    int sl = blockIdx.x * blockDim.x + threadIdx.x;
    if (sl >= nslots) return;
    int c = slot_node[sl];
    double h[3] = {half[3L * c], half[3L * c + 1], half[3L * c + 2]};
    double hm = dmax(dmax(h[0], h[1]), h[2]);
#pragma unroll
    for (int d = 0; d < 3; d++) {
        geom[6L * sl + d] = center[3L * c + d];
        double v = h[d];
        if (!(v > 0.0)) v = hm > 0.0 ? hm * 1.0e-3 : 1.0;
        geom[6L * sl + 3 + d] = v;
    }
}

constexpr int P2M_CHUNK = 2048;

}  // namespace

int build_lists(Plan &p, cudaStream_t s) {
    Arena tmp;
    tmp.stream = s;
    Arena &ar = p.arena;
    int rc = TAGI_OK;
    auto sync_int = [&](const int *d, int *h) -> int {
        if (cudaMemcpyAsync(h, d, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return set_error(TAGI_ERR_CUDA, "list build sync: %s",
                             cudaGetErrorString(cudaGetLastError()));
        return TAGI_OK;
    };
    do {
        const int nt = p.tgt.n, nns = p.src.nnodes, nnt = p.tgt.nnodes;
        int *mark = nullptr, *flags = nullptr, *idx = nullptr, *total = nullptr;
        if ((rc = tmp.alloc(&mark, nt)) || (rc = tmp.alloc(&flags, nt)) ||
            (rc = tmp.alloc(&idx, nt)) || (rc = tmp.alloc(&total, 1)))
            break;
        cudaMemsetAsync(mark, 0, sizeof(int) * nt, s);
        launch(mark_leaves, (nnt + 255) / 256, 256, 0, s, nnt, p.tgt.nchild, p.tgt.begin, mark);
        launch(nonzero_flags, (nt + 255) / 256, 256, 0, s, mark, nt, flags);
        if ((rc = exclusive_scan(flags, idx, nt, total, tmp, s))) break;
        if ((rc = sync_int(total, &p.nbatch))) break;
        if ((rc = ar.alloc(&p.batch_node, p.nbatch))) break;
        launch(compact_leaves, (nt + 255) / 256, 256, 0, s, mark, idx, nt, p.batch_node);

        const int nb = p.nbatch;
        int *ncnt = nullptr, *fcnt = nullptr;
        if ((rc = tmp.alloc(&ncnt, nb)) || (rc = tmp.alloc(&fcnt, nb))) break;
        if ((rc = ar.alloc(&p.near_off, nb + 1)) || (rc = ar.alloc(&p.far_off, nb + 1))) break;
        int *node_flag = nullptr;
        if ((rc = tmp.alloc(&node_flag, nns))) break;
        cudaMemsetAsync(node_flag, 0, sizeof(int) * nns, s);
        TravArgs ta;
        ta.nbatch = nb;
        ta.batch_node = p.batch_node;
        ta.tc = p.tgt.center;
        ta.tr = p.tgt.radius;
        ta.sc = p.src.center;
        ta.sr = p.src.radius;
        ta.sbegin = p.src.begin;
        ta.send = p.src.end;
        ta.snchild = p.src.nchild;
        ta.sfirst = p.src.first_child;
        ta.theta = p.theta;
        ta.thresh = p.size_check * (double)p.P;
        ta.near_cnt = ncnt;
        ta.far_cnt = fcnt;
        ta.near_off = p.near_off;
        ta.far_off = p.far_off;
        ta.near_list = nullptr;
        ta.far_list = nullptr;
        ta.node_flag = node_flag;
        ta.err = p.err_flag;
        launch(traverse<false>, (nb + 63) / 64, 64, 0, s, ta);
        if ((rc = exclusive_scan(ncnt, p.near_off, nb, p.near_off + nb, tmp, s))) break;
        if ((rc = exclusive_scan(fcnt, p.far_off, nb, p.far_off + nb, tmp, s))) break;
        if ((rc = sync_int(p.near_off + nb, &p.near_total))) break;
        if ((rc = sync_int(p.far_off + nb, &p.far_total))) break;
        if ((rc = ar.alloc(&p.near_list, p.near_total)) || (rc = ar.alloc(&p.far_list, p.far_total)))
            break;
        ta.near_list = p.near_list;
        ta.far_list = p.far_list;
        launch(traverse<true>, (nb + 63) / 64, 64, 0, s, ta);
        int h_err = 0;
        if ((rc = sync_int(p.err_flag, &h_err))) break;
        if (h_err) { rc = set_error(TAGI_ERR_DEVICE, "source tree deeper than the traversal stack"); break; }

        // Slots (far nodes, ascending node index).
        int *sidx = nullptr;
        if ((rc = tmp.alloc(&sidx, nns))) break;
        if ((rc = exclusive_scan(node_flag, sidx, nns, total, tmp, s))) break;
        if ((rc = sync_int(total, &p.nslots))) break;
        if ((rc = ar.alloc(&p.node_slot, nns)) || (rc = ar.alloc(&p.slot_node, p.nslots))) break;
        launch(assign_slots, (nns + 255) / 256, 256, 0, s, nns, node_flag, sidx, p.node_slot, p.slot_node);
        if ((rc = ar.alloc(&p.slot_geom, 6L * p.nslots))) break;
        if (p.nslots)
            launch(slot_geometry, (p.nslots + 127) / 128, 128, 0, s, p.nslots, p.slot_node, p.src.center,
                                                                 p.src.half, p.slot_geom);

        // Merged near ranges.
        int *rcnt = nullptr;
        if ((rc = tmp.alloc(&rcnt, nb))) break;
        if ((rc = ar.alloc(&p.rng_off, nb + 1))) break;
        launch(merge_ranges<false>, (nb + 127) / 128, 128, 0, s, nb, p.near_off, p.near_list, p.src.begin,
               p.src.end, p.src.center, p.src.half, p.batch_node, p.tgt.center, p.tgt.half, p.tgt.radius, rcnt,
               nullptr, nullptr, nullptr);
        if ((rc = exclusive_scan(rcnt, p.rng_off, nb, p.rng_off + nb, tmp, s))) break;
        if ((rc = sync_int(p.rng_off + nb, &p.rng_total))) break;
        if ((rc = ar.alloc(&p.rng, p.rng_total)) || (rc = ar.alloc(&p.rng_dmin, p.rng_total))) break;
        launch(merge_ranges<true>, (nb + 127) / 128, 128, 0, s, nb, p.near_off, p.near_list, p.src.begin,
               p.src.end, p.src.center, p.src.half, p.batch_node, p.tgt.center, p.tgt.half, p.tgt.radius, nullptr,
               p.rng_off, p.rng, p.rng_dmin);

        // Upward-pass work items.
        if ((rc = ar.alloc(&p.slot_item_off, p.nslots + 1))) break;
        if (p.nslots) {
            int *nch = nullptr;
            if ((rc = tmp.alloc(&nch, p.nslots))) break;
            launch(slot_chunks, (p.nslots + 127) / 128, 128, 0, s, p.nslots, p.slot_node, p.src.begin,
                                                               p.src.end, P2M_CHUNK, nch);
            if ((rc = exclusive_scan(nch, p.slot_item_off, p.nslots, p.slot_item_off + p.nslots, tmp, s)))
                break;
            if ((rc = sync_int(p.slot_item_off + p.nslots, &p.nitems))) break;
        } else {
            cudaMemsetAsync(p.slot_item_off, 0, sizeof(int), s);
            p.nitems = 0;
        }
        if ((rc = ar.alloc(&p.item_slot, p.nitems)) || (rc = ar.alloc(&p.item_begin, p.nitems)) ||
            (rc = ar.alloc(&p.item_end, p.nitems)))
            break;
        if (p.nslots)
            launch(fill_items, (p.nslots + 127) / 128, 128, 0, s, p.nslots, p.slot_node, p.src.begin,
                                                              p.src.end, P2M_CHUNK, p.slot_item_off,
                                                              p.item_slot, p.item_begin, p.item_end);

        // Per-batch pair counts: the field kernels' work lists go heaviest first.
        long long *cn = nullptr, *cf = nullptr, *cc2 = nullptr;
        int *bsz = nullptr;
        if ((rc = tmp.alloc(&cn, nb)) || (rc = tmp.alloc(&cf, nb)) || (rc = tmp.alloc(&bsz, nb)) ||
            (rc = tmp.alloc(&cc2, nb)))
            break;
        launch(batch_costs, (nb + 127) / 128, 128, 0, s, nb, p.batch_node, p.tgt.begin, p.tgt.end,
                                                     p.rng_off, p.rng, p.far_off, cn, cf, bsz, cc2);
        std::vector<long long> hcn(nb), hcf(nb), hcc(nb);
        std::vector<int> hsz(nb);
        if (cudaMemcpyAsync(hcn.data(), cn, sizeof(long long) * nb, cudaMemcpyDeviceToHost, s) ||
            cudaMemcpyAsync(hcf.data(), cf, sizeof(long long) * nb, cudaMemcpyDeviceToHost, s) ||
            cudaMemcpyAsync(hsz.data(), bsz, sizeof(int) * nb, cudaMemcpyDeviceToHost, s) ||
            cudaMemcpyAsync(hcc.data(), cc2, sizeof(long long) * nb, cudaMemcpyDeviceToHost, s) ||
            cudaStreamSynchronize(s)) {
            rc = set_error(TAGI_ERR_CUDA, "batch cost copy failed");
            break;
        }
        p.near_pairs = 0;
        p.near_close_pairs = 0;
        p.far_pairs = 0;
        p.max_batch = 0;
        p.cost_near.resize(nb);
        p.cost_close.resize(nb);
        p.cost_far.resize(nb);
        for (int b = 0; b < nb; b++) {
            p.near_pairs += (double)hcn[b];
            p.near_close_pairs += (double)hcc[b];
            p.far_pairs += (double)hcf[b] * p.P;
            p.max_batch = std::max(p.max_batch, hsz[b]);
            p.cost_near[b] = hcn[b] - hcc[b];
            p.cost_close[b] = hcc[b];
            p.cost_far[b] = hcf[b] * (long long)p.P;
        }
        if (cudaGetLastError() != cudaSuccess) { rc = set_error(TAGI_ERR_CUDA, "list kernels failed"); break; }
    } while (0);
    tmp.release();
    return rc;
}

}  // namespace tagi
