// Device mesh generation: the reference's cell refinement for the
// "coarsenedUniformTwoLevel" divide criterion and the first-kind Chebyshev
// quadrature meshes built on the resulting cells (coarse and two-level fine).
//
// Follows, in 3D-GreenIteration/src:
//   divide rule     dataStructures/CellStruct_CC.py:2344-2439
//                   (refineCoarseningUniform_TwoLevel)
//   recursion       dataStructures/TreeStruct_CC.py:1049-1131 (recursiveDivide:
//                   level < minDepth divides; midpoint split,
//                   CellStruct_CC.py:3060-3100)
//   cell order      depth first, children x-major (the uniqueID order of the
//                   tree's masterList, CellStruct_CC.py:220-221,
//                   TreeStruct_CC.py:2387), base cells in their given order
//   cell table      TreeStruct_CC.py:2390-2406 (centre, width, points per cell)
//   coarse points   utilities/mpiMeshBuilding.py:725-752
//   fine points     utilities/mpiMeshBuilding.py:755-840
//
// GPU layout.  Refinement is level-synchronous: one thread per cell of the
// current level decides divide / leaf; an exclusive scan of the divide flags
// places the 8 children of each dividing cell in the next level and each leaf
// in this level's leaf list.  Every cell carries a 64-bit path key (base cell
// index in bits 48-63, then 3 bits per level, child digit 4i+2j+k), so one
// radix sort of the leaf keys gives the depth-first order.  Point generation
// is one thread per output point (32 bytes written: x, y, z, w); fine points
// find their cell by binary search over the per-cell offsets.  All arithmetic
// is FP64 with explicit round-to-nearest intrinsics in the order the
// reference's numpy expressions evaluate, so the cells and points are
// bit-identical to the reference's on the same 1-D node and weight tables.
#include "tagi_internal.h"

#include <cmath>

namespace tagi {
namespace {

constexpr int MESH_MAX_DEPTH = 16;          // 3 bits per level below bit 48
constexpr int MESH_MAX_BASE = 1 << 16;      // base cell index in bits 48..63
constexpr long MESH_MAX_CELLS = 1L << 24;   // cells per level / leaves in total
constexpr int MESH_MAX_P1 = 16;             // order <= 15
constexpr int MT = 256;

struct Rule {
    double h, H, r;
    int ge2, ge1, fine;  // level >= 2, level >= 1, level < -1
    int nsub;            // -int(level): fine children per side
    int min_depth, max_depth;
};

struct Tables {
    double u[MESH_MAX_P1];  // first-kind nodes cos(theta_i) on [-1, 1], ascending
    double w[MESH_MAX_P1];  // unscaled first-kind weights
};

__device__ __forceinline__ double half_of(double a) { return __dmul_rn(a, 0.5); }

// divide flag and fine children of one cell (CellStruct_CC.py:2344-2439).
__global__ void __launch_bounds__(MT) mesh_classify(const double *__restrict__ cells, int n, int depth,
                                                    const double *__restrict__ atoms, int natoms,
                                                    Rule p, int *__restrict__ divide,
                                                    int *__restrict__ fine, int *__restrict__ err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *c = cells + 6L * i;
    const double xmin = c[0], xmax = c[1], ymin = c[2], ymax = c[3], zmin = c[4], zmax = c[5];
    int div = 0, nf = 1;
    if (depth < p.min_depth) {
        div = 1;
    } else {
        double dist = __dadd_rn(10.0, p.H);
        for (int a = 0; a < natoms; a++) {
            const double ax = atoms[3 * a], ay = atoms[3 * a + 1], az = atoms[3 * a + 2];
            if (ax < xmax && ay < ymax && az < zmax && ax > xmin && ay > ymin && az > zmin) {
                dist = 0.0;
            } else {
#pragma unroll
                for (int q = 0; q < 8; q++) {
                    const double dx = __dsub_rn((q & 4) ? xmin : xmax, ax);
                    const double dy = __dsub_rn((q & 2) ? ymax : ymin, ay);
                    const double dz = __dsub_rn((q & 1) ? zmax : zmin, az);
                    const double d = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)),
                                                          __dmul_rn(dz, dz)));
                    if (d < dist) dist = d;
                }
            }
        }
        const double sz = __dsub_rn(zmax, zmin), sx = __dsub_rn(xmax, xmin), sy = __dsub_rn(ymax, ymin);
        double side = sz;
        if (sx > side) side = sx;
        if (sy > side) side = sy;
        const double h = p.h, r = p.r;
        const double h2 = __dmul_rn(2.0, h), h4 = __dmul_rn(4.0, h), h8 = __dmul_rn(8.0, h);
        const double a1 = __dadd_rn(r, __dmul_rn(h2, 1.0));
        const double a2 = __dadd_rn(r, __dmul_rn(__dadd_rn(h2, h4), 1.0));
        const double a3 = __dadd_rn(r, __dmul_rn(__dadd_rn(__dadd_rn(h2, h4), h8), 1.0));
        if (side > p.H)
            div = 1;
        else if (p.ge2 && dist < __ddiv_rn(r, 4.0))
            div = side > __ddiv_rn(h, 4.0);
        else if (p.ge1 && dist < __ddiv_rn(r, 2.0))
            div = side > __ddiv_rn(h, 2.0);
        else if (dist < r)
            div = side > h;
        else if (dist < a1)
            div = side > h2;
        else if (dist < a2)
            div = side > h4;
        else if (dist < a3)
            div = side > h8;
        if (!div && p.fine && dist < __dmul_rn(r, 1.5)) nf = p.nsub * p.nsub * p.nsub;
    }
    if (div && depth >= p.max_depth) {
        atomicOr(err, 1);
        div = 0;
    }
    divide[i] = div;
    fine[i] = nf;
}

// Children of dividing cells into the next level; leaves into this level's
// leaf list.  rank = exclusive scan of divide.
__global__ void __launch_bounds__(MT) mesh_emit(const double *__restrict__ cells,
                                                const uint64_t *__restrict__ keys, int n, int depth,
                                                const int *__restrict__ divide,
                                                const int *__restrict__ fine,
                                                const int *__restrict__ rank,
                                                double *__restrict__ next_cells,
                                                uint64_t *__restrict__ next_keys,
                                                double *__restrict__ leaf_cells,
                                                uint64_t *__restrict__ leaf_keys,
                                                int *__restrict__ leaf_fine) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *c = cells + 6L * i;
    const uint64_t key = keys[i];
    const int rk = rank[i];
    if (divide[i]) {
        // xdiv = (xmax + xmin)/2 (TreeStruct_CC.py:1129-1131)
        const double xb[3] = {c[0], half_of(__dadd_rn(c[1], c[0])), c[1]};
        const double yb[3] = {c[2], half_of(__dadd_rn(c[3], c[2])), c[3]};
        const double zb[3] = {c[4], half_of(__dadd_rn(c[5], c[4])), c[5]};
        const int shift = 3 * (MESH_MAX_DEPTH - 1 - depth);
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const int ii = q >> 2, jj = (q >> 1) & 1, kk = q & 1;
            double *o = next_cells + 6L * (8L * rk + q);
            o[0] = xb[ii];
            o[1] = xb[ii + 1];
            o[2] = yb[jj];
            o[3] = yb[jj + 1];
            o[4] = zb[kk];
            o[5] = zb[kk + 1];
            next_keys[8L * rk + q] = key | ((uint64_t)q << shift);
        }
    } else {
        const long l = (long)i - rk;
        double *o = leaf_cells + 6L * l;
#pragma unroll
        for (int k = 0; k < 6; k++) o[k] = c[k];
        leaf_keys[l] = key;
        leaf_fine[l] = fine[i];
    }
}

__global__ void mesh_base_keys(uint64_t *__restrict__ keys, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) keys[i] = (uint64_t)i << 48;
}

__global__ void mesh_iota(int *__restrict__ v, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = i;
}

// Leaves in key order -> the reference's cell table (TreeStruct_CC.py:2390-2406).
__global__ void __launch_bounds__(MT) mesh_cell_table(const int *__restrict__ order_idx, int n,
                                                      const double *__restrict__ leaf_cells,
                                                      const int *__restrict__ leaf_fine, int p3,
                                                      double *__restrict__ cx, double *__restrict__ cy,
                                                      double *__restrict__ cz, double *__restrict__ dx,
                                                      double *__restrict__ dy, double *__restrict__ dz,
                                                      int *__restrict__ ppc_c,
                                                      int *__restrict__ ppc_f) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int s = order_idx[i];
    const double *c = leaf_cells + 6L * s;
    cx[i] = half_of(__dadd_rn(c[0], c[1]));
    cy[i] = half_of(__dadd_rn(c[2], c[3]));
    cz[i] = half_of(__dadd_rn(c[4], c[5]));
    dx[i] = __dsub_rn(c[1], c[0]);
    dy[i] = __dsub_rn(c[3], c[2]);
    dz[i] = __dsub_rn(c[5], c[4]);
    if (ppc_c) ppc_c[i] = p3;
    if (ppc_f) ppc_f[i] = leaf_fine[s] * p3;
}

// x/2 and x/4 are written as products with 0.5 and 0.25: the same correctly
// rounded value as the reference's divisions, without a division sequence.

// One cell's bounds from centre and width: xl = cx - dx/2, xh = cx + dx/2
// (mpiMeshBuilding.py:519-527).
__device__ __forceinline__ void cell_bounds(const double *cx, const double *cy, const double *cz,
                                            const double *dx, const double *dy, const double *dz,
                                            long c, double lo[3], double hi[3]) {
    const double ctr[3] = {cx[c], cy[c], cz[c]};
    const double wid[3] = {dx[c], dy[c], dz[c]};
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const double hw = __dmul_rn(wid[d], 0.5);
        lo[d] = __dsub_rn(ctr[d], hw);
        hi[d] = __dadd_rn(ctr[d], hw);
    }
}

// Interior split points of [lo, hi] into m equal parts, as
// fineQuadraturePointsSingleCell writes them (mpiMeshBuilding.py:766-800).
__device__ __forceinline__ double split_point(double lo, double hi, int m, int s) {
    if (s == 0) return lo;
    if (s == m) return hi;
    if (m == 2) return __dmul_rn(__dadd_rn(lo, hi), 0.5);
    if (m == 3)
        return s == 1 ? __ddiv_rn(__dadd_rn(__dmul_rn(2.0, lo), hi), 3.0)
                      : __ddiv_rn(__dadd_rn(__dmul_rn(2.0, hi), lo), 3.0);
    // m == 4
    if (s == 2) return __dmul_rn(__dadd_rn(lo, hi), 0.5);
    return s == 1 ? __dmul_rn(__dadd_rn(__dmul_rn(3.0, lo), hi), 0.25)
                  : __dmul_rn(__dadd_rn(__dmul_rn(3.0, hi), lo), 0.25);
}

// m (children per side) and m^3 per cell from the fine point counts.
__global__ void mesh_fine_counts(const int *__restrict__ ppc_f, int n, int p3, int *__restrict__ sub,
                                 int *__restrict__ nsub, int *__restrict__ err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int v = ppc_f[i];
    int m = 0;
    if (v == p3) m = 1;
    else if (v == 8 * p3) m = 2;
    else if (v == 27 * p3) m = 3;
    else if (v == 64 * p3) m = 4;
    if (!m) atomicOr(err, 2);
    sub[i] = m;
    nsub[i] = m * m * m;
}

constexpr int PW = 8;  // warps per CTA in mesh_points_warp

// One warp per sub-cell: a coarse cell (sub_off == nullptr), or child
// (ii, jj, kk) of a fine cell.  Every sub-cell holds (order+1)^3 points, so
// sub-cell s writes points [s p3, (s+1) p3).  Lanes < order+1 evaluate the
// 1-D nodes x = lo + (hi-lo)/2 (u+1) and scaled weights (hi-lo)/2 W of each
// axis once (meshUtilities.py:857-883), then the (order+1)^2 products
// wx_i wy_j; every point is then four shared loads, w = (wx_i wy_j) wz_k
// (the same two roundings in the same order as the reference's tensor
// product, one of them shared by a row of points) and four coalesced stores.
__global__ void __launch_bounds__(PW * 32) mesh_points_warp(const double *__restrict__ cx,
                                                            const double *__restrict__ cy,
                                                            const double *__restrict__ cz,
                                                            const double *__restrict__ dx,
                                                            const double *__restrict__ dy,
                                                            const double *__restrict__ dz,
                                                            const int *__restrict__ sub_off,
                                                            const int *__restrict__ sub, int ncells,
                                                            long nsubcells, int p1, unsigned m1,
                                                            unsigned m2, const __grid_constant__ Tables t,
                                                            double *__restrict__ X, double *__restrict__ Y,
                                                            double *__restrict__ Z, double *__restrict__ W) {
    __shared__ double sh[PW][6][MESH_MAX_P1];
    __shared__ double sh_wxy[PW][MESH_MAX_P1 * MESH_MAX_P1];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int p3 = p1 * p1 * p1;
    double(*nd)[MESH_MAX_P1] = sh[wid];
    double *wxy = sh_wxy[wid];
    for (long s = (long)blockIdx.x * PW + wid; s < nsubcells; s += (long)gridDim.x * PW) {
        int c = (int)s, m = 1, child = 0;
        if (sub_off) {
            // last cell whose first sub-cell is <= s (every cell has >= 1)
            int a = 0, b = ncells - 1;
            while (a < b) {
                const int mid = (a + b + 1) >> 1;
                if ((long)sub_off[mid] <= s) a = mid;
                else b = mid - 1;
            }
            c = a;
            m = sub[c];
            child = (int)(s - sub_off[c]);
        }
        if (lane < p1) {
            double lo[3], hi[3];
            cell_bounds(cx, cy, cz, dx, dy, dz, c, lo, hi);
            const int ch[3] = {child / (m * m), (child / m) % m, child % m};
#pragma unroll
            for (int d = 0; d < 3; d++) {
                const double l = split_point(lo[d], hi[d], m, ch[d]);
                const double h = split_point(lo[d], hi[d], m, ch[d] + 1);
                const double hw = __dmul_rn(__dsub_rn(h, l), 0.5);
                nd[d][lane] = __dadd_rn(l, __dmul_rn(hw, __dadd_rn(t.u[lane], 1.0)));
                nd[3 + d][lane] = __dmul_rn(hw, t.w[lane]);
            }
        }
        __syncwarp();
        for (int ij = lane; ij < p1 * p1; ij += 32) {
            const int i = ij / p1, j = ij - i * p1;
            wxy[ij] = __dmul_rn(nd[3][i], nd[4][j]);
        }
        __syncwarp();
        const long base = s * p3;
        for (int q = lane; q < p3; q += 32) {
            // i = q / p2, j = (q / p1) % p1, k = q % p1 by high multiplies with
            // m = ceil(2^32 / d): exact for q d < 2^32 (q < 4096, d <= 256)
            const unsigned uq = (unsigned)q, tq = __umulhi(uq, m1);
            const int i = (int)__umulhi(uq, m2);
            const int j = (int)(tq - __umulhi(tq, m1) * (unsigned)p1);
            const int k = (int)(uq - tq * (unsigned)p1);
            X[base + q] = nd[0][i];
            Y[base + q] = nd[1][j];
            Z[base + q] = nd[2][k];
            W[base + q] = __dmul_rn(wxy[i * p1 + j], nd[5][k]);
        }
        __syncwarp();
    }
}

int grid_for(long n) {
    long g = (n + MT - 1) / MT;
    return (int)(g < 1 ? 1 : (g > (1L << 30) ? (1L << 30) : g));
}

// Host copies of small device counters, on the call's stream.
int read_ints(const int *d, int *h, int n, cudaStream_t s) {
    TAGI_CUDA(cudaMemcpyAsync(h, d, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
    TAGI_CUDA(cudaStreamSynchronize(s));
    return TAGI_OK;
}

// u_i and W_i of meshUtilities.py:835-883 from libm, for callers that pass
// no tables.  A caller that needs the bit pattern of a particular numpy
// build passes its own.
void default_tables(int order, Tables &t) {
    const int n1 = order + 1;
    const double pi = 3.141592653589793;
    // theta_i = (e_{i+1} + e_i)/2 with e_i = i * (-pi/(order+1)) + pi, e_{order+1} = 0
    const double step = -pi / n1;
    for (int i = 0; i < n1; i++) {
        const double e0 = i * step + pi, e1 = (i + 1 == n1) ? 0.0 : (i + 1) * step + pi;
        t.u[i] = std::cos((e1 + e0) / 2);
    }
    double Wv[MESH_MAX_P1] = {};
    for (int i = 0; i < n1; i++) Wv[i] = i == 0 ? 1.0 : (i % 2 == 0 ? 2.0 / (1.0 - (double)i * i) : 0.0);
    for (int j = 0; j < n1; j++) {
        double s = 0.0;
        for (int i = 0; i < n1; i++) s += 2.0 / n1 * std::cos(i * (j + 0.5) * pi / n1) * Wv[i];
        t.w[j] = s;
    }
}

}  // namespace
}  // namespace tagi

extern "C" {

int tagi_mesh_refine(const double *baseCells, int numBase, const double *atomXYZ, int numAtoms, int order,
                     double h, double H, double r, double level, int minDepth, int maxDepth, double *cellX,
                     double *cellY, double *cellZ, double *cellDX, double *cellDY, double *cellDZ,
                     int *ptsPerCellCoarse, int *ptsPerCellFine, int capacity, int *numCells,
                     long long *numCoarsePoints, long long *numFinePoints, void *stream) {
    using namespace tagi;
    if (!numCells) return set_error(TAGI_ERR_ARG, "numCells is null");
    *numCells = 0;
    if (numCoarsePoints) *numCoarsePoints = 0;
    if (numFinePoints) *numFinePoints = 0;
    if (numBase < 1 || numBase > MESH_MAX_BASE)
        return set_error(TAGI_ERR_ARG, "numBase %d outside [1, %d]", numBase, MESH_MAX_BASE);
    if (!baseCells) return set_error(TAGI_ERR_ARG, "baseCells is null");
    if (numAtoms < 0 || (numAtoms > 0 && !atomXYZ)) return set_error(TAGI_ERR_ARG, "bad atom array");
    if (order < 0 || order + 1 > MESH_MAX_P1)
        return set_error(TAGI_ERR_UNSUPPORTED, "order %d outside [0, %d]", order, MESH_MAX_P1 - 1);
    if (!std::isfinite(h) || !std::isfinite(H) || !std::isfinite(r) || !std::isfinite(level))
        return set_error(TAGI_ERR_ARG, "divide parameters must be finite");
    if (maxDepth < 0 || maxDepth > MESH_MAX_DEPTH || minDepth < 0)
        return set_error(TAGI_ERR_ARG, "maxDepth %d outside [0, %d] or minDepth %d < 0", maxDepth,
                         MESH_MAX_DEPTH, minDepth);
    if (capacity < 0) return set_error(TAGI_ERR_ARG, "capacity < 0");
    const bool query = cellX == nullptr;
    if (!query && (!cellY || !cellZ || !cellDX || !cellDY || !cellDZ))
        return set_error(TAGI_ERR_ARG, "cell table arrays must all be given (or cellX null to count)");
    Rule p;
    p.h = h;
    p.H = H;
    p.r = r;
    p.ge2 = level >= 2;
    p.ge1 = level >= 1;
    p.fine = level < -1;
    p.nsub = p.fine ? -(int)level : 1;
    p.min_depth = minDepth;
    p.max_depth = maxDepth;
    if (p.fine && p.nsub > 4)
        return set_error(TAGI_ERR_UNSUPPORTED, "fine mesh of %d^3 children per cell (1, 8, 27 or 64 supported)",
                         p.nsub);
    const int p1 = order + 1, p3 = p1 * p1 * p1;
    cudaStream_t s = (cudaStream_t)stream;
    Arena tmp;
    tmp.stream = s;
    int rc = TAGI_OK;
    do {
        int *err = nullptr, *hcnt = nullptr;
        double *cells = nullptr;
        uint64_t *keys = nullptr;
        if ((rc = tmp.alloc(&err, 2)) || (rc = tmp.alloc(&cells, 6L * numBase)) ||
            (rc = tmp.alloc(&keys, numBase)))
            break;
        (void)hcnt;
        if (cudaMemsetAsync(err, 0, 2 * sizeof(int), s) != cudaSuccess ||
            cudaMemcpyAsync(cells, baseCells, sizeof(double) * 6 * numBase, cudaMemcpyDeviceToDevice, s) !=
                cudaSuccess) {
            rc = set_error(TAGI_ERR_CUDA, "mesh setup copy failed");
            break;
        }
        launch(mesh_base_keys, grid_for(numBase), MT, 0, s, keys, numBase);
        struct Level {
            double *cells;
            uint64_t *keys;
            int *fine;
            long n;
        };
        std::vector<Level> leaves;
        long n = numBase, total = 0;
        for (int depth = 0; n > 0; depth++) {
            int *divide = nullptr, *fine = nullptr, *rank = nullptr;
            if ((rc = tmp.alloc(&divide, n)) || (rc = tmp.alloc(&fine, n)) || (rc = tmp.alloc(&rank, n + 1)))
                break;
            launch(mesh_classify, grid_for(n), MT, 0, s, cells, (int)n, depth, atomXYZ, numAtoms, p, divide,
                   fine, err);
            if (cudaGetLastError() != cudaSuccess) {
                rc = set_error(TAGI_ERR_CUDA, "mesh_classify launch failed");
                break;
            }
            if ((rc = exclusive_scan(divide, rank, (int)n, rank + n, tmp, s))) break;
            int h_div = 0;
            if ((rc = read_ints(rank + n, &h_div, 1, s))) break;
            const long nleaf = n - h_div, nnext = 8L * h_div;
            if (total + nleaf > MESH_MAX_CELLS || nnext > MESH_MAX_CELLS) {
                rc = set_error(TAGI_ERR_ARG, "refinement exceeds %ld cells", MESH_MAX_CELLS);
                break;
            }
            Level L{nullptr, nullptr, nullptr, nleaf};
            double *ncells = nullptr;
            uint64_t *nkeys = nullptr;
            if ((rc = tmp.alloc(&L.cells, 6 * nleaf)) || (rc = tmp.alloc(&L.keys, nleaf)) ||
                (rc = tmp.alloc(&L.fine, nleaf)) || (rc = tmp.alloc(&ncells, 6 * nnext)) ||
                (rc = tmp.alloc(&nkeys, nnext)))
                break;
            launch(mesh_emit, grid_for(n), MT, 0, s, cells, keys, (int)n, depth, divide, fine, rank, ncells,
                   nkeys, L.cells, L.keys, L.fine);
            if (cudaGetLastError() != cudaSuccess) {
                rc = set_error(TAGI_ERR_CUDA, "mesh_emit launch failed");
                break;
            }
            leaves.push_back(L);
            total += nleaf;
            cells = ncells;
            keys = nkeys;
            n = nnext;
        }
        if (rc) break;
        int h_err[2] = {0, 0};
        if ((rc = read_ints(err, h_err, 2, s))) break;
        if (h_err[0]) {
            rc = set_error(TAGI_ERR_ARG, "the divide rule refines below maxDepth %d", maxDepth);
            break;
        }
        *numCells = (int)total;
        if (numCoarsePoints) *numCoarsePoints = (long long)total * p3;
        // gather every level's leaves, then sort by path key (depth-first order)
        double *all_cells = nullptr;
        uint64_t *all_keys = nullptr;
        int *all_fine = nullptr, *idx = nullptr, *fsum = nullptr;
        if ((rc = tmp.alloc(&all_cells, 6 * total)) || (rc = tmp.alloc(&all_keys, total)) ||
            (rc = tmp.alloc(&all_fine, total)) || (rc = tmp.alloc(&idx, total)) ||
            (rc = tmp.alloc(&fsum, total + 1)))
            break;
        long at = 0;
        for (const Level &L : leaves) {
            if (L.n == 0) continue;
            if (cudaMemcpyAsync(all_cells + 6 * at, L.cells, sizeof(double) * 6 * L.n, cudaMemcpyDeviceToDevice,
                                s) != cudaSuccess ||
                cudaMemcpyAsync(all_keys + at, L.keys, sizeof(uint64_t) * L.n, cudaMemcpyDeviceToDevice, s) !=
                    cudaSuccess ||
                cudaMemcpyAsync(all_fine + at, L.fine, sizeof(int) * L.n, cudaMemcpyDeviceToDevice, s) !=
                    cudaSuccess) {
                rc = set_error(TAGI_ERR_CUDA, "mesh leaf gather failed");
                break;
            }
            at += L.n;
        }
        if (rc) break;
        if ((rc = exclusive_scan(all_fine, fsum, (int)total, fsum + total, tmp, s))) break;
        int h_fine = 0;
        if ((rc = read_ints(fsum + total, &h_fine, 1, s))) break;
        if (numFinePoints) *numFinePoints = (long long)h_fine * p3;
        if (query) break;
        if (capacity < total) {
            rc = set_error(TAGI_ERR_ARG, "capacity %d < %ld cells (numCells holds the count)", capacity, total);
            break;
        }
        launch(mesh_iota, grid_for(total), MT, 0, s, idx, (int)total);
        if ((rc = radix_sort_u64(all_keys, idx, (int)total, tmp, s))) break;
        launch(mesh_cell_table, grid_for(total), MT, 0, s, idx, (int)total, all_cells, all_fine, p3, cellX, cellY,
               cellZ, cellDX, cellDY, cellDZ, ptsPerCellCoarse, ptsPerCellFine);
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
            rc = set_error(TAGI_ERR_CUDA, "mesh cell table failed");
    } while (0);
    tmp.release();
    return rc;
}

int tagi_mesh_points(const double *cellX, const double *cellY, const double *cellZ, const double *cellDX,
                     const double *cellDY, const double *cellDZ, const int *ptsPerCellFine, int numCells,
                     int order, const double *unitNodes, const double *unitWeights, double *X, double *Y,
                     double *Z, double *W, long long numCoarsePoints, double *Xf, double *Yf, double *Zf,
                     double *Wf, long long numFinePoints, void *stream) {
    using namespace tagi;
    if (numCells < 0) return set_error(TAGI_ERR_ARG, "numCells < 0");
    if (order < 0 || order + 1 > MESH_MAX_P1)
        return set_error(TAGI_ERR_UNSUPPORTED, "order %d outside [0, %d]", order, MESH_MAX_P1 - 1);
    const int p1 = order + 1, p3 = p1 * p1 * p1;
    if (numCoarsePoints != (long long)numCells * p3)
        return set_error(TAGI_ERR_ARG, "numCoarsePoints %lld != numCells * (order+1)^3 = %lld", numCoarsePoints,
                         (long long)numCells * p3);
    if (numCells == 0) return TAGI_OK;
    if (!cellX || !cellY || !cellZ || !cellDX || !cellDY || !cellDZ || !X || !Y || !Z || !W)
        return set_error(TAGI_ERR_ARG, "null cell table or coarse point array");
    const bool fine = Xf || Yf || Zf || Wf;
    if (fine && (!Xf || !Yf || !Zf || !Wf || !ptsPerCellFine))
        return set_error(TAGI_ERR_ARG, "fine mesh needs Xf, Yf, Zf, Wf and ptsPerCellFine");
    if (fine && (numFinePoints < 0 || numFinePoints > 0x7fffffffLL))
        return set_error(TAGI_ERR_ARG, "numFinePoints %lld outside [0, 2^31)", numFinePoints);
    Tables t;
    if (unitNodes && unitWeights) {
        for (int i = 0; i < p1; i++) {
            t.u[i] = unitNodes[i];
            t.w[i] = unitWeights[i];
        }
    } else if (!unitNodes && !unitWeights) {
        default_tables(order, t);
    } else {
        return set_error(TAGI_ERR_ARG, "give both unitNodes and unitWeights, or neither");
    }
    for (int i = p1; i < MESH_MAX_P1; i++) t.u[i] = t.w[i] = 0.0;
    cudaStream_t s = (cudaStream_t)stream;
    const int p2 = p1 * p1;
    const unsigned m1 = p1 > 1 ? (unsigned)((0x100000000ULL + p1 - 1) / p1) : 0u;
    const unsigned m2 = p2 > 1 ? (unsigned)((0x100000000ULL + p2 - 1) / p2) : 0u;
    auto warp_grid = [](long nsubcells) {
        long g = (nsubcells + PW - 1) / PW;
        return (int)(g < 1 ? 1 : (g > 152L * 32 ? 152L * 32 : g));
    };
    launch(mesh_points_warp, warp_grid(numCells), PW * 32, 0, s, cellX, cellY, cellZ, cellDX, cellDY, cellDZ,
           (const int *)nullptr, (const int *)nullptr, numCells, (long)numCells, p1, m1, m2, t, X, Y, Z, W);
    TAGI_LAUNCH_CHECK();
    if (!fine) return TAGI_OK;
    Arena tmp;
    tmp.stream = s;
    int rc = TAGI_OK;
    do {
        // off[numCells] receives the sub-cell total, off[numCells + 1] the error flag
        int *sub = nullptr, *nsub = nullptr, *off = nullptr;
        if ((rc = tmp.alloc(&sub, numCells)) || (rc = tmp.alloc(&nsub, numCells)) ||
            (rc = tmp.alloc(&off, numCells + 2)))
            break;
        int *err = off + numCells + 1;
        if (cudaMemsetAsync(err, 0, sizeof(int), s) != cudaSuccess) {
            rc = set_error(TAGI_ERR_CUDA, "mesh memset failed");
            break;
        }
        launch(mesh_fine_counts, grid_for(numCells), MT, 0, s, ptsPerCellFine, numCells, p3, sub, nsub, err);
        if ((rc = exclusive_scan(nsub, off, numCells, off + numCells, tmp, s))) break;
        int h[2] = {0, 0};
        if ((rc = read_ints(off + numCells, h, 2, s))) break;
        if (h[1]) {
            rc = set_error(TAGI_ERR_ARG, "a fine cell holds a point count other than 1, 8, 27 or 64 x (order+1)^3");
            break;
        }
        const long long fine_pts = (long long)h[0] * p3;
        if (fine_pts != numFinePoints) {
            rc = set_error(TAGI_ERR_ARG, "ptsPerCellFine sums to %lld, numFinePoints is %lld", fine_pts,
                           numFinePoints);
            break;
        }
        if (numFinePoints == 0) break;
        launch(mesh_points_warp, warp_grid(h[0]), PW * 32, 0, s, cellX, cellY, cellZ, cellDX, cellDY, cellDZ,
               (const int *)off, (const int *)sub, numCells, (long)h[0], p1, m1, m2, t, Xf, Yf, Zf, Wf);
        if (cudaGetLastError() != cudaSuccess) rc = set_error(TAGI_ERR_CUDA, "mesh_points_warp launch failed");
    } while (0);
    tmp.release();
    return rc;
}

}  // extern "C"
