/*
 * tagi_oracle.c -- CPU FP64 oracle for the treecode convolution path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py load this library, and only as the checker or
 * the timed CPU baseline.  The product (libtagi_gb300.so) never links it.
 *
 * What it restates, and how far parity is pinned:
 *
 *  - oracle_direct(): FP64 direct sum of the Yukawa / Coulomb convolution with
 *    singularity subtraction or skipping.  Formulas follow the reference call
 *    sites and its in-repo prototypes:
 *      Yukawa SS   phi_i = sum_{j!=i} w_j (f_j - f_i) e^{-k r}/r + f_i 4 pi / k^2
 *                  (3D-GreenIteration/src/dataStructures/TreeStruct_CC.py:2782,2795;
 *                   kernel parameter k from greenIterationFixedPoint.py:207,222)
 *      Coulomb SS  V_i = sum_{j!=i} w_j (rho_j - rho_i e^{-a^2 r^2})/r + rho_i 2 pi / a^2
 *                  (TreeStruct_CC.py:2931; parameter a from scfFixedPoint.py:244)
 *      skipping    sum_{j!=i} w_j f_j G(r)
 *    Pinned against closed-form integrals in the tests (math, not reference).
 *
 *  - oracle_plan_*(): the treecode.  BaryTree, the library the reference calls
 *    (3D-GreenIteration/src/utilities/BaryTreeInterface.py:52-83), is not part
 *    of the reference tree, so its tree rules cannot be read.  PARITY UNPINNED
 *    against BaryTree: this file and the CUDA library implement the same
 *    project-defined rules (compressed Morton octree, MAC (rB+rC) < theta*R,
 *    size check count > sizeCheck*(n+1)^3, particle-cluster barycentric
 *    Lagrange interpolation on Chebyshev 2nd-kind proxy grids), and the GPU
 *    lists must equal these integer-for-integer.
 *
 *  - oracle_mgs(): restates modifiedGramSchmidt_singleWavefunction,
 *    3D-GreenIteration/src/utilities/Orthogonalization.c:14-119 (one rank).
 *  - oracle_interp(): restates InterpolateBetweenTwoMeshes and
 *    interapolateBetweenTwoMeshesSingleCell,
 *    3D-GreenIteration/src/utilities/TwoMeshInterpolation.c:12-153,163-234,
 *    including the x exact-node test against the z index (:127).
 *    Both are pinned against the reference C compiled from its own sources
 *    (oracle/_ref) and against committed golden vectors.
 *
 * Build: gcc -O2 -fopenmp -ffp-contract=off -fPIC -shared (oracle/Makefile).
 * -ffp-contract=off keeps every FP64 operation separately rounded so the
 * tree decisions match the device kernels bit for bit.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Kernel / singularity enum values: BaryTreeInterface.py:20-37 */
enum { K_COULOMB = 1, K_YUKAWA = 2 };
enum { S_NONE = 0, S_SKIPPING = 1, S_SUBTRACTION = 2 };

static const double PI_D = 3.14159265358979323846;

/* ------------------------------------------------------------------------ */
/* Pair kernel, FP64.                                                        */
/* ------------------------------------------------------------------------ */
static inline double pair_term(int kernel, int sing, double kp, double r,
                               double fj, double wj, double fi)
{
    if (kernel == K_YUKAWA) {
        double g = exp(-kp * r) / r;
        if (sing == S_SUBTRACTION) return wj * (fj - fi) * g;
        return wj * fj * g;
    } else { /* Coulomb */
        if (sing == S_SUBTRACTION) return wj * (fj - fi * exp(-kp * kp * r * r)) / r;
        return wj * fj / r;
    }
}

static inline double ss_term(int kernel, int sing, double kp, double fi)
{
    if (sing != S_SUBTRACTION) return 0.0;
    if (kernel == K_YUKAWA) return fi * 4.0 * PI_D / (kp * kp);
    return fi * 2.0 * PI_D / (kp * kp);
}

/*
 * Direct sum over all sources for the targets listed in sub[0..nsub) (or all
 * targets when sub == NULL, nsub = nt).  out[q] is the value at target sub[q].
 */
void oracle_direct(int nt, const double *tx, const double *ty, const double *tz,
                   const double *tv, int ns, const double *sx, const double *sy,
                   const double *sz, const double *sv, const double *sw,
                   int kernel, const double *kparams, int sing,
                   int nsub, const int *sub, double *out, int nthreads)
{
    double kp = kparams[0];
    (void)nt;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (int q = 0; q < nsub; q++) {
        int i = sub ? sub[q] : q;
        double xi = tx[i], yi = ty[i], zi = tz[i], fi = tv[i];
        double acc = 0.0;
        for (int j = 0; j < ns; j++) {
            double dx = xi - sx[j], dy = yi - sy[j], dz = zi - sz[j];
            double r2 = dx * dx + dy * dy + dz * dz;
            if (r2 > 0.0) acc += pair_term(kernel, sing, kp, sqrt(r2), sv[j], sw[j], fi);
        }
        out[q] = acc + ss_term(kernel, sing, kp, fi);
    }
}

/* ------------------------------------------------------------------------ */
/* Compressed Morton octree (project-defined rules, shared with the device). */
/* ------------------------------------------------------------------------ */
typedef struct {
    int n;               /* points */
    int nnodes;
    int nlevels;
    uint64_t *codes;     /* sorted Morton codes [n] */
    int *perm;           /* sorted position -> original index [n] */
    double *x, *y, *z;   /* sorted coordinates [n] */
    int *begin, *end, *parent, *first_child, *nchild, *depth;  /* [nnodes] */
    int *level_start;    /* [nlevels+1] node index where each BFS level starts */
    double *center;      /* [3*nnodes] */
    double *half;        /* [3*nnodes] tight half widths */
    double *radius;      /* [nnodes] */
} otree;

static inline uint64_t spread21(uint32_t v)
{
    uint64_t r = 0;
    for (int b = 0; b < 21; b++) r |= (uint64_t)((v >> b) & 1u) << (3 * b);
    return r;
}

typedef struct { uint64_t code; int idx; } keyidx;
static int cmp_keyidx(const void *a, const void *b)
{
    const keyidx *p = (const keyidx *)a, *q = (const keyidx *)b;
    if (p->code < q->code) return -1;
    if (p->code > q->code) return 1;
    return (p->idx > q->idx) - (p->idx < q->idx);
}

static inline int digit_at(uint64_t code, int g) { return (int)((code >> (3 * g)) & 7u); }

/* Split digit of a range [b,e) of sorted codes, or -1 when it cannot split. */
static int split_digit(const uint64_t *codes, int b, int e)
{
    uint64_t x = codes[b] ^ codes[e - 1];
    if (x == 0) return -1;
    int hb = 63 - __builtin_clzll(x);
    return hb / 3;
}

static void tree_build(otree *t, int n, const double *x, const double *y, const double *z, int leaf)
{
    memset(t, 0, sizeof(*t));
    t->n = n;
    double lo[3] = {x[0], y[0], z[0]}, hi[3] = {x[0], y[0], z[0]};
    for (int i = 1; i < n; i++) {
        if (x[i] < lo[0]) lo[0] = x[i];
        if (x[i] > hi[0]) hi[0] = x[i];
        if (y[i] < lo[1]) lo[1] = y[i];
        if (y[i] > hi[1]) hi[1] = y[i];
        if (z[i] < lo[2]) lo[2] = z[i];
        if (z[i] > hi[2]) hi[2] = z[i];
    }
    double ext = hi[0] - lo[0];
    if (hi[1] - lo[1] > ext) ext = hi[1] - lo[1];
    if (hi[2] - lo[2] > ext) ext = hi[2] - lo[2];
    if (!(ext > 0.0)) ext = 1.0;
    double scale = 2097152.0 / ext;

    keyidx *ki = (keyidx *)malloc(sizeof(keyidx) * (size_t)n);
    for (int i = 0; i < n; i++) {
        const double p[3] = {x[i], y[i], z[i]};
        uint32_t q[3];
        for (int d = 0; d < 3; d++) {
            double s = (p[d] - lo[d]) * scale;
            uint32_t v = (uint32_t)s;
            q[d] = v > 2097151u ? 2097151u : v;
        }
        ki[i].code = (spread21(q[0]) << 2) | (spread21(q[1]) << 1) | spread21(q[2]);
        ki[i].idx = i;
    }
    qsort(ki, (size_t)n, sizeof(keyidx), cmp_keyidx);
    t->codes = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n);
    t->perm = (int *)malloc(sizeof(int) * (size_t)n);
    t->x = (double *)malloc(sizeof(double) * (size_t)n);
    t->y = (double *)malloc(sizeof(double) * (size_t)n);
    t->z = (double *)malloc(sizeof(double) * (size_t)n);
    for (int i = 0; i < n; i++) {
        t->codes[i] = ki[i].code;
        t->perm[i] = ki[i].idx;
        t->x[i] = x[ki[i].idx];
        t->y[i] = y[ki[i].idx];
        t->z[i] = z[ki[i].idx];
    }
    free(ki);

    int cap = 2 * n + 1;
    t->begin = (int *)malloc(sizeof(int) * cap);
    t->end = (int *)malloc(sizeof(int) * cap);
    t->parent = (int *)malloc(sizeof(int) * cap);
    t->first_child = (int *)malloc(sizeof(int) * cap);
    t->nchild = (int *)malloc(sizeof(int) * cap);
    t->depth = (int *)malloc(sizeof(int) * cap);
    t->level_start = (int *)malloc(sizeof(int) * 66);

    /* BFS: level by level, children in (parent order, digit order). */
    int nn = 1;
    t->begin[0] = 0; t->end[0] = n; t->parent[0] = -1; t->depth[0] = 0;
    int lvl = 0, ls = 0, le = 1;
    t->level_start[0] = 0;
    while (ls < le) {
        for (int v = ls; v < le; v++) {
            int b = t->begin[v], e = t->end[v];
            t->first_child[v] = -1;
            t->nchild[v] = 0;
            if (e - b <= leaf) continue;
            int g = split_digit(t->codes, b, e);
            if (g < 0) continue;
            t->first_child[v] = nn;
            int pos = b;
            for (int d = 0; d < 8; d++) {
                int s = pos;
                while (pos < e && digit_at(t->codes[pos], g) == d) pos++;
                if (pos > s) {
                    t->begin[nn] = s; t->end[nn] = pos; t->parent[nn] = v;
                    t->depth[nn] = lvl + 1;
                    nn++;
                    t->nchild[v]++;
                }
            }
        }
        lvl++;
        ls = le; le = nn;
        t->level_start[lvl] = ls;
    }
    t->nnodes = nn;
    t->nlevels = lvl;

    t->center = (double *)malloc(sizeof(double) * 3 * nn);
    t->half = (double *)malloc(sizeof(double) * 3 * nn);
    t->radius = (double *)malloc(sizeof(double) * nn);
    for (int v = 0; v < nn; v++) {
        double l[3] = {t->x[t->begin[v]], t->y[t->begin[v]], t->z[t->begin[v]]};
        double h[3] = {l[0], l[1], l[2]};
        for (int i = t->begin[v] + 1; i < t->end[v]; i++) {
            double p[3] = {t->x[i], t->y[i], t->z[i]};
            for (int d = 0; d < 3; d++) {
                if (p[d] < l[d]) l[d] = p[d];
                if (p[d] > h[d]) h[d] = p[d];
            }
        }
        for (int d = 0; d < 3; d++) {
            t->center[3 * v + d] = (l[d] + h[d]) * 0.5;
            t->half[3 * v + d] = (h[d] - l[d]) * 0.5;
        }
        double hx = t->half[3 * v], hy = t->half[3 * v + 1], hz = t->half[3 * v + 2];
        double s = hx * hx;
        s = s + hy * hy;
        s = s + hz * hz;
        t->radius[v] = sqrt(s);
    }
}

static void tree_free(otree *t)
{
    free(t->codes); free(t->perm); free(t->x); free(t->y); free(t->z);
    free(t->begin); free(t->end); free(t->parent); free(t->first_child);
    free(t->nchild); free(t->depth); free(t->level_start);
    free(t->center); free(t->half); free(t->radius);
}

/* ------------------------------------------------------------------------ */
/* Plan: source tree, target batches, interaction lists.                    */
/* ------------------------------------------------------------------------ */
typedef struct {
    otree src, tgt;
    int degree;
    double theta, size_check;
    int nbatch;
    int *batch_node;          /* target-tree leaf node of each batch, ascending begin */
    int *near_off, *near_list, *far_off, *far_list;
    int nslots;
    int *node_slot;           /* [src.nnodes] slot or -1 */
    int *slot_node;
    double *what;             /* [nslots * P] weight modified charges */
} oplan;

static inline int mac_far(const otree *s, int c, const otree *t, int b, double theta)
{
    double dx = t->center[3 * b] - s->center[3 * c];
    double dy = t->center[3 * b + 1] - s->center[3 * c + 1];
    double dz = t->center[3 * b + 2] - s->center[3 * c + 2];
    double d2 = dx * dx;
    d2 = d2 + dy * dy;
    d2 = d2 + dz * dz;
    double dist = sqrt(d2);
    return (t->radius[b] + s->radius[c]) < theta * dist;
}

/* Pre-order DFS of the source tree for one batch.  mode 0 counts, 1 fills. */
static void traverse(const oplan *p, int b, int *nn, int *nf, int *near_out, int *far_out)
{
    const otree *s = &p->src;
    int P = (p->degree + 1) * (p->degree + 1) * (p->degree + 1);
    double thresh = p->size_check * (double)P;
    int stack[256];
    int sp = 0;
    stack[sp++] = 0;
    int cn = 0, cf = 0;
    while (sp > 0) {
        int c = stack[--sp];
        int cnt = s->end[c] - s->begin[c];
        if (mac_far(s, c, &p->tgt, b, p->theta)) {
            if ((double)cnt > thresh) { if (far_out) far_out[cf] = c; cf++; }
            else { if (near_out) near_out[cn] = c; cn++; }
        } else if (s->nchild[c] == 0) {
            if (near_out) near_out[cn] = c; cn++;
        } else {
            for (int k = s->nchild[c] - 1; k >= 0; k--) stack[sp++] = s->first_child[c] + k;
        }
    }
    *nn = cn; *nf = cf;
}

static const double *cheb2_nodes(int degree, double *buf)
{
    for (int m = 0; m <= degree; m++) buf[m] = cos(PI_D * (double)m / (double)degree);
    return buf;
}

/* Barycentric Lagrange basis on 2nd-kind Chebyshev nodes, at u in [-1,1]. */
static void bary_basis(int degree, const double *tn, double u, double *L)
{
    int exact = -1;
    double den = 0.0;
    for (int m = 0; m <= degree; m++) {
        double d = u - tn[m];
        if (d == 0.0) exact = m;
    }
    if (exact >= 0) {
        for (int m = 0; m <= degree; m++) L[m] = (m == exact) ? 1.0 : 0.0;
        return;
    }
    for (int m = 0; m <= degree; m++) {
        double wm = ((m & 1) ? -1.0 : 1.0) * ((m == 0 || m == degree) ? 0.5 : 1.0);
        L[m] = wm / (u - tn[m]);
        den += L[m];
    }
    for (int m = 0; m <= degree; m++) L[m] = L[m] / den;
}

/* Proxy half width of a node along one axis: zero widths get a small one. */
static inline double proxy_half(const otree *s, int c, int d)
{
    double h = s->half[3 * c + d];
    if (h > 0.0) return h;
    double hm = s->half[3 * c];
    if (s->half[3 * c + 1] > hm) hm = s->half[3 * c + 1];
    if (s->half[3 * c + 2] > hm) hm = s->half[3 * c + 2];
    return hm > 0.0 ? hm * 1.0e-3 : 1.0;
}

/* Modified charges of one slot: out[P] = sum_j L_k(y_j) * q_j (sorted order). */
static void p2m(const oplan *p, int slot, const double *qsorted, double *out)
{
    const otree *s = &p->src;
    int n1 = p->degree + 1, P = n1 * n1 * n1;
    int c = p->slot_node[slot];
    double tn[32], Lx[32], Ly[32], Lz[32];
    cheb2_nodes(p->degree, tn);
    double cx = s->center[3 * c], cy = s->center[3 * c + 1], cz = s->center[3 * c + 2];
    double hx = proxy_half(s, c, 0), hy = proxy_half(s, c, 1), hz = proxy_half(s, c, 2);
    for (int k = 0; k < P; k++) out[k] = 0.0;
    for (int j = s->begin[c]; j < s->end[c]; j++) {
        bary_basis(p->degree, tn, (s->x[j] - cx) / hx, Lx);
        bary_basis(p->degree, tn, (s->y[j] - cy) / hy, Ly);
        bary_basis(p->degree, tn, (s->z[j] - cz) / hz, Lz);
        double q = qsorted[j];
        for (int a = 0; a < n1; a++)
            for (int bb = 0; bb < n1; bb++) {
                double lxy = Lx[a] * Ly[bb] * q;
                for (int g = 0; g < n1; g++) out[(a * n1 + bb) * n1 + g] += lxy * Lz[g];
            }
    }
}

void *oracle_plan_create(int nt, const double *tx, const double *ty, const double *tz,
                         int ns, const double *sx, const double *sy, const double *sz,
                         const double *sw, double theta, int degree, int src_leaf,
                         int tgt_leaf, double size_check)
{
    if (nt <= 0 || ns <= 0 || degree < 1 || degree > 30) return NULL;
    oplan *p = (oplan *)calloc(1, sizeof(oplan));
    p->degree = degree; p->theta = theta; p->size_check = size_check;
    tree_build(&p->src, ns, sx, sy, sz, src_leaf);
    tree_build(&p->tgt, nt, tx, ty, tz, tgt_leaf);

    /* Batches: leaves of the target tree in ascending begin (Morton) order. */
    int *leaf_at = (int *)malloc(sizeof(int) * (size_t)nt);
    for (int i = 0; i < nt; i++) leaf_at[i] = -1;
    for (int v = 0; v < p->tgt.nnodes; v++)
        if (p->tgt.nchild[v] == 0) leaf_at[p->tgt.begin[v]] = v;
    p->nbatch = 0;
    for (int i = 0; i < nt; i++) if (leaf_at[i] >= 0) p->nbatch++;
    p->batch_node = (int *)malloc(sizeof(int) * p->nbatch);
    for (int i = 0, k = 0; i < nt; i++) if (leaf_at[i] >= 0) p->batch_node[k++] = leaf_at[i];
    free(leaf_at);

    p->near_off = (int *)malloc(sizeof(int) * (p->nbatch + 1));
    p->far_off = (int *)malloc(sizeof(int) * (p->nbatch + 1));
    p->near_off[0] = p->far_off[0] = 0;
    for (int b = 0; b < p->nbatch; b++) {
        int cn, cf;
        traverse(p, p->batch_node[b], &cn, &cf, NULL, NULL);
        p->near_off[b + 1] = p->near_off[b] + cn;
        p->far_off[b + 1] = p->far_off[b] + cf;
    }
    p->near_list = (int *)malloc(sizeof(int) * (p->near_off[p->nbatch] + 1));
    p->far_list = (int *)malloc(sizeof(int) * (p->far_off[p->nbatch] + 1));
    for (int b = 0; b < p->nbatch; b++) {
        int cn, cf;
        traverse(p, p->batch_node[b], &cn, &cf, p->near_list + p->near_off[b],
                 p->far_list + p->far_off[b]);
    }

    /* Slots: far-list nodes in ascending node index. */
    p->node_slot = (int *)malloc(sizeof(int) * p->src.nnodes);
    for (int v = 0; v < p->src.nnodes; v++) p->node_slot[v] = -1;
    for (int e = 0; e < p->far_off[p->nbatch]; e++) p->node_slot[p->far_list[e]] = 1;
    p->nslots = 0;
    for (int v = 0; v < p->src.nnodes; v++)
        if (p->node_slot[v] >= 0) p->node_slot[v] = p->nslots++;
    p->slot_node = (int *)malloc(sizeof(int) * (p->nslots + 1));
    for (int v = 0; v < p->src.nnodes; v++)
        if (p->node_slot[v] >= 0) p->slot_node[p->node_slot[v]] = v;

    /* Weight modified charges do not depend on the charges: build once. */
    int n1 = degree + 1, P = n1 * n1 * n1;
    p->what = (double *)malloc(sizeof(double) * (size_t)P * (p->nslots + 1));
    double *wsorted = (double *)malloc(sizeof(double) * ns);
    for (int j = 0; j < ns; j++) wsorted[j] = sw[p->src.perm[j]];
    for (int sl = 0; sl < p->nslots; sl++) p2m(p, sl, wsorted, p->what + (size_t)sl * P);
    free(wsorted);
    return p;
}

void oracle_plan_destroy(void *vp)
{
    oplan *p = (oplan *)vp;
    if (!p) return;
    tree_free(&p->src); tree_free(&p->tgt);
    free(p->batch_node); free(p->near_off); free(p->near_list);
    free(p->far_off); free(p->far_list); free(p->node_slot); free(p->slot_node);
    free(p->what);
    free(p);
}

/* info[0..8] = src nodes, tgt nodes, batches, near total, far total, slots,
 *              src levels, tgt levels, P */
void oracle_plan_info(void *vp, int *info)
{
    oplan *p = (oplan *)vp;
    int n1 = p->degree + 1;
    info[0] = p->src.nnodes; info[1] = p->tgt.nnodes; info[2] = p->nbatch;
    info[3] = p->near_off[p->nbatch]; info[4] = p->far_off[p->nbatch];
    info[5] = p->nslots; info[6] = p->src.nlevels; info[7] = p->tgt.nlevels;
    info[8] = n1 * n1 * n1;
}

/* which: 0 = source tree, 1 = target tree. */
void oracle_plan_get_tree(void *vp, int which, uint64_t *codes, int *perm, int *begin,
                          int *end, int *parent, int *first_child, int *nchild,
                          double *center, double *half, double *radius)
{
    oplan *p = (oplan *)vp;
    otree *t = which ? &p->tgt : &p->src;
    memcpy(codes, t->codes, sizeof(uint64_t) * t->n);
    memcpy(perm, t->perm, sizeof(int) * t->n);
    memcpy(begin, t->begin, sizeof(int) * t->nnodes);
    memcpy(end, t->end, sizeof(int) * t->nnodes);
    memcpy(parent, t->parent, sizeof(int) * t->nnodes);
    memcpy(first_child, t->first_child, sizeof(int) * t->nnodes);
    memcpy(nchild, t->nchild, sizeof(int) * t->nnodes);
    memcpy(center, t->center, sizeof(double) * 3 * t->nnodes);
    memcpy(half, t->half, sizeof(double) * 3 * t->nnodes);
    memcpy(radius, t->radius, sizeof(double) * t->nnodes);
}

void oracle_plan_get_lists(void *vp, int *batch_node, int *near_off, int *near_list,
                           int *far_off, int *far_list, int *slot_node)
{
    oplan *p = (oplan *)vp;
    memcpy(batch_node, p->batch_node, sizeof(int) * p->nbatch);
    memcpy(near_off, p->near_off, sizeof(int) * (p->nbatch + 1));
    memcpy(far_off, p->far_off, sizeof(int) * (p->nbatch + 1));
    memcpy(near_list, p->near_list, sizeof(int) * p->near_off[p->nbatch]);
    memcpy(far_list, p->far_list, sizeof(int) * p->far_off[p->nbatch]);
    memcpy(slot_node, p->slot_node, sizeof(int) * p->nslots);
}

/* Modified charges for a charge vector given in ORIGINAL source order
 * (q_j = sourceValue_j * sourceWeight_j is formed here). */
void oracle_plan_modified_charges(void *vp, const double *sv, const double *sw, double *qhat)
{
    oplan *p = (oplan *)vp;
    int ns = p->src.n, n1 = p->degree + 1, P = n1 * n1 * n1;
    double *qs = (double *)malloc(sizeof(double) * ns);
    for (int j = 0; j < ns; j++) qs[j] = sv[p->src.perm[j]] * sw[p->src.perm[j]];
    for (int sl = 0; sl < p->nslots; sl++) p2m(p, sl, qs, qhat + (size_t)sl * P);
    free(qs);
}

void oracle_plan_weight_charges(void *vp, double *what)
{
    oplan *p = (oplan *)vp;
    int n1 = p->degree + 1, P = n1 * n1 * n1;
    memcpy(what, p->what, sizeof(double) * (size_t)P * p->nslots);
}

static double wall_s(void)
{
#ifdef _OPENMP
    return omp_get_wtime();
#else
    return 0.0;
#endif
}

/*
 * FP64 treecode convolution for the batches listed in sel[0..nsel) (all
 * batches when sel == NULL).  tv, sv, sw in original order; out in original
 * target order (only the selected batches' targets are written).
 * phi_i = near(direct) + far(proxy) + SS term.  times[0] = upward pass s,
 * times[1] = field s; pairs[0] = near pairs, pairs[1] = far pairs (selected).
 */
void oracle_plan_convolve_batches_timed(void *vp, const double *tv, const double *sv, const double *sw,
                                        int kernel, const double *kparams, int sing, double *out,
                                        int nthreads, int nsel, const int *sel, double *times,
                                        double *pairs, double *batch_s);

void oracle_plan_convolve_batches(void *vp, const double *tv, const double *sv, const double *sw,
                                  int kernel, const double *kparams, int sing, double *out,
                                  int nthreads, int nsel, const int *sel, double *times,
                                  double *pairs)
{
    oracle_plan_convolve_batches_timed(vp, tv, sv, sw, kernel, kparams, sing, out, nthreads, nsel, sel,
                                       times, pairs, NULL);
}

/* As oracle_plan_convolve_batches; batch_s (if not NULL) receives each
 * evaluated batch's own seconds, in the order of sel. */
void oracle_plan_convolve_batches_timed(void *vp, const double *tv, const double *sv, const double *sw,
                                        int kernel, const double *kparams, int sing, double *out,
                                        int nthreads, int nsel, const int *sel, double *times,
                                        double *pairs, double *batch_s)
{
    oplan *p = (oplan *)vp;
    const otree *s = &p->src, *t = &p->tgt;
    int ns = s->n, n1 = p->degree + 1, P = n1 * n1 * n1;
    double kp = kparams[0];
    double t0 = wall_s();
    double *qs = (double *)malloc(sizeof(double) * ns);
    double *ws = (double *)malloc(sizeof(double) * ns);
    double *fs = (double *)malloc(sizeof(double) * ns);
    for (int j = 0; j < ns; j++) {
        int o = s->perm[j];
        qs[j] = sv[o] * sw[o];
        ws[j] = sw[o];
        fs[j] = sv[o];
    }
    double *qhat = (double *)malloc(sizeof(double) * (size_t)P * (p->nslots + 1));
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int sl = 0; sl < p->nslots; sl++) p2m(p, sl, qs, qhat + (size_t)sl * P);
    double t1 = wall_s();

    double tn[32];
    cheb2_nodes(p->degree, tn);
    int sing_ss = (sing == S_SUBTRACTION);
    int nrun = sel ? nsel : p->nbatch;
    double npairs = 0.0, fpairs = 0.0, busy = 0.0;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : npairs, fpairs, busy)
#endif
    for (int bi = 0; bi < nrun; bi++) {
        double tb = wall_s();
        int b = sel ? sel[bi] : bi;
        int bn = p->batch_node[b];
        int nb = t->end[bn] - t->begin[bn];
        for (int e = p->near_off[b]; e < p->near_off[b + 1]; e++) {
            int c = p->near_list[e];
            npairs += (double)nb * (double)(s->end[c] - s->begin[c]);
        }
        fpairs += (double)nb * (double)(p->far_off[b + 1] - p->far_off[b]) * (double)P;
        for (int i = t->begin[bn]; i < t->end[bn]; i++) {
            int oi = t->perm[i];
            double xi = t->x[i], yi = t->y[i], zi = t->z[i], fi = tv[oi];
            double acc = 0.0;
            for (int e = p->near_off[b]; e < p->near_off[b + 1]; e++) {
                int c = p->near_list[e];
                for (int j = s->begin[c]; j < s->end[c]; j++) {
                    double dx = xi - s->x[j], dy = yi - s->y[j], dz = zi - s->z[j];
                    double r2 = dx * dx + dy * dy + dz * dz;
                    if (r2 > 0.0) acc += pair_term(kernel, sing, kp, sqrt(r2), fs[j], ws[j], fi);
                }
            }
            for (int e = p->far_off[b]; e < p->far_off[b + 1]; e++) {
                int c = p->far_list[e];
                int sl = p->node_slot[c];
                const double *qh = qhat + (size_t)sl * P, *wh = p->what + (size_t)sl * P;
                double cx = s->center[3 * c], cy = s->center[3 * c + 1], cz = s->center[3 * c + 2];
                double hx = proxy_half(s, c, 0), hy = proxy_half(s, c, 1), hz = proxy_half(s, c, 2);
                for (int a = 0; a < n1; a++) {
                    double dx = xi - (cx + hx * tn[a]);
                    for (int bb = 0; bb < n1; bb++) {
                        double dy = yi - (cy + hy * tn[bb]);
                        for (int g = 0; g < n1; g++) {
                            double dz = zi - (cz + hz * tn[g]);
                            double r = sqrt(dx * dx + dy * dy + dz * dz);
                            int k = (a * n1 + bb) * n1 + g;
                            if (kernel == K_YUKAWA) {
                                double gk = exp(-kp * r) / r;
                                acc += gk * (sing_ss ? (qh[k] - fi * wh[k]) : qh[k]);
                            } else {
                                if (sing_ss) acc += (qh[k] - fi * wh[k] * exp(-kp * kp * r * r)) / r;
                                else acc += qh[k] / r;
                            }
                        }
                    }
                }
            }
            out[oi] = acc + ss_term(kernel, sing, kp, fi);
        }
        double dt = wall_s() - tb;
        busy += dt;
        if (batch_s) batch_s[bi] = dt;
    }
    double t2 = wall_s();
    /* times: upward pass (wall), fields (wall), fields summed over the batches (thread-seconds) */
    if (times) { times[0] = t1 - t0; times[1] = t2 - t1; times[2] = busy; }
    if (pairs) { pairs[0] = npairs; pairs[1] = fpairs; }
    free(qs); free(ws); free(fs); free(qhat);
}

void oracle_plan_convolve(void *vp, const double *tv, const double *sv, const double *sw,
                          int kernel, const double *kparams, int sing, double *out,
                          int nthreads)
{
    oracle_plan_convolve_batches(vp, tv, sv, sw, kernel, kparams, sing, out, nthreads, 0, NULL,
                                 NULL, NULL);
}

/* ------------------------------------------------------------------------ */
/* Weighted modified Gram-Schmidt: Orthogonalization.c:14-119, one rank.    */
/* ------------------------------------------------------------------------ */
void oracle_mgs(double *V, double *U, const double *W, int target, int npts, int nwave)
{
    (void)nwave;
    double *r = (double *)malloc(sizeof(double) * (target > 0 ? target : 1));
    for (int i = 0; i < target; i++) {           /* :44-54 */
        double s = 0.0;
        for (int j = 0; j < npts; j++) s += V[(size_t)i * npts + j] * U[j] * W[j];
        r[i] = s;
    }
    for (int i = 0; i < target; i++)             /* :71-79 */
        for (int j = 0; j < npts; j++) U[j] -= V[(size_t)i * npts + j] * r[i];
    double nrm2 = 0.0;                           /* :85-87 */
    for (int j = 0; j < npts; j++) nrm2 += U[j] * U[j] * W[j];
    double nrm = sqrt(nrm2);                     /* :95 */
    for (int j = 0; j < npts; j++) {             /* :103-106 */
        U[j] /= nrm;
        V[(size_t)target * npts + j] = U[j];
    }
    free(r);
}

/* ------------------------------------------------------------------------ */
/* Two-mesh interpolation: TwoMeshInterpolation.c:12-153,163-234.          */
/* ------------------------------------------------------------------------ */
static void interp_cell(const double *cX, const double *cY, const double *cZ, const double *cF,
                        int nc, int cidx, const double *fX, const double *fY, const double *fZ,
                        double *fF, int nf, int fidx, int order)
{
    int p1 = order + 1;
    double nx[64], ny[64], nz[64], w[64];
    for (int i = 0; i < p1; i++) {               /* :40-44 */
        nx[i] = cX[cidx + i * p1 * p1];
        ny[i] = cY[cidx + i * p1];
        nz[i] = cZ[cidx + i];
    }
    for (int i = 0; i < p1; i++)                 /* :49-51 */
        w[i] = pow(-1, i) * sin((2 * i + 1) * PI_D / (2 * (p1 - 1) + 2));
    for (int i = 0; i < nf; i++) {
        double sx = 0, sy = 0, sz = 0;
        double tx = fX[fidx + i], ty = fY[fidx + i], tz = fZ[fidx + i];
        int eix = -1, eiy = -1, eiz = -1;
        for (int j = 0; j < p1; j++) {           /* :73-91 */
            double cx = tx - nx[j], cy = ty - ny[j], cz = tz - nz[j];
            if (fabs(cx) < DBL_MIN) eix = j;
            if (fabs(cy) < DBL_MIN) eiy = j;
            if (fabs(cz) < DBL_MIN) eiz = j;
            sx += w[j] / cx;
            sy += w[j] / cy;
            sz += w[j] / cz;
        }
        double den = 1.0;                        /* :93-96 */
        if (eix == -1) den /= sx;
        if (eiy == -1) den /= sy;
        if (eiz == -1) den /= sz;
        double temp = 0.0;
        for (int j = 0; j < nc; j++) {           /* :103-143 */
            int k1 = j % p1;
            int kk = (j - k1) / p1;
            int k2 = kk % p1;
            kk = kk - k2;
            int k3 = kk / p1;
            double w3 = w[k1], w2 = w[k2], w1 = w[k3];
            double cx = nx[k3], cy = ny[k2], cz = nz[k1];
            double cq = cF[cidx + j];
            double num = 1.0;
            if (eix == -1) num *= w1 / (tx - cx);
            else if (eix != k1) num *= 0;        /* :127 compares with k1, kept as is */
            if (eiy == -1) num *= w2 / (ty - cy);
            else if (eiy != k2) num *= 0;
            if (eiz == -1) num *= w3 / (tz - cz);
            else if (eiz != k3) num *= 0;
            temp += num * den * cq;
        }
        fF[i + fidx] += temp;
    }
}

void oracle_interp(const double *cX, const double *cY, const double *cZ, const double *cF,
                   const int *ppc_c, int coarseN, const double *fX, const double *fY,
                   const double *fZ, double *fF, const int *ppc_f, int fineN, int ncells,
                   int order)
{
    if (coarseN == fineN) {                      /* :175-180 */
        for (int i = 0; i < coarseN; i++) fF[i] = cF[i];
        return;
    }
    double *same = (double *)calloc((size_t)fineN, sizeof(double));
    int ci = 0, fi = 0;
    for (int c = 0; c < ncells; c++) {           /* :201-221 */
        if (ppc_c[c] == ppc_f[c]) {
            for (int j = 0; j < ppc_f[c]; j++) same[fi + j] = cF[ci + j];
        } else {
            interp_cell(cX, cY, cZ, cF, ppc_c[c], ci, fX, fY, fZ, fF, ppc_f[c], fi, order);
        }
        ci += ppc_c[c];
        fi += ppc_f[c];
    }
    for (int i = 0; i < fineN; i++) fF[i] = fF[i] + same[i];   /* :228-230 */
    free(same);
}
