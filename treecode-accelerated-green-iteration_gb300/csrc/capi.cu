// C ABI of libtagi_gb300.so (declared in include/tagi_gb300.h).
//
// Host-pointer drop-ins keep the reference's signatures and argument
// meaning; device-pointer entry points return a status.  No entry point
// exits the process: a failure sets a thread-local code + message, and the
// void drop-ins also print that message to stderr (the reference's library
// printed and exited instead).
#include "tagi_internal.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <mutex>

namespace tagi {

namespace {
thread_local int g_err = 0;
thread_local char g_msg[1024] = "";
int g_precision = -1;
std::mutex g_mu;
cudaStream_t g_streams[64] = {};

cudaStream_t host_stream() {
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_streams[dev]) cudaStreamCreateWithFlags(&g_streams[dev], cudaStreamNonBlocking);
    return g_streams[dev];
}

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
}  // namespace

int set_error(int code, const char *fmt, ...) {
    g_err = code;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
    va_end(ap);
    return code;
}

int last_error() { return g_err; }

int validate(int nt, int ns, int kernel, int nkp, const double *kp, int sing, int approx,
             int ctype, double theta, int degree, int sl, int tl, double size_check, int precision) {
    if (nt < 0 || ns < 0) return set_error(TAGI_ERR_ARG, "negative point count (%d targets, %d sources)", nt, ns);
    if (kernel != KERNEL_COULOMB && kernel != KERNEL_YUKAWA)
        return set_error(TAGI_ERR_UNSUPPORTED, "kernel %d not supported (COULOMB=1, YUKAWA=2)", kernel);
    if (sing != SING_NONE && sing != SING_SKIPPING && sing != SING_SUBTRACTION)
        return set_error(TAGI_ERR_UNSUPPORTED, "singularity handling %d not supported", sing);
    if (approx != APPROX_LAGRANGE)
        return set_error(TAGI_ERR_UNSUPPORTED, "approximation %d not supported (LAGRANGE=1)", approx);
    if (ctype != COMPUTE_PARTICLE_CLUSTER)
        return set_error(TAGI_ERR_UNSUPPORTED, "compute type %d not supported (PARTICLE_CLUSTER=1)", ctype);
    if (nkp < 1 || !kp) return set_error(TAGI_ERR_ARG, "kernel needs at least one kernel parameter");
    if (!(theta >= 0.0) || !std::isfinite(theta)) return set_error(TAGI_ERR_ARG, "theta %g must be >= 0", theta);
    if (degree < 1 || degree > MAX_DEGREE)
        return set_error(TAGI_ERR_UNSUPPORTED, "degree %d outside [1, %d]", degree, MAX_DEGREE);
    if (sl < 1 || tl < 1) return set_error(TAGI_ERR_ARG, "leaf sizes must be >= 1 (%d, %d)", sl, tl);
    if (!(size_check >= 0.0)) return set_error(TAGI_ERR_ARG, "sizeCheck %g must be >= 0", size_check);
    if (precision != PREC_MIXED && precision != PREC_FP64)
        return set_error(TAGI_ERR_ARG, "precision %d must be 0 (mixed) or 1 (fp64)", precision);
    return TAGI_OK;
}

int validate_kparam(int kernel, int sing, double k) {
    if (!std::isfinite(k)) return set_error(TAGI_ERR_ARG, "kernel parameter %g is not finite", k);
    if (kernel == KERNEL_YUKAWA && !(k > 0.0))
        return set_error(TAGI_ERR_ARG, "Yukawa parameter k = %g must be > 0", k);
    if (kernel == KERNEL_COULOMB && sing == SING_SUBTRACTION && !(k > 0.0))
        return set_error(TAGI_ERR_ARG, "Coulomb subtraction parameter alpha = %g must be > 0", k);
    return TAGI_OK;
}

namespace {

int default_precision() {
    if (g_precision < 0) {
        const char *e = getenv("TAGI_PRECISION");
        g_precision = (e && (strcmp(e, "mixed") == 0 || strcmp(e, "MIXED") == 0)) ? PREC_MIXED : PREC_FP64;
    }
    return g_precision;
}

void beta_map(double beta, double *theta, int *degree, int *sl, int *tl) {
    double b = beta < 0 ? 0 : (beta > 1 ? 1 : beta);
    *degree = std::min(MAX_DEGREE, std::max(1, (int)std::lround(1.0 + 9.0 * b)));
    *theta = 0.95 - 0.6 * b;
    *sl = 500;
    *tl = 500;
}

__global__ void gather_weights(const double *__restrict__ w, const int *__restrict__ perm, int n,
                               double *__restrict__ w64, float *__restrict__ w32) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v = w[perm[i]];
    w64[i] = v;
    w32[i] = (float)v;
}

// FP32 hi/lo split of each sorted point's coordinates (hi + lo = x to ~2^-48).
__global__ void split_points(const double *__restrict__ x, const double *__restrict__ y,
                             const double *__restrict__ z, int n, float4 *__restrict__ hi,
                             float4 *__restrict__ lo) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v[3] = {x[i], y[i], z[i]};
    float h[3], l[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        h[d] = (float)v[d];
        l[d] = (float)(v[d] - (double)h[d]);
    }
    hi[i] = make_float4(h[0], h[1], h[2], 0.f);
    lo[i] = make_float4(l[0], l[1], l[2], 0.f);
}

// SS term only (no sources): phi_i = f_i * 4pi/k^2 or f_i * 2pi/a^2.
__global__ void ss_only(const double *__restrict__ tv, int nt, double c, double *__restrict__ out) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nt) out[i] = c * tv[i];
}

double ss_constant(int kernel, int sing, double k) {
    if (sing != SING_SUBTRACTION) return 0.0;
    return kernel == KERNEL_YUKAWA ? 4.0 * M_PI / (k * k) : 2.0 * M_PI / (k * k);
}

}  // namespace

int plan_create(Plan **out, int nt, const double *tx, const double *ty, const double *tz, int ns,
                const double *sx, const double *sy, const double *sz, const double *sw,
                double theta, int degree, int sl, int tl, double size_check, cudaStream_t s) {
    *out = nullptr;
    if (nt < 1 || ns < 1) return set_error(TAGI_ERR_ARG, "a plan needs >= 1 target and source (%d, %d)", nt, ns);
    if (!tx || !ty || !tz || !sx || !sy || !sz || !sw) return set_error(TAGI_ERR_ARG, "null device pointer");
    if (degree < 1 || degree > MAX_DEGREE)
        return set_error(TAGI_ERR_UNSUPPORTED, "degree %d outside [1, %d]", degree, MAX_DEGREE);
    if (!(theta >= 0.0) || sl < 1 || tl < 1 || !(size_check >= 0.0))
        return set_error(TAGI_ERR_ARG, "bad tree parameters (theta %g, leaves %d/%d, sizeCheck %g)", theta, sl, tl,
                         size_check);
    Plan *p = new Plan();
    cudaGetDevice(&p->device);
    p->arena.stream = s;
    p->degree = degree;
    p->n1 = degree + 1;
    p->P = p->n1 * p->n1 * p->n1;
    p->theta = theta;
    p->size_check = size_check;
    p->source_leaf = sl;
    p->target_leaf = tl;
    for (int m = 0; m <= MAX_DEGREE; m++) p->cheb[m] = m <= degree ? std::cos(M_PI * (double)m / (double)degree) : 0.0;
    int rc = TAGI_OK;
    do {
        // err_flag[0]: tree/list build; err_flag[1]: kernel parameters a call could not use
        if ((rc = p->arena.alloc(&p->queue, 3)) || (rc = p->arena.alloc(&p->err_flag, 2))) break;
        cudaMemsetAsync(p->err_flag, 0, 2 * sizeof(int), s);
        phase_mark(PH_TREE, true, s);
        if ((rc = build_tree(p->src, sx, sy, sz, ns, sl, p->arena, p->err_flag, s))) break;
        // Green iteration convolves a mesh with itself: same points and leaf size give the
        // same (deterministic) tree, so the target tree shares the source tree's arrays
        const bool same = tx == sx && ty == sy && tz == sz && nt == ns && tl == sl;
        if (same) p->tgt = p->src;
        else if ((rc = build_tree(p->tgt, tx, ty, tz, nt, tl, p->arena, p->err_flag, s))) break;
        phase_mark(PH_TREE, false, s);
        phase_mark(PH_LISTS, true, s);
        if ((rc = p->arena.alloc(&p->sw64, ns)) || (rc = p->arena.alloc(&p->sw32, ns))) break;
        launch(gather_weights, (ns + 255) / 256, 256, 0, s, sw, p->src.perm, ns, p->sw64, p->sw32);
        if ((rc = p->arena.alloc(&p->src_hi, ns)) || (rc = p->arena.alloc(&p->src_lo, ns))) break;
        launch(split_points, (ns + 255) / 256, 256, 0, s, p->src.x, p->src.y, p->src.z, ns, p->src_hi, p->src_lo);
        if (same) {
            p->tgt_hi = p->src_hi;
            p->tgt_lo = p->src_lo;
        } else {
            if ((rc = p->arena.alloc(&p->tgt_hi, nt)) || (rc = p->arena.alloc(&p->tgt_lo, nt))) break;
            launch(split_points, (nt + 255) / 256, 256, 0, s, p->tgt.x, p->tgt.y, p->tgt.z, nt, p->tgt_hi, p->tgt_lo);
        }
        if ((rc = build_lists(*p, s))) break;
        if ((rc = build_weight_charges(*p, s))) break;
        phase_mark(PH_LISTS, false, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) { rc = set_error(TAGI_ERR_CUDA, "plan build: %s", cudaGetErrorString(e)); break; }
    } while (0);
    if (rc) {
        cudaStreamSynchronize(s);
        p->arena.release();
        cudaStreamSynchronize(s);
        delete p;
        return rc;
    }
    *out = p;
    return TAGI_OK;
}

void plan_destroy(Plan *p) {
    if (!p) return;
    cudaDeviceSynchronize();
    for (void *v : p->scratch) cudaFree(v);
    for (Schedule &sc : p->scheds) sc.release();
    for (void *v : p->arena.ptrs) cudaFree(v);
    delete p;
}

// Full call on device arrays (the body of BaryTreeInterface).
int treecode_device(int nt, int ns, const double *tx, const double *ty, const double *tz,
                    const double *tv, const double *sx, const double *sy, const double *sz,
                    const double *sv, const double *sw, double *out, int kernel, int nkp,
                    const double *kp, int sing, int approx, int ctype, double theta, int degree,
                    int sl, int tl, double size_check, double beta, int verbosity, int precision,
                    cudaStream_t s) {
    if (beta >= 0.0) beta_map(beta, &theta, &degree, &sl, &tl);
    TAGI_TRY(validate(nt, ns, kernel, nkp, kp, sing, approx, ctype, theta, degree, sl, tl, size_check,
                      precision));
    TAGI_TRY(validate_kparam(kernel, sing, kp[0]));
    if (nt == 0) return TAGI_OK;
    if (ns == 0) {
        launch(ss_only, (nt + 255) / 256, 256, 0, s, tv, nt, ss_constant(kernel, sing, kp[0]), out);
        TAGI_LAUNCH_CHECK();
        return TAGI_OK;
    }
    double t0 = now_s();
    Plan *p = nullptr;
    TAGI_TRY(plan_create(&p, nt, tx, ty, tz, ns, sx, sy, sz, sw, theta, degree, sl, tl, size_check, s));
    double t1 = now_s();
    int rc = convolve(*p, tv, sv, out, 1, kernel, kp, nkp, sing, precision, s);
    if (!rc && verbosity > 0) {
        cudaStreamSynchronize(s);
        double t2 = now_s();
        fprintf(stderr,
                "[tagi] %d targets, %d sources: plan %.3f s (%d batches, %d near / %d far entries, %d slots), "
                "convolution %.3f s (%.3g near + %.3g far pairs, %s)\n",
                nt, ns, t1 - t0, p->nbatch, p->near_total, p->far_total, p->nslots, t2 - t1, p->near_pairs,
                p->far_pairs, precision == PREC_MIXED ? "mixed" : "fp64");
    }
    plan_destroy(p);
    return rc;
}

}  // namespace tagi

using namespace tagi;

namespace {

// Host-pointer version: copy in, run, copy out, all on the library's stream.
int treecode_host(int nt, int ns, const double *tx, const double *ty, const double *tz,
                  const double *tv, const double *sx, const double *sy, const double *sz,
                  const double *sv, const double *sw, double *out, int kernel, int nkp,
                  const double *kp, int sing, int approx, int ctype, double theta, int degree,
                  int sl, int tl, double size_check, double beta, int verbosity, int precision) {
    if (nt < 0 || ns < 0) return set_error(TAGI_ERR_ARG, "negative point count");
    {  // every argument is checked on the host before any CUDA call
        double th = theta;
        int dg = degree, a = sl, b = tl;
        if (beta >= 0.0) beta_map(beta, &th, &dg, &a, &b);
        TAGI_TRY(validate(nt, ns, kernel, nkp, kp, sing, approx, ctype, th, dg, a, b, size_check, precision));
        TAGI_TRY(validate_kparam(kernel, sing, kp[0]));
    }
    if (nt == 0) return TAGI_OK;
    if (!tx || !ty || !tz || !tv || !out || (ns > 0 && (!sx || !sy || !sz || !sv || !sw)))
        return set_error(TAGI_ERR_ARG, "null host pointer");
    cudaStream_t s = host_stream();
    if (!s) return set_error(TAGI_ERR_CUDA, "no CUDA device or stream: %s", cudaGetErrorString(cudaGetLastError()));
    Arena ar;
    ar.stream = s;
    int rc = TAGI_OK;
    do {
        double *d[10] = {};
        const double *h[9] = {tx, ty, tz, tv, sx, sy, sz, sv, sw};
        const int n[9] = {nt, nt, nt, nt, ns, ns, ns, ns, ns};
        for (int i = 0; i < 9 && !rc; i++) {
            rc = ar.alloc(&d[i], n[i] > 0 ? n[i] : 1);
            if (!rc && n[i] > 0 &&
                cudaMemcpyAsync(d[i], h[i], sizeof(double) * n[i], cudaMemcpyHostToDevice, s) != cudaSuccess)
                rc = set_error(TAGI_ERR_CUDA, "host to device copy failed");
        }
        if (rc) break;
        if ((rc = ar.alloc(&d[9], nt))) break;
        rc = treecode_device(nt, ns, d[0], d[1], d[2], d[3], d[4], d[5], d[6], d[7], d[8], d[9], kernel, nkp,
                             kp, sing, approx, ctype, theta, degree, sl, tl, size_check, beta, verbosity,
                             precision, s);
        if (rc) break;
        if (cudaMemcpyAsync(out, d[9], sizeof(double) * nt, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            rc = set_error(TAGI_ERR_CUDA, "device to host copy failed: %s", cudaGetErrorString(cudaGetLastError()));
    } while (0);
    cudaStreamSynchronize(s);
    ar.release();
    cudaStreamSynchronize(s);
    return rc;
}

}  // namespace

extern "C" {

int tagi_version(void) { return 100; }
int tagi_last_error(void) { return g_err; }
const char *tagi_last_error_message(void) { return g_msg; }
void tagi_clear_error(void) {
    g_err = 0;
    g_msg[0] = 0;
}

int tagi_set_precision(int precision) {
    if (precision != PREC_MIXED && precision != PREC_FP64)
        return set_error(TAGI_ERR_ARG, "precision %d must be 0 (mixed) or 1 (fp64)", precision);
    g_precision = precision;
    return TAGI_OK;
}
int tagi_get_precision(void) { return default_precision(); }

int tagi_beta_parameters(double beta, double *theta, int *degree, int *sl, int *tl) {
    if (!theta || !degree || !sl || !tl) return set_error(TAGI_ERR_ARG, "null pointer");
    beta_map(beta, theta, degree, sl, tl);
    return TAGI_OK;
}

int tagi_orbitals_per_item(int kernel, int precision, int maxOrbitals, int requested, int degree, int *og) {
    if (!og) return set_error(TAGI_ERR_ARG, "null pointer");
    if (requested != 0 && requested != 1 && requested != 4 && requested != 8 && requested != 16)
        return set_error(TAGI_ERR_ARG, "orbitalsPerItem %d must be 0 (automatic), 1, 4, 8 or 16", requested);
    if (maxOrbitals < 1 || degree < 1 || degree > MAX_DEGREE)
        return set_error(TAGI_ERR_ARG, "maxOrbitals %d, degree %d", maxOrbitals, degree);
    *og = orbitals_per_item(kernel, precision, &maxOrbitals, nullptr, 1, requested, degree + 1);
    return TAGI_OK;
}

int tagi_BaryTreeInterface_ex(int numTargets, int numSources, const double *targetX,
                              const double *targetY, const double *targetZ, const double *targetValue,
                              const double *sourceX, const double *sourceY, const double *sourceZ,
                              const double *sourceValue, const double *sourceWeight, double *outputArray,
                              int kernel, int numberOfKernelParameters, const double *kernelParameters,
                              int singularity, int approximation, int computeType, double theta, int degree,
                              int sourceLeafSize, int targetLeafSize, double sizeCheck, double beta,
                              int verbosity, int precision) {
    return treecode_host(numTargets, numSources, targetX, targetY, targetZ, targetValue, sourceX, sourceY,
                         sourceZ, sourceValue, sourceWeight, outputArray, kernel, numberOfKernelParameters,
                         kernelParameters, singularity, approximation, computeType, theta, degree,
                         sourceLeafSize, targetLeafSize, sizeCheck, beta, verbosity, precision);
}

void BaryTreeInterface(int numTargets, int numSources, double *targetX, double *targetY, double *targetZ,
                       double *targetValue, double *sourceX, double *sourceY, double *sourceZ,
                       double *sourceValue, double *sourceWeight, double *outputArray, int kernel,
                       int numberOfKernelParameters, double *kernelParameters, int singularity,
                       int approximation, int computeType, double theta, int degree, int sourceLeafSize,
                       int targetLeafSize, double sizeCheck, double beta, int verbosity) {
    tagi_clear_error();
    int rc = treecode_host(numTargets, numSources, targetX, targetY, targetZ, targetValue, sourceX, sourceY,
                           sourceZ, sourceValue, sourceWeight, outputArray, kernel, numberOfKernelParameters,
                           kernelParameters, singularity, approximation, computeType, theta, degree,
                           sourceLeafSize, targetLeafSize, sizeCheck, beta, verbosity, default_precision());
    if (rc) fprintf(stderr, "BaryTreeInterface (tagi_gb300): error %d: %s\n", rc, g_msg);
}

int tagi_treecode_dev(int numTargets, int numSources, const double *targetX, const double *targetY,
                      const double *targetZ, const double *targetValue, const double *sourceX,
                      const double *sourceY, const double *sourceZ, const double *sourceValue,
                      const double *sourceWeight, double *outputArray, int kernel,
                      int numberOfKernelParameters, const double *kernelParameters, int singularity,
                      int approximation, int computeType, double theta, int degree, int sourceLeafSize,
                      int targetLeafSize, double sizeCheck, double beta, int verbosity, int precision,
                      void *stream) {
    if (numTargets > 0 && (!targetX || !targetY || !targetZ || !targetValue || !outputArray))
        return set_error(TAGI_ERR_ARG, "null device pointer");
    if (numSources > 0 && (!sourceX || !sourceY || !sourceZ || !sourceValue || !sourceWeight))
        return set_error(TAGI_ERR_ARG, "null device pointer");
    return treecode_device(numTargets, numSources, targetX, targetY, targetZ, targetValue, sourceX, sourceY,
                           sourceZ, sourceValue, sourceWeight, outputArray, kernel, numberOfKernelParameters,
                           kernelParameters, singularity, approximation, computeType, theta, degree,
                           sourceLeafSize, targetLeafSize, sizeCheck, beta, verbosity, precision,
                           (cudaStream_t)stream);
}

int tagi_plan_create(tagi_plan **plan, int numTargets, const double *targetX, const double *targetY,
                     const double *targetZ, int numSources, const double *sourceX, const double *sourceY,
                     const double *sourceZ, const double *sourceWeight, double theta, int degree,
                     int sourceLeafSize, int targetLeafSize, double sizeCheck, void *stream) {
    if (!plan) return set_error(TAGI_ERR_ARG, "null plan pointer");
    *plan = nullptr;
    Plan *p = nullptr;
    int rc = plan_create(&p, numTargets, targetX, targetY, targetZ, numSources, sourceX, sourceY, sourceZ,
                         sourceWeight, theta, degree, sourceLeafSize, targetLeafSize, sizeCheck,
                         (cudaStream_t)stream);
    if (rc) return rc;
    *plan = reinterpret_cast<tagi_plan *>(p);  // opaque handle
    return TAGI_OK;
}

int tagi_plan_destroy(tagi_plan *plan) {
    plan_destroy(reinterpret_cast<Plan *>(plan));
    return TAGI_OK;
}

int tagi_plan_convolve(tagi_plan *plan, int numOrbitals, const double *targetValues,
                       const double *sourceValues, double *output, int kernel, int numberOfKernelParameters,
                       const double *kernelParameters, int singularity, int precision, void *stream) {
    if (!plan) return set_error(TAGI_ERR_ARG, "null plan");
    Plan &p = *reinterpret_cast<Plan *>(plan);
    if (numOrbitals < 1) return set_error(TAGI_ERR_ARG, "numOrbitals %d must be >= 1", numOrbitals);
    if (!targetValues || !sourceValues || !output) return set_error(TAGI_ERR_ARG, "null device pointer");
    TAGI_TRY(validate(p.tgt.n, p.src.n, kernel, numberOfKernelParameters, kernelParameters, singularity,
                      APPROX_LAGRANGE, COMPUTE_PARTICLE_CLUSTER, p.theta, p.degree, p.source_leaf,
                      p.target_leaf, p.size_check, precision));
    for (int o = 0; o < numOrbitals; o++)
        TAGI_TRY(validate_kparam(kernel, singularity, kernelParameters[(long)o * numberOfKernelParameters]));
    return convolve(p, targetValues, sourceValues, output, numOrbitals, kernel, kernelParameters,
                    numberOfKernelParameters, singularity, precision, (cudaStream_t)stream);
}

int tagi_plan_info(const tagi_plan *plan, double *info) {
    if (!plan || !info) return set_error(TAGI_ERR_ARG, "null pointer");
    const Plan &p = *reinterpret_cast<const Plan *>(plan);
    double v[13] = {(double)p.src.nnodes, (double)p.tgt.nnodes, (double)p.nbatch, (double)p.near_total,
                    (double)p.far_total, (double)p.nslots, (double)p.P, (double)p.nitems,
                    (double)p.rng_total, (double)p.max_batch, p.near_pairs, p.far_pairs,
                    p.near_close_pairs};
    memcpy(info, v, sizeof(v));
    return TAGI_OK;
}

int tagi_plan_get_tree(const tagi_plan *plan, int which, uint64_t *codes, int *perm, int *begin, int *end,
                       int *parent, int *first_child, int *nchild, double *center, double *half,
                       double *radius) {
    if (!plan) return set_error(TAGI_ERR_ARG, "null plan");
    const Plan &p = *reinterpret_cast<const Plan *>(plan);
    const Tree &t = which ? p.tgt : p.src;
    const size_t n = t.n, nn = t.nnodes;
    TAGI_CUDA(cudaDeviceSynchronize());
    TAGI_CUDA(cudaMemcpy(codes, t.codes, 8 * n, cudaMemcpyDeviceToHost));
    TAGI_CUDA(cudaMemcpy(perm, t.perm, 4 * n, cudaMemcpyDeviceToHost));
    TAGI_CUDA(cudaMemcpy(begin, t.begin, 4 * nn, cudaMemcpyDeviceToHost));
    TAGI_CUDA(cudaMemcpy(end, t.end, 4 * nn, cudaMemcpyDeviceToHost));
    TAGI_CUDA(cudaMemcpy(parent, t.parent, 4 * nn, cudaMemcpyDeviceToHost));
    TAGI_CUDA(cudaMemcpy(first_child, t.first_child, 4 * nn, cudaMemcpyDeviceToHost));
    TAGI_CUDA(cudaMemcpy(nchild, t.nchild, 4 * nn, cudaMemcpyDeviceToHost));
    TAGI_CUDA(cudaMemcpy(center, t.center, 24 * nn, cudaMemcpyDeviceToHost));
    TAGI_CUDA(cudaMemcpy(half, t.half, 24 * nn, cudaMemcpyDeviceToHost));
    TAGI_CUDA(cudaMemcpy(radius, t.radius, 8 * nn, cudaMemcpyDeviceToHost));
    return TAGI_OK;
}

int tagi_plan_get_lists(const tagi_plan *plan, int *batch_node, int *near_off, int *near_list, int *far_off,
                        int *far_list, int *slot_node) {
    if (!plan) return set_error(TAGI_ERR_ARG, "null plan");
    const Plan &p = *reinterpret_cast<const Plan *>(plan);
    TAGI_CUDA(cudaDeviceSynchronize());
    TAGI_CUDA(cudaMemcpy(batch_node, p.batch_node, 4L * p.nbatch, cudaMemcpyDeviceToHost));
    TAGI_CUDA(cudaMemcpy(near_off, p.near_off, 4L * (p.nbatch + 1), cudaMemcpyDeviceToHost));
    TAGI_CUDA(cudaMemcpy(far_off, p.far_off, 4L * (p.nbatch + 1), cudaMemcpyDeviceToHost));
    if (p.near_total) TAGI_CUDA(cudaMemcpy(near_list, p.near_list, 4L * p.near_total, cudaMemcpyDeviceToHost));
    if (p.far_total) TAGI_CUDA(cudaMemcpy(far_list, p.far_list, 4L * p.far_total, cudaMemcpyDeviceToHost));
    if (p.nslots) TAGI_CUDA(cudaMemcpy(slot_node, p.slot_node, 4L * p.nslots, cudaMemcpyDeviceToHost));
    return TAGI_OK;
}

int tagi_plan_get_charges(tagi_plan *plan, int which, int numOrbitals, double *out) {
    if (!plan || !out) return set_error(TAGI_ERR_ARG, "null pointer");
    Plan &p = *reinterpret_cast<Plan *>(plan);
    const size_t per = (size_t)p.nslots * p.P;
    TAGI_CUDA(cudaDeviceSynchronize());
    if (which == 0) {
        TAGI_TRY(ensure_weight_charges64(p, p.arena.stream));
        TAGI_CUDA(cudaDeviceSynchronize());
        TAGI_CUDA(cudaMemcpy(out, p.what64, 8 * per, cudaMemcpyDeviceToHost));
        return TAGI_OK;
    }
    if (which == 3) {
        std::vector<float> tmp(per);
        TAGI_CUDA(cudaMemcpy(tmp.data(), p.what32, 4 * per, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < per; i++) out[i] = tmp[i];
        return TAGI_OK;
    }
    if ((size_t)numOrbitals > p.scratch_orbitals) return set_error(TAGI_ERR_ARG, "no charges for %d orbitals", numOrbitals);
    if (which == 1) {
        TAGI_CUDA(cudaMemcpy(out, p.qhat64, 8 * per * numOrbitals, cudaMemcpyDeviceToHost));
    } else {
        std::vector<float> tmp(per * numOrbitals);
        TAGI_CUDA(cudaMemcpy(tmp.data(), p.qhat32, 4 * per * numOrbitals, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < tmp.size(); i++) out[i] = tmp[i];
    }
    return TAGI_OK;
}

int tagi_direct_dev(int numTargets, const double *targetX, const double *targetY, const double *targetZ,
                    const double *targetValue, int numSubset, const int *subset, int numSources,
                    const double *sourceX, const double *sourceY, const double *sourceZ,
                    const double *sourceValue, const double *sourceWeight, double *output, int kernel,
                    const double *kernelParameters, int singularity, void *stream) {
    if (!kernelParameters) return set_error(TAGI_ERR_ARG, "null kernelParameters");
    TAGI_TRY(validate(numTargets, numSources, kernel, 1, kernelParameters, singularity, APPROX_LAGRANGE,
                      COMPUTE_PARTICLE_CLUSTER, 0.0, 1, 1, 1, 1.0, PREC_FP64));
    TAGI_TRY(validate_kparam(kernel, singularity, kernelParameters[0]));
    if (numSubset < 0) return set_error(TAGI_ERR_ARG, "negative subset size");
    int nsub = subset ? numSubset : numTargets;
    return direct_sum(numTargets, targetX, targetY, targetZ, targetValue, nsub, subset, numSources, sourceX,
                      sourceY, sourceZ, sourceValue, sourceWeight, output, kernel, kernelParameters[0],
                      singularity, PREC_FP64, (cudaStream_t)stream);
}

int tagi_pair_peak(int kernel, int singularity, int variant, double kernelParameter, double *pairsPerSecond,
                   void *stream) {
    if (!pairsPerSecond) return set_error(TAGI_ERR_ARG, "null output");
    if (kernel != KERNEL_COULOMB && kernel != KERNEL_YUKAWA) return set_error(TAGI_ERR_UNSUPPORTED, "kernel %d", kernel);
    if (variant < 0 || variant > 5)
        return set_error(TAGI_ERR_ARG,
                         "variant must be 0 (near), 1 (far), 2/3 (near/far, groups of 8 orbitals) or 4/5 "
                         "(near/far, groups of 16)");
    return pair_peak(kernel, singularity, variant, kernelParameter, pairsPerSecond, (cudaStream_t)stream);
}

int tagi_mgs_dev(double *V, double *U, const double *W, int targetWavefunction, int numPoints,
                 int numWavefunctions, void *stream) {
    if (numPoints < 0 || numWavefunctions < 1) return set_error(TAGI_ERR_ARG, "bad MGS sizes");
    if (numPoints > 0 && (!V || !U || !W)) return set_error(TAGI_ERR_ARG, "null device pointer");
    return mgs_device(V, U, W, targetWavefunction, numPoints, numWavefunctions, (cudaStream_t)stream);
}

int tagi_interp_dev(const double *coarseX, const double *coarseY, const double *coarseZ, const double *coarseF,
                    const int *pointsPerCell_coarse, int coarseN, const double *fineX, const double *fineY,
                    const double *fineZ, double *fineF, const int *pointsPerCell_fine, int fineN,
                    int numberOfCells, int cellOrder, void *stream) {
    if (coarseN < 0 || fineN < 0 || numberOfCells < 0) return set_error(TAGI_ERR_ARG, "negative size");
    return interp_device(coarseX, coarseY, coarseZ, coarseF, pointsPerCell_coarse, coarseN, fineX, fineY, fineZ,
                         fineF, pointsPerCell_fine, fineN, numberOfCells, cellOrder, nullptr, nullptr,
                         (cudaStream_t)stream);
}

void modifiedGramSchmidt_singleWavefunction(double *V, double *U, double *W, int targetWavefunction,
                                            int numPoints, int numWavefunctions) {
    tagi_clear_error();
    int rc = TAGI_OK;
    if (numPoints < 0 || numWavefunctions < 1 || targetWavefunction < 0 || targetWavefunction >= numWavefunctions)
        rc = set_error(TAGI_ERR_ARG, "bad MGS arguments (target %d, %d points, %d wavefunctions)", targetWavefunction,
                       numPoints, numWavefunctions);
    cudaStream_t s = rc ? nullptr : host_stream();
    if (!rc && !s) rc = set_error(TAGI_ERR_CUDA, "no CUDA device");
    Arena ar;
    ar.stream = s;
    if (!rc && numPoints > 0) {
        const size_t n = numPoints, rows = (size_t)targetWavefunction + 1;
        double *dV = nullptr, *dU = nullptr, *dW = nullptr;
        if (!(rc = ar.alloc(&dV, rows * n)) && !(rc = ar.alloc(&dU, n)) && !(rc = ar.alloc(&dW, n))) {
            if (cudaMemcpyAsync(dV, V, 8 * rows * n, cudaMemcpyHostToDevice, s) ||
                cudaMemcpyAsync(dU, U, 8 * n, cudaMemcpyHostToDevice, s) ||
                cudaMemcpyAsync(dW, W, 8 * n, cudaMemcpyHostToDevice, s))
                rc = set_error(TAGI_ERR_CUDA, "MGS host to device copy failed");
            if (!rc) rc = mgs_device(dV, dU, dW, targetWavefunction, numPoints, (int)rows, s);
            if (!rc && (cudaMemcpyAsync(U, dU, 8 * n, cudaMemcpyDeviceToHost, s) ||
                        cudaMemcpyAsync(V + (size_t)targetWavefunction * n, dV + (size_t)targetWavefunction * n,
                                        8 * n, cudaMemcpyDeviceToHost, s) ||
                        cudaStreamSynchronize(s)))
                rc = set_error(TAGI_ERR_CUDA, "MGS device to host copy failed");
        }
        cudaStreamSynchronize(s);
        ar.release();
        cudaStreamSynchronize(s);
    }
    if (rc) fprintf(stderr, "modifiedGramSchmidt_singleWavefunction (tagi_gb300): error %d: %s\n", rc, g_msg);
}

void InterpolateBetweenTwoMeshes(double *coarseX, double *coarseY, double *coarseZ, double *coarseF,
                                 int *pointsPerCell_coarse, int coarseN, double *fineX, double *fineY,
                                 double *fineZ, double *fineF, int *pointsPerCell_fine, int fineN,
                                 int numberOfCells, int cellOrder) {
    tagi_clear_error();
    int rc = TAGI_OK;
    if (coarseN < 0 || fineN < 0 || numberOfCells < 0) rc = set_error(TAGI_ERR_ARG, "negative size");
    if (!rc && coarseN == fineN) {  // TwoMeshInterpolation.c:175-180
        for (int i = 0; i < coarseN; i++) fineF[i] = coarseF[i];
        return;
    }
    if (!rc) {  // the cell counts must fit the arrays (TwoMeshInterpolation.c walks them unchecked)
        long sc = 0, sf = 0;
        for (int c = 0; c < numberOfCells; c++) {
            sc += pointsPerCell_coarse[c];
            sf += pointsPerCell_fine[c];
        }
        if (sc > coarseN || sf > fineN)
            rc = set_error(TAGI_ERR_ARG, "points per cell sum to %ld / %ld, arrays hold %d / %d", sc, sf, coarseN,
                           fineN);
    }
    cudaStream_t s = rc ? nullptr : host_stream();
    if (!rc && !s) rc = set_error(TAGI_ERR_CUDA, "no CUDA device");
    if (!rc) {
        Arena ar;
        ar.stream = s;
        double *d[8] = {};
        int *pc = nullptr, *pf = nullptr;
        const double *h[8] = {coarseX, coarseY, coarseZ, coarseF, fineX, fineY, fineZ, fineF};
        const int n[8] = {coarseN, coarseN, coarseN, coarseN, fineN, fineN, fineN, fineN};
        for (int i = 0; i < 8 && !rc; i++) {
            rc = ar.alloc(&d[i], n[i] > 0 ? n[i] : 1);
            if (!rc && n[i] > 0 && cudaMemcpyAsync(d[i], h[i], 8L * n[i], cudaMemcpyHostToDevice, s))
                rc = set_error(TAGI_ERR_CUDA, "interpolation host to device copy failed");
        }
        if (!rc && !(rc = ar.alloc(&pc, numberOfCells + 1)) && !(rc = ar.alloc(&pf, numberOfCells + 1))) {
            if (numberOfCells > 0 &&
                (cudaMemcpyAsync(pc, pointsPerCell_coarse, 4L * numberOfCells, cudaMemcpyHostToDevice, s) ||
                 cudaMemcpyAsync(pf, pointsPerCell_fine, 4L * numberOfCells, cudaMemcpyHostToDevice, s)))
                rc = set_error(TAGI_ERR_CUDA, "interpolation host to device copy failed");
            if (!rc)
                rc = interp_device(d[0], d[1], d[2], d[3], pc, coarseN, d[4], d[5], d[6], d[7], pf, fineN,
                                   numberOfCells, cellOrder, pointsPerCell_coarse, pointsPerCell_fine, s);
            if (!rc && fineN > 0 &&
                (cudaMemcpyAsync(fineF, d[7], 8L * fineN, cudaMemcpyDeviceToHost, s) || cudaStreamSynchronize(s)))
                rc = set_error(TAGI_ERR_CUDA, "interpolation device to host copy failed");
        }
        cudaStreamSynchronize(s);
        ar.release();
        cudaStreamSynchronize(s);
    }
    if (rc) fprintf(stderr, "InterpolateBetweenTwoMeshes (tagi_gb300): error %d: %s\n", rc, g_msg);
}

}  // extern "C"
