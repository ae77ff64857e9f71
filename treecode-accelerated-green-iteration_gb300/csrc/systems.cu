// Batched calls: many orbitals of one mesh, several meshes ("systems") in one
// persistent launch per field pass, kernel parameters read from device
// memory, and CUDA-graph capture of a call sequence.
//
// The reference convolves one orbital per BaryTreeInterface call
// (3D-GreenIteration/src/greenIterationFixedPoint.py:314-324, one call per
// orbital per Green-iteration sweep).  Here all orbitals of all systems of a
// sweep share one launch of each field kernel; a sweep's launches can be
// captured once and replayed (tagi_graph_*), with the orbital energies (hence
// the Yukawa parameters k_i) updated in device memory between replays.
#include "tagi_internal.h"

#include <vector>

namespace tagi {

namespace {

struct Systems {
    std::vector<Plan *> plans;  // borrowed
    std::vector<int> norb;
    int kernel = KERNEL_YUKAWA, precision = PREC_MIXED;
    int nt_request = 0;  // targets per thread: 0 automatic, 1 or 2
    Schedule sched;
    int *queue = nullptr;  // 3 work counters
    cudaStream_t stream = nullptr;
};

struct Graph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

// Validation of a host kernel-parameter array for norb orbitals.
int check_kparams(int kernel, int sing, int norb, int nkp, const double *kp) {
    if (nkp < 1 || !kp) return set_error(TAGI_ERR_ARG, "kernel needs at least one kernel parameter per orbital");
    for (int o = 0; o < norb; o++) TAGI_TRY(validate_kparam(kernel, sing, kp[(long)o * nkp]));
    return TAGI_OK;
}

int check_call(int kernel, int sing, int precision) {
    // validate() wants a parameter array; the parameters are checked separately
    const double one = 1.0;
    return validate(1, 1, kernel, 1, &one, sing, APPROX_LAGRANGE, COMPUTE_PARTICLE_CLUSTER, 0.7, 1, 1, 1, 1.0,
                    precision);
}

}  // namespace

}  // namespace tagi

using namespace tagi;

extern "C" {

int tagi_plan_convolve_ex(tagi_plan *plan, int numOrbitals, const double *targetValues, const double *sourceValues,
                          double *output, int kernel, int numberOfKernelParameters, const double *kernelParameters,
                          int kernelParametersOnDevice, int singularity, int precision, int orbitalsPerItem,
                          int targetsPerThread, void *stream) {
    if (!plan) return set_error(TAGI_ERR_ARG, "null plan");
    Plan &p = *reinterpret_cast<Plan *>(plan);
    if (numOrbitals < 1 || numOrbitals > 0xffff)
        return set_error(TAGI_ERR_ARG, "numOrbitals %d outside [1, 65535]", numOrbitals);
    if (!targetValues || !sourceValues || !output) return set_error(TAGI_ERR_ARG, "null device pointer");
    if (orbitalsPerItem != 0 && orbitalsPerItem != 1 && orbitalsPerItem != 4 && orbitalsPerItem != 8 &&
        orbitalsPerItem != 16)
        return set_error(TAGI_ERR_ARG, "orbitalsPerItem %d must be 0 (automatic), 1, 4, 8 or 16", orbitalsPerItem);
    if (targetsPerThread < 0 || targetsPerThread > 2)
        return set_error(TAGI_ERR_ARG, "targetsPerThread %d must be 0 (automatic), 1 or 2", targetsPerThread);
    TAGI_TRY(check_call(kernel, singularity, precision));
    if (kernelParametersOnDevice) {
        if (!kernelParameters || numberOfKernelParameters < 1)
            return set_error(TAGI_ERR_ARG, "kernel needs at least one kernel parameter per orbital");
    } else {
        TAGI_TRY(check_kparams(kernel, singularity, numOrbitals, numberOfKernelParameters, kernelParameters));
    }
    return convolve(p, targetValues, sourceValues, output, numOrbitals, kernel, kernelParameters,
                    numberOfKernelParameters, singularity, precision, (cudaStream_t)stream,
                    kernelParametersOnDevice != 0, orbitalsPerItem, targetsPerThread);
}

int tagi_plan_check_parameters(tagi_plan *plan, int *flags, void *stream) {
    if (!plan || !flags) return set_error(TAGI_ERR_ARG, "null pointer");
    Plan &p = *reinterpret_cast<Plan *>(plan);
    cudaStream_t s = (cudaStream_t)stream;
    TAGI_CUDA(cudaMemcpyAsync(flags, p.err_flag + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
    TAGI_CUDA(cudaStreamSynchronize(s));
    TAGI_CUDA(cudaMemsetAsync(p.err_flag + 1, 0, sizeof(int), s));
    return TAGI_OK;
}

int tagi_systems_create(tagi_systems **systems, int numSystems, tagi_plan *const *plans, const int *numOrbitals,
                        int kernel, int precision, int orbitalsPerItem, int targetsPerThread, void *stream) {
    if (!systems) return set_error(TAGI_ERR_ARG, "null systems pointer");
    *systems = nullptr;
    if (numSystems < 1 || numSystems > MAX_SYSTEMS)
        return set_error(TAGI_ERR_ARG, "numSystems %d outside [1, %d]", numSystems, MAX_SYSTEMS);
    if (!plans || !numOrbitals) return set_error(TAGI_ERR_ARG, "null plans or numOrbitals");
    if (orbitalsPerItem != 0 && orbitalsPerItem != 1 && orbitalsPerItem != 4 && orbitalsPerItem != 8 &&
        orbitalsPerItem != 16)
        return set_error(TAGI_ERR_ARG, "orbitalsPerItem %d must be 0 (automatic), 1, 4, 8 or 16", orbitalsPerItem);
    if (targetsPerThread < 0 || targetsPerThread > 2)
        return set_error(TAGI_ERR_ARG, "targetsPerThread %d must be 0 (automatic), 1 or 2", targetsPerThread);
    TAGI_TRY(check_call(kernel, SING_SUBTRACTION, precision));
    int maxo = 0;
    for (int i = 0; i < numSystems; i++) {
        if (!plans[i]) return set_error(TAGI_ERR_ARG, "system %d: null plan", i);
        if (numOrbitals[i] < 1 || numOrbitals[i] > 0xffff)
            return set_error(TAGI_ERR_ARG, "system %d: numOrbitals %d outside [1, 65535]", i, numOrbitals[i]);
        maxo = numOrbitals[i] > maxo ? numOrbitals[i] : maxo;
    }
    Systems *y = new Systems();
    y->stream = (cudaStream_t)stream;
    y->kernel = kernel;
    y->precision = precision;
    y->nt_request = targetsPerThread;
    for (int i = 0; i < numSystems; i++) {
        y->plans.push_back(reinterpret_cast<Plan *>(plans[i]));
        y->norb.push_back(numOrbitals[i]);
    }
    int maxn1 = 0;
    std::vector<double> wt;
    for (Plan *q : y->plans) {
        maxn1 = q->n1 > maxn1 ? q->n1 : maxn1;
        wt.push_back((double)q->src.n);
    }
    const int og = orbitals_per_item(kernel, precision, y->norb.data(), wt.data(), numSystems, orbitalsPerItem, maxn1);
    int rc = build_schedule(y->plans.data(), y->norb.data(), numSystems, og, y->sched, y->stream);
    if (!rc) {
        void *v = nullptr;
        if (cudaMalloc(&v, 3 * sizeof(int)) != cudaSuccess)
            rc = set_error(TAGI_ERR_CUDA, "work counter allocation failed");
        y->queue = static_cast<int *>(v);
    }
    // scratch for every system now, so later calls can be captured
    for (int i = 0; !rc && i < numSystems; i++) rc = ensure_scratch(*y->plans[i], y->norb[i]);
    if (!rc && cudaStreamSynchronize(y->stream) != cudaSuccess) rc = set_error(TAGI_ERR_CUDA, "systems setup failed");
    if (rc) {
        cudaStreamSynchronize(y->stream);
        y->sched.release();
        if (y->queue) cudaFree(y->queue);
        delete y;
        return rc;
    }
    *systems = reinterpret_cast<tagi_systems *>(y);
    return TAGI_OK;
}

int tagi_systems_info(const tagi_systems *systems, int *info) {
    if (!systems || !info) return set_error(TAGI_ERR_ARG, "null pointer");
    const Systems &y = *reinterpret_cast<const Systems *>(systems);
    info[0] = (int)y.plans.size();
    info[1] = y.sched.og;
    info[2] = y.sched.count[0];
    info[3] = y.sched.count[1];
    info[4] = y.sched.count[2];
    return TAGI_OK;
}

int tagi_systems_convolve(tagi_systems *systems, const double *const *targetValues,
                          const double *const *sourceValues, double *const *outputs, int numberOfKernelParameters,
                          const double *const *kernelParameters, int kernelParametersOnDevice, int singularity,
                          void *stream) {
    if (!systems) return set_error(TAGI_ERR_ARG, "null systems");
    Systems &y = *reinterpret_cast<Systems *>(systems);
    if (!targetValues || !sourceValues || !outputs || !kernelParameters)
        return set_error(TAGI_ERR_ARG, "null pointer array");
    TAGI_TRY(check_call(y.kernel, singularity, y.precision));
    const int n = (int)y.plans.size();
    SysCall calls[MAX_SYSTEMS];
    for (int i = 0; i < n; i++) {
        if (!targetValues[i] || !sourceValues[i] || !outputs[i] || !kernelParameters[i])
            return set_error(TAGI_ERR_ARG, "system %d: null pointer", i);
        if (kernelParametersOnDevice) {
            if (numberOfKernelParameters < 1) return set_error(TAGI_ERR_ARG, "numberOfKernelParameters < 1");
        } else {
            TAGI_TRY(check_kparams(y.kernel, singularity, y.norb[i], numberOfKernelParameters, kernelParameters[i]));
        }
        calls[i].p = y.plans[i];
        calls[i].tv = targetValues[i];
        calls[i].sv = sourceValues[i];
        calls[i].out = outputs[i];
        calls[i].norb = y.norb[i];
        calls[i].kp = kernelParameters[i];
        calls[i].nkp = numberOfKernelParameters;
        calls[i].kp_device = kernelParametersOnDevice != 0;
    }
    return convolve_systems(calls, n, y.kernel, singularity, y.precision, y.sched, y.queue, (cudaStream_t)stream,
                            y.nt_request);
}

int tagi_systems_destroy(tagi_systems *systems) {
    if (!systems) return TAGI_OK;
    Systems *y = reinterpret_cast<Systems *>(systems);
    cudaDeviceSynchronize();
    if (y->sched.items) cudaFree(y->sched.items);
    if (y->queue) cudaFree(y->queue);
    delete y;
    return TAGI_OK;
}

int tagi_treecode_batched(int numSystems, const int *pointOffsets, const int *numOrbitals, const double *x,
                          const double *y, const double *z, const double *w, const double *values, double *output,
                          int kernel, const double *kernelParameters, int singularity, double theta, int degree,
                          int sourceLeafSize, int targetLeafSize, double sizeCheck, int precision, void *stream) {
    if (numSystems < 1) return set_error(TAGI_ERR_ARG, "numSystems %d < 1", numSystems);
    if (!pointOffsets || !numOrbitals || !x || !y || !z || !w || !values || !output || !kernelParameters)
        return set_error(TAGI_ERR_ARG, "null pointer");
    cudaStream_t s = (cudaStream_t)stream;
    long korb = 0;
    for (int i = 0; i < numSystems; i++) {
        const int n = pointOffsets[i + 1] - pointOffsets[i];
        if (pointOffsets[i] < 0 || n < 1) return set_error(TAGI_ERR_ARG, "system %d: %d points", i, n);
        TAGI_TRY(validate(n, n, kernel, 1, kernelParameters + korb, singularity, APPROX_LAGRANGE,
                          COMPUTE_PARTICLE_CLUSTER, theta, degree, sourceLeafSize, targetLeafSize, sizeCheck,
                          precision));
        if (numOrbitals[i] < 1 || numOrbitals[i] > 0xffff)
            return set_error(TAGI_ERR_ARG, "system %d: numOrbitals %d outside [1, 65535]", i, numOrbitals[i]);
        TAGI_TRY(check_kparams(kernel, singularity, numOrbitals[i], 1, kernelParameters + korb));
        korb += numOrbitals[i];
    }
    int rc = TAGI_OK;
    long voff = 0;
    korb = 0;
    for (int c0 = 0; c0 < numSystems && !rc; c0 += MAX_SYSTEMS) {
        const int nc = numSystems - c0 < MAX_SYSTEMS ? numSystems - c0 : MAX_SYSTEMS;
        tagi_plan *plans[MAX_SYSTEMS] = {};
        const double *tv[MAX_SYSTEMS], *kp[MAX_SYSTEMS];
        double *out[MAX_SYSTEMS];
        for (int i = 0; i < nc && !rc; i++) {
            const int sid = c0 + i, o = pointOffsets[sid], n = pointOffsets[sid + 1] - o;
            Plan *p = nullptr;
            rc = plan_create(&p, n, x + o, y + o, z + o, n, x + o, y + o, z + o, w + o, theta, degree, sourceLeafSize,
                             targetLeafSize, sizeCheck, s);
            plans[i] = reinterpret_cast<tagi_plan *>(p);
            tv[i] = values + voff;
            out[i] = output + voff;
            kp[i] = kernelParameters + korb;
            voff += (long)numOrbitals[sid] * n;
            korb += numOrbitals[sid];
        }
        tagi_systems *sys = nullptr;
        if (!rc) rc = tagi_systems_create(&sys, nc, plans, numOrbitals + c0, kernel, precision, 0, 0, stream);
        if (!rc) rc = tagi_systems_convolve(sys, tv, tv, out, 1, kp, 0, singularity, stream);
        if (!rc && cudaStreamSynchronize(s) != cudaSuccess) rc = set_error(TAGI_ERR_CUDA, "batched convolution failed");
        tagi_systems_destroy(sys);
        for (int i = 0; i < nc; i++) plan_destroy(reinterpret_cast<Plan *>(plans[i]));
    }
    return rc;
}

// Stream capture of any sequence of this library's calls (and the caller's
// own kernels) into a replayable CUDA graph.  Calls made under capture must
// not allocate: make each call once uncaptured first (the plan keeps its
// scratch and work lists), and pass kernel parameters on the device.
int tagi_graph_begin(void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    if (!s) return set_error(TAGI_ERR_ARG, "graph capture needs a created stream, not the default stream");
    TAGI_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    return TAGI_OK;
}

int tagi_graph_end(void *stream, tagi_graph **graph) {
    if (!graph) return set_error(TAGI_ERR_ARG, "null graph pointer");
    *graph = nullptr;
    cudaStream_t s = (cudaStream_t)stream;
    Graph *g = new Graph();
    cudaError_t e = cudaStreamEndCapture(s, &g->graph);
    if (e != cudaSuccess || !g->graph) {
        if (g->graph) cudaGraphDestroy(g->graph);
        delete g;
        return set_error(TAGI_ERR_CUDA, "stream capture failed: %s", cudaGetErrorString(e));
    }
    e = cudaGraphInstantiate(&g->exec, g->graph, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g->graph);
        delete g;
        return set_error(TAGI_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(e));
    }
    *graph = reinterpret_cast<tagi_graph *>(g);
    return TAGI_OK;
}

int tagi_graph_launch(tagi_graph *graph, void *stream) {
    if (!graph) return set_error(TAGI_ERR_ARG, "null graph");
    Graph *g = reinterpret_cast<Graph *>(graph);
    TAGI_CUDA(cudaGraphLaunch(g->exec, (cudaStream_t)stream));
    return TAGI_OK;
}

int tagi_graph_nodes(const tagi_graph *graph, int *numNodes) {
    if (!graph || !numNodes) return set_error(TAGI_ERR_ARG, "null pointer");
    const Graph *g = reinterpret_cast<const Graph *>(graph);
    size_t n = 0;
    TAGI_CUDA(cudaGraphGetNodes(g->graph, nullptr, &n));
    *numNodes = (int)n;
    return TAGI_OK;
}

int tagi_graph_destroy(tagi_graph *graph) {
    if (!graph) return TAGI_OK;
    Graph *g = reinterpret_cast<Graph *>(graph);
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
    return TAGI_OK;
}

}  // extern "C"
