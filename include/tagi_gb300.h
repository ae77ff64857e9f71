/*
 * tagi_gb300.h -- C ABI of libtagi_gb300.so, the GB300 (sm_103a) treecode
 * convolution path of Treecode-Accelerated Green Iteration.
 *
 * Three groups of entry points:
 *
 *  1. Drop-ins with the exact signatures the reference binds through ctypes
 *     (host pointers, copies in and out inside the call).
 *  2. Device-pointer entry points (pointers from cudaMalloc or torch tensors,
 *     a cudaStream_t passed as void*), including the reusable plan that keeps
 *     the tree and lists resident across Green-iteration steps.
 *  3. Error reporting.  Nothing in this library calls exit(); every failure
 *     sets a thread-local code and message.
 *
 * Enum values (kernel, singularity, approximation, compute type) are those of
 * 3D-GreenIteration/src/utilities/BaryTreeInterface.py:20-46:
 *   kernel         COULOMB = 1, YUKAWA = 2
 *   singularity    NO_SINGULARITY = 0, SKIPPING = 1, SUBTRACTION = 2
 *   approximation  LAGRANGE = 1
 *   computeType    PARTICLE_CLUSTER = 1
 * Supported: COULOMB/YUKAWA, all three singularity modes (NO_SINGULARITY is
 * treated as SKIPPING: coincident pairs are left out), LAGRANGE,
 * PARTICLE_CLUSTER, degree 1..10.  Anything else returns TAGI_ERR_UNSUPPORTED.
 *
 * Kernel parameters: COULOMB and YUKAWA read kernelParameters[0] (k for
 * Yukawa, the Gaussian exponent alpha for Coulomb subtraction) and accept
 * numberOfKernelParameters >= 1; further values are ignored.  TAGI's
 * regularize=True call form passes Kernel.YUKAWA with two parameters [k,
 * epsilon] (greenIterationFixedPoint.py:223-227, scfFixedPoint.py:246-250,
 * where the caller itself warns if epsilon != 0): that call gives exactly the
 * one-parameter result.  REGULARIZED_COULOMB / REGULARIZED_YUKAWA (kernel 3 /
 * 4), the kernels that would use epsilon, return TAGI_ERR_UNSUPPORTED.
 *
 * Precision: TAGI_PREC_MIXED (FP32 pair sums with compensated accumulation,
 * FP64 singularity term) or TAGI_PREC_FP64.
 */
#ifndef TAGI_GB300_H
#define TAGI_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    TAGI_OK = 0,
    TAGI_ERR_ARG = 1,
    TAGI_ERR_CUDA = 2,
    TAGI_ERR_UNSUPPORTED = 3,
    TAGI_ERR_DEVICE = 4,
    TAGI_ERR_STATE = 5  /* call order: e.g. a capture before the first uncaptured call */
};
enum { TAGI_PREC_MIXED = 0, TAGI_PREC_FP64 = 1 };

/* ---------------------------------------------------------------------- */
/* 1. Drop-ins (host pointers).                                            */
/* ---------------------------------------------------------------------- */

/* Replaces BaryTree's BaryTreeInterface as bound in
 * 3D-GreenIteration/src/utilities/BaryTreeInterface.py:67-72 (argtypes) and
 * called at :140-145.  Same argument order and meaning; outputArray receives
 * the convolution (overwritten).  If beta >= 0 it selects theta, degree and
 * leaf sizes (project-defined map, see tagi_beta_parameters).  Precision is
 * the library default (tagi_set_precision; TAGI_PREC_FP64 unless the
 * environment variable TAGI_PRECISION=mixed is set).  Errors: prints one line
 * to stderr and sets tagi_last_error(); never exits. */
void BaryTreeInterface(int numTargets, int numSources, double *targetX, double *targetY,
                       double *targetZ, double *targetValue, double *sourceX, double *sourceY,
                       double *sourceZ, double *sourceValue, double *sourceWeight,
                       double *outputArray, int kernel, int numberOfKernelParameters,
                       double *kernelParameters, int singularity, int approximation,
                       int computeType, double theta, int degree, int sourceLeafSize,
                       int targetLeafSize, double sizeCheck, double beta, int verbosity);

/* BaryTreeInterface with an explicit precision and a status return. */
int tagi_BaryTreeInterface_ex(int numTargets, int numSources, const double *targetX,
                              const double *targetY, const double *targetZ,
                              const double *targetValue, const double *sourceX,
                              const double *sourceY, const double *sourceZ,
                              const double *sourceValue, const double *sourceWeight,
                              double *outputArray, int kernel, int numberOfKernelParameters,
                              const double *kernelParameters, int singularity, int approximation,
                              int computeType, double theta, int degree, int sourceLeafSize,
                              int targetLeafSize, double sizeCheck, double beta, int verbosity,
                              int precision);

/* Replaces modifiedGramSchmidt_singleWavefunction,
 * 3D-GreenIteration/src/utilities/Orthogonalization.h:5 (Orthogonalization.c:14),
 * bound in orthogonalization_wrapper.py:28-30.  V is row-major
 * [numWavefunctions x numPoints]; U is orthogonalized against rows
 * 0..targetWavefunction-1, normalized in the W inner product and written to
 * U and to row targetWavefunction of V. */
void modifiedGramSchmidt_singleWavefunction(double *V, double *U, double *W, int targetWavefunction,
                                            int numPoints, int numWavefunctions);

/* Replaces InterpolateBetweenTwoMeshes,
 * 3D-GreenIteration/src/utilities/TwoMeshInterpolation.c:163-165, bound in
 * interpolation_wrapper.py:27-31.  fineF is accumulated into, as there. */
void InterpolateBetweenTwoMeshes(double *coarseX, double *coarseY, double *coarseZ,
                                 double *coarseF, int *pointsPerCell_coarse, int coarseN,
                                 double *fineX, double *fineY, double *fineZ, double *fineF,
                                 int *pointsPerCell_fine, int fineN, int numberOfCells,
                                 int cellOrder);

/* ---------------------------------------------------------------------- */
/* 2. Device pointers.                                                     */
/* ---------------------------------------------------------------------- */

/* One-shot treecode on device arrays (the device form of BaryTreeInterface:
 * same parameters, BaryTreeInterface.py:140-145, plus precision and stream).
 * Returns a status. */
int tagi_treecode_dev(int numTargets, int numSources, const double *targetX,
                      const double *targetY, const double *targetZ, const double *targetValue,
                      const double *sourceX, const double *sourceY, const double *sourceZ,
                      const double *sourceValue, const double *sourceWeight, double *outputArray,
                      int kernel, int numberOfKernelParameters, const double *kernelParameters,
                      int singularity, int approximation, int computeType, double theta,
                      int degree, int sourceLeafSize, int targetLeafSize, double sizeCheck,
                      double beta, int verbosity, int precision, void *stream);

/* Reusable plan: trees, interaction lists, proxy grids and weight charges for
 * one (targets, sources, weights) set; device inputs are read during the call
 * only.  Corresponds to the part of one callTreedriver call
 * (BaryTreeInterface.py:88-158) that depends on the mesh alone. */
typedef struct tagi_plan tagi_plan;
int tagi_plan_create(tagi_plan **plan, int numTargets, const double *targetX,
                     const double *targetY, const double *targetZ, int numSources,
                     const double *sourceX, const double *sourceY, const double *sourceZ,
                     const double *sourceWeight, double theta, int degree, int sourceLeafSize,
                     int targetLeafSize, double sizeCheck, void *stream);
int tagi_plan_destroy(tagi_plan *plan);

/* Convolve numOrbitals charge vectors over one plan in one launch sequence.
 * targetValues [numOrbitals x numTargets], sourceValues [numOrbitals x
 * numSources], output [numOrbitals x numTargets] (device, row-major);
 * kernelParameters [numOrbitals x numberOfKernelParameters] on the HOST
 * (orbital o uses kernelParameters[o * numberOfKernelParameters]).  With
 * numOrbitals = 1 this is the per-call convolution of callTreedriver. */
int tagi_plan_convolve(tagi_plan *plan, int numOrbitals, const double *targetValues,
                       const double *sourceValues, double *output, int kernel,
                       int numberOfKernelParameters, const double *kernelParameters,
                       int singularity, int precision, void *stream);

/* tagi_plan_convolve with two more controls.  kernelParametersOnDevice != 0:
 * kernelParameters is a DEVICE array (same layout), read when the call runs
 * on the GPU -- the form for calls inside a captured graph, whose parameters
 * (k_i = sqrt(-2 eps_i)) change between replays; such values are not checked
 * on the host: an unusable one (not finite, or <= 0 where the kernel uses it)
 * gives NaN output and sets a flag that tagi_plan_check_parameters returns.
 * orbitalsPerItem: 0 = automatic, 1, 4, 8 or 16 (Yukawa mixed precision
 * shares each pair's geometry across a group of orbitals; other cases use 1).
 * targetsPerThread: 0 = automatic (2 when a batch exceeds 256 targets), 1 or
 * 2 (mixed single-orbital field kernels; a tuning knob, results unchanged).
 * Extends callTreedriver (BaryTreeInterface.py:88-158), which has neither. */
int tagi_plan_convolve_ex(tagi_plan *plan, int numOrbitals, const double *targetValues,
                          const double *sourceValues, double *output, int kernel,
                          int numberOfKernelParameters, const double *kernelParameters,
                          int kernelParametersOnDevice, int singularity, int precision,
                          int orbitalsPerItem, int targetsPerThread, void *stream);
/* Waits for the stream, returns (and clears) the plan's flag of unusable
 * device kernel parameters: *flags != 0 if any call since the last check
 * had one. */
int tagi_plan_check_parameters(tagi_plan *plan, int *flags, void *stream);

/* Several systems (plans over different meshes, each with its own orbital
 * count) convolved together: per-system charge preparation and upward pass,
 * then ONE persistent launch per field pass (near, near close ranges, far)
 * whose work list holds every (system, target batch, orbital group) item,
 * heaviest first.  Up to 8 systems; all share kernel and precision.  Plans
 * are borrowed and must outlive the object.  No counterpart in the reference
 * (one BaryTreeInterface call per orbital, greenIterationFixedPoint.py:314). */
typedef struct tagi_systems tagi_systems;
int tagi_systems_create(tagi_systems **systems, int numSystems, tagi_plan *const *plans,
                        const int *numOrbitals, int kernel, int precision, int orbitalsPerItem,
                        int targetsPerThread, void *stream);
/* Arrays of numSystems device pointers, each laid out as tagi_plan_convolve's
 * arguments for that system; kernelParameters[i] host or device (flag). */
int tagi_systems_convolve(tagi_systems *systems, const double *const *targetValues,
                          const double *const *sourceValues, double *const *outputs,
                          int numberOfKernelParameters, const double *const *kernelParameters,
                          int kernelParametersOnDevice, int singularity, void *stream);
/* info[0..4] = systems, orbitals per item, work items of the near pass, the
 * close-range pass and the far pass. */
int tagi_systems_info(const tagi_systems *systems, int *info);
int tagi_systems_destroy(tagi_systems *systems);

/* One-shot batched convolution over numSystems meshes concatenated in device
 * arrays x, y, z, w (system s = points pointOffsets[s] .. pointOffsets[s+1]-1,
 * targets = sources as in Green iteration).  values/output hold, system after
 * system, numOrbitals[s] rows of that system's point count.  kernelParameters
 * (HOST): one value per orbital, system after system.  Systems go 8 per
 * launch. */
int tagi_treecode_batched(int numSystems, const int *pointOffsets, const int *numOrbitals,
                          const double *x, const double *y, const double *z, const double *w,
                          const double *values, double *output, int kernel,
                          const double *kernelParameters, int singularity, double theta,
                          int degree, int sourceLeafSize, int targetLeafSize, double sizeCheck,
                          int precision, void *stream);

/* CUDA-graph capture of a call sequence on a created (non-default) stream:
 * begin, then any of this library's device calls (each made once uncaptured
 * before, so nothing allocates; kernel parameters on the device), then end.
 * Replays re-run the captured launches on the data then in the same
 * buffers. */
typedef struct tagi_graph tagi_graph;
int tagi_graph_begin(void *stream);
int tagi_graph_end(void *stream, tagi_graph **graph);
int tagi_graph_launch(tagi_graph *graph, void *stream);
int tagi_graph_nodes(const tagi_graph *graph, int *numNodes);
int tagi_graph_destroy(tagi_graph *graph);

/* Plan statistics: info[0..12] = source nodes, target nodes, batches,
 * near-list entries, far-list entries, slots, proxy points P, upward items,
 * merged near ranges, largest batch, near pairs, far pairs, near pairs in
 * close ranges (pair counts per orbital). */
int tagi_plan_info(const tagi_plan *plan, double *info);

/* Copies of the plan's integer structure to HOST arrays, for parity checks.
 * which = 0: source tree, 1: target tree.  Array sizes from tagi_plan_info. */
int tagi_plan_get_tree(const tagi_plan *plan, int which, uint64_t *codes, int *perm, int *begin,
                       int *end, int *parent, int *first_child, int *nchild, double *center,
                       double *half, double *radius);
int tagi_plan_get_lists(const tagi_plan *plan, int *batch_node, int *near_off, int *near_list,
                        int *far_off, int *far_list, int *slot_node);
/* which = 0: weight charges (FP64, built here if no FP64 call built them);
 * 1: charges of the last FP64 call; 2: charges of the last mixed call;
 * 3: weight charges of the mixed path.  [orbital][slot][P] to host, widened
 * to double. */
int tagi_plan_get_charges(tagi_plan *plan, int which, int numOrbitals, double *out);

/* FP64 direct sum for the targets listed in subset (NULL = all); output[q]
 * is the value at target subset[q].  The exact convolution. */
int tagi_direct_dev(int numTargets, const double *targetX, const double *targetY,
                    const double *targetZ, const double *targetValue, int numSubset,
                    const int *subset, int numSources, const double *sourceX,
                    const double *sourceY, const double *sourceZ, const double *sourceValue,
                    const double *sourceWeight, double *output, int kernel,
                    const double *kernelParameters, int singularity, void *stream);

/* Device form of modifiedGramSchmidt_singleWavefunction (Orthogonalization.c:14). */
int tagi_mgs_dev(double *V, double *U, const double *W, int targetWavefunction, int numPoints,
                 int numWavefunctions, void *stream);

/* Same work as tagi_mgs_dev, but the call allocates no device memory: for
 * callers that cannot allocate while they run (device memory handed to
 * another allocator or held to a fixed budget, or a loop in which a
 * cudaMalloc/cudaFree would synchronize the device).  No counterpart in the
 * reference.  Its scratch is a fixed ~1.06 MB device array that every GPU
 * loading this library keeps until exit; targetWavefunction may be at most
 * 128 (larger requests return TAGI_ERR_ARG).  The first call on a device
 * looks the array's address up (make it before any stream capture); all calls
 * share the array, so calls that overlap on the GPU race. */
int tagi_mgs_dev_noalloc(double *V, double *U, const double *W, int targetWavefunction,
                         int numPoints, int numWavefunctions, void *stream);

/* Green-iteration and SCF steps around the convolution (device pointers,
 * FP64, no allocation: `work` is a caller workspace of at least
 * tagi_gi_workspace_doubles(numPoints, rows) doubles).  With these, one
 * Green-iteration sweep over all orbitals is a sequence of launches that can
 * be captured as one CUDA graph.  psi, f, conv: [numOrbitals x numPoints]. */
long long tagi_gi_workspace_doubles(long long numPoints, int rows);
/* f = -2 psi V_eff (greenIterationFixedPoint.py:155). */
int tagi_gi_source(const double *psi, const double *veff, long long numPoints, int numOrbitals,
                   double *f, void *stream);
/* Harrison update (greenIterationFixedPoint.py:373-399): psi_new = convScale *
 * conv; dE = -<psi V_eff (psi - psi_new)>_W / <psi_new^2>_W; epsPrev = eps;
 * eps += dE (an eigenvalue that is not negative is set to gaugeShift - 1.5
 * and flagged, as :470-477 does with a random offset); k = sqrt(-2 eps);
 * psi <- psi_new. */
int tagi_gi_update(double *psi, const double *conv, const double *veff, const double *weights,
                   long long numPoints, int numOrbitals, double convScale, double *eps,
                   double *epsPrev, double *k, double gaugeShift, double *deltaE, int *flags,
                   double *work, long long workDoubles, void *stream);
/* residual[m] = sqrt(|psi_m - psiPrev_m|_W^2 + (eps_m - epsPrev_m)^2), the
 * norm of scfFixedPoint.py:62-67; psiResidual[m] without the eigenvalue. */
int tagi_gi_residual(const double *psi, const double *psiPrev, const double *weights,
                     long long numPoints, int numOrbitals, const double *eps, const double *epsPrev,
                     double *residual, double *psiResidual, double *work, long long workDoubles,
                     void *stream);
/* Anderson mixing of every orbital's (psi, eps) over its last numHistory
 * sweeps (<= 8), the orbital-wise mixing of scfFixedPoint.py:483-597 done for
 * all orbitals at once.  F = out - in rows, layout [H x numOrbitals x numPoints].
 * gram[m][q] = sum_i w_i F_a[m][i] F_b[m][i] for the pairs a <= b of rows
 * 0..numHistory-1 in row-major order (q = a H - a(a-1)/2 + b - a); the caller
 * adds the eigenvalue parts and solves the small systems.  work: at least
 * tagi_gi_anderson_workspace_doubles doubles. */
long long tagi_gi_anderson_workspace_doubles(long long numPoints, int numHistory, int numOrbitals);
int tagi_gi_anderson_gram(const double *F, int numHistory, int numOrbitals, long long numPoints,
                          const double *weights, double *gram, double *work, long long workDoubles,
                          void *stream);
/* psi[m] = x_l + sum_k c_mk (x_k - x_l) + b (F_l + sum_k c_mk (F_k - F_l)) with
 * X the input rows, l = newestRow, k over olderRows, c [numOrbitals x (H-1)]. */
int tagi_gi_anderson_mix(const double *X, const double *F, int numHistory, int newestRow,
                         const int *olderRows, const double *coefficients, double mixingParameter,
                         int numOrbitals, long long numPoints, double *psi, void *stream);
/* out[r] = sum_i w_i a[r][i] b[r][i] (row strides; bStride 0 shares one b;
 * b NULL: b = 1; weights NULL: w = 1). */
int tagi_wdot_rows(const double *a, long long aStride, const double *b, long long bStride,
                   const double *weights, long long numPoints, int rows, double *out, double *work,
                   long long workDoubles, void *stream);
/* rho = sum_m occ_m psi_m^2, then scaled so sum_i w_i rho_i = numElectrons
 * (skipped if numElectrons <= 0) (scfFixedPoint.py:624-636). */
int tagi_scf_density(const double *psi, const double *occupations, int numOrbitals,
                     long long numPoints, const double *weights, double numElectrons, double *rho,
                     double *work, long long workDoubles, void *stream);
/* Slater exchange, spin-unpolarized LDA: vx = -(3/pi)^(1/3) rho^(1/3), ex
 * (energy per electron) = 3/4 vx. */
int tagi_lda_exchange(const double *rho, long long numPoints, double *vx, double *ex, void *stream);
/* veff = vHartree + vx + vExternal + gaugeShift (scfFixedPoint.py:345). */
int tagi_veff(const double *vHartree, const double *vx, const double *vExternal, double gaugeShift,
              long long numPoints, double *veff, void *stream);
/* Anderson combination (densityMixingSchemes.py:60-97) of ring-buffer
 * histories [H x numPoints]: newestRow is the latest (in, out) pair,
 * olderRows[k] the k-th older row, coefficients c_k from the caller's solve of
 * the weighted linear system; next = b mix_out + (1 - b) mix_in. */
int tagi_anderson_combine(const double *inHistory, const double *outHistory, int numHistory,
                          int newestRow, const int *olderRows, const double *coefficients,
                          double mixingParameter, long long numPoints, double *next, void *stream);

/* Learned extrapolation network (no counterpart in the reference): kernels
 * for a 3-layer MLP on per-cell patches with BF16 weights and FP32
 * accumulation, trained on the device.  BF16 arrays are passed as void*. */
/* C[M x N] = A[M x K] B[K x N] on the tensor cores; element (m, k) of A is
 * A[m sAm + k sAk], (k, n) of B is B[k sBk + n sBn].  epilogue 0: f32 C32;
 * 1: bf16 C16 = relu(C + bias); 2: bf16 C16 = C * (mask > 0) (mask bf16,
 * same layout as C); 3: f32 C32 = C + bias.  ldc: row stride of C. */
int tagi_mlp_gemm(const void *A, long long sAm, long long sAk, const void *B, long long sBk,
                  long long sBn, int M, int N, int K, int epilogue, float *C32, void *C16,
                  long long ldc, const float *bias, const void *mask, void *stream);
/* f32 C = A B with K split over up to `splits` blocks (partial holds splits *
 * M * N floats); the partials are added in a fixed order. */
int tagi_mlp_gemm_splitk(const void *A, long long sAm, long long sAk, const void *B, long long sBk,
                         long long sBn, int M, int N, int K, int splits, float *partial, float *C,
                         void *stream);
/* Rows (orbital, cell) of features [psi/s_psi, d/s_d, eps, 0...] (bf16, row
 * stride ldx >= 2P+1), the patch scales s_d (floored by dfloor[orbital]) and
 * d/s_d in f32.  The mesh stores each cell's P points contiguously. */
int tagi_mlp_patch_features(const double *psi, const double *d, const double *eps,
                            const double *dfloor, int numOrbitals, int numCells, int P,
                            long long numPoints, int ldx, void *X, float *scale, float *dn,
                            void *stream);
/* T = dnext / s_d per row. */
int tagi_mlp_patch_target(const double *dnext, const float *scale, int numOrbitals, int numCells,
                          int P, long long numPoints, float *T, void *stream);
/* r = alpha dn + Y - T; lossAndDalpha = {sum r^2, sum dY dn}; dY = 2r/(rows P)
 * in f32 and bf16; part: 2*rows floats. */
int tagi_mlp_mse_grad(const float *Y, const float *dn, const float *T, const float *alpha, int rows,
                      int P, float *dY, void *dY16, float *part, float *lossAndDalpha, void *stream);
long long tagi_mlp_colsum_workspace(long long rows, int N);
/* Column sums of a [rows x N] f32 (isBf16 = 0) or bf16 matrix. */
int tagi_mlp_colsum(const void *G, int isBf16, long long rows, int N, float *out, float *work,
                    long long workFloats, void *stream);
/* One Adam step on FP32 weights (bias-corrected with `step`); w16 (optional)
 * receives the BF16 copy. */
int tagi_mlp_adam(float *w, const float *g, float *m1, float *m2, long long n, float lr, float beta1,
                  float beta2, float epsilon, int step, void *w16, void *stream);
/* psiOut = psi + s_d (alpha dn + Y) per patch, dOut = the increment (may alias). */
int tagi_mlp_patch_apply(const double *psi, const float *Y, const float *dn, const float *scale,
                         const float *alpha, int numOrbitals, int numCells, int P,
                         long long numPoints, double *psiOut, double *dOut, void *stream);
int tagi_mlp_to_bf16(const float *a, long long n, void *b, void *stream);

/* Device form of InterpolateBetweenTwoMeshes (TwoMeshInterpolation.c:163);
 * the points-per-cell arrays are device int32 arrays. */
int tagi_interp_dev(const double *coarseX, const double *coarseY, const double *coarseZ,
                    const double *coarseF, const int *pointsPerCell_coarse, int coarseN,
                    const double *fineX, const double *fineY, const double *fineZ,
                    double *fineF, const int *pointsPerCell_fine, int fineN, int numberOfCells,
                    int cellOrder, void *stream);

/* Mesh generation on the device, in two calls.
 *
 * tagi_mesh_refine replaces the per-cell refinement the reference runs in
 * Python for the "coarsenedUniformTwoLevel" divide criterion
 * (mpiMeshBuilding.py:402-421 refineCellReturnCells -> TreeStruct_CC.py:1049
 * recursiveDivide -> CellStruct_CC.py:2344 refineCoarseningUniform_TwoLevel,
 * then TreeStruct_CC.py:2360 extractCellXYZ).  baseCells: device
 * [numBase x 6] rows (xmin, xmax, ymin, ymax, zmin, zmax), the rows
 * inializeBaseMesh_distributed returns (mpiMeshBuilding.py:103); atomXYZ:
 * device [numAtoms x 3].  h, H, r, level are divideParameter1..4 (near
 * spacing, far spacing, ball radius, level); cells below minDepth always
 * divide (the tree's minDepth); a cell at maxDepth (<= 16) that the rule would
 * divide is an error.  Writes the leaf cells depth first, children x-major
 * (the reference's uniqueID order), as centre (cellX..Z), width
 * (cellDX..DZ), (order+1)^3 points per coarse cell and 1, 8, 27 or 64 times
 * that per fine cell: the arrays extractCellXYZ returns.  cellX == NULL
 * counts only.  numCells / numCoarsePoints / numFinePoints (host) receive the
 * counts, also when capacity is too small (TAGI_ERR_ARG).  Synchronizes the
 * stream once per refinement level.
 *
 * tagi_mesh_points replaces the point loop of buildMeshFromMinimumDepthCells
 * (mpiMeshBuilding.py:517-556: coarseQuadraturePointsSingleCell and
 * fineQuadraturePointsSingleCell): the coarse mesh X, Y, Z, W
 * [numCoarsePoints] and, when Xf..Wf are given, the two-level fine mesh
 * [numFinePoints] of the cell table.  unitNodes / unitWeights (host,
 * order+1 each) are the first-kind nodes cos(theta_i) on [-1, 1] and the
 * unscaled weights (meshUtilities.py:835-883); NULL for both computes them
 * with libm.  Results are bit-identical to the reference's for the same
 * tables.  These two entry points have no device counterpart in the
 * reference. */
int tagi_mesh_refine(const double *baseCells, int numBase, const double *atomXYZ, int numAtoms,
                     int order, double h, double H, double r, double level, int minDepth,
                     int maxDepth, double *cellX, double *cellY, double *cellZ, double *cellDX,
                     double *cellDY, double *cellDZ, int *ptsPerCellCoarse, int *ptsPerCellFine,
                     int capacity, int *numCells, long long *numCoarsePoints,
                     long long *numFinePoints, void *stream);
int tagi_mesh_points(const double *cellX, const double *cellY, const double *cellZ,
                     const double *cellDX, const double *cellDY, const double *cellDZ,
                     const int *ptsPerCellFine, int numCells, int order, const double *unitNodes,
                     const double *unitWeights, double *X, double *Y, double *Z, double *W,
                     long long numCoarsePoints, double *Xf, double *Yf, double *Zf, double *Wf,
                     long long numFinePoints, void *stream);

/* ---------------------------------------------------------------------- */
/* 3. Configuration and errors.                                            */
/* ---------------------------------------------------------------------- */
int tagi_set_precision(int precision);   /* default for BaryTreeInterface */
int tagi_get_precision(void);
/* beta in [0, 1] -> theta, degree, leaf sizes (project-defined). */
int tagi_beta_parameters(double beta, double *theta, int *degree, int *sourceLeafSize,
                         int *targetLeafSize);
/* Orbitals per work item that a convolution of maxOrbitals orbitals at this
 * degree runs with (requested 0 = automatic, else 1, 4, 8 or 16; the rule of
 * tagi_plan_convolve_ex and tagi_systems_create). */
int tagi_orbitals_per_item(int kernel, int precision, int maxOrbitals, int requested, int degree,
                           int *orbitalsPerItem);
/* Instrumentation: number of kernels this library has launched in this
 * process; optional per-phase device timing with CUDA events on the
 * launching stream.  Phases: 0 tree, 1 lists, 2 upward pass, 3 near field,
 * 4 far field, 5 glue, 6 near field close-range pass.  tagi_profile_read
 * waits for the recorded events, returns summed milliseconds and mark
 * counts per phase (nphase >= 7), and clears the record. */
long long tagi_launch_count(void);
/* Pair-throughput ceiling of the mixed-precision field kernels' inner loops
 * on this GPU: their arithmetic (variant 0: near-field loop, 1: far-field
 * proxy-grid loop, 2: Yukawa orbital-group near loop and 3: Yukawa
 * orbital-group far loop, 8 orbitals per pair geometry, 4 and 5: the same
 * with 16 orbitals packed by orbital; groups counted per pair and orbital)
 * with operands in shared memory and registers and no global-memory
 * traffic, timed with CUDA events.  Pair interactions / s.  A field kernel's
 * rate over this is its loop efficiency, not a hardware roofline. */
int tagi_pair_peak(int kernel, int singularity, int variant, double kernelParameter,
                   double *pairsPerSecond, void *stream);
/* Hardware pipe rates of this GPU, measured with every SM busy and no memory
 * traffic, in lane operations per second: rates[0] FP32 FFMA, rates[1]
 * packed FFMA2 (two lanes per instruction), rates[2] MUFU ex2, rates[3]
 * MUFU rsqrt, rates[4] the SM clock in MHz seen during the FFMA run (clock64
 * cycles over CUDA-event time), rates[5] the number of SMs, rates[6] FP64
 * DFMA, rates[7] MUFU lg2.  rates must hold 8 values.  The field kernels' roofline is their
 * arithmetic per pair against these rates. */
int tagi_pipe_rates(double *rates, void *stream);
int tagi_profile(int enable);
int tagi_profile_read(double *ms, long long *count, int nphase);

int tagi_last_error(void);
const char *tagi_last_error_message(void);
void tagi_clear_error(void);
int tagi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* TAGI_GB300_H */
