/*
 * cfx.h - C ABI of libcudaLduSolvers.so, the GB300 (sm_103a) lduMatrix solvers.
 *
 * The library replaces, for one GPU, the reference's lduMatrix::solver path:
 * an OpenFOAM plugin class (cudaPCG, cudaPBiCGStab, cudaGAMG deriving
 * Foam::lduMatrix::solver) holds a cfx_mesh per lduMesh,
 * re-uploads coefficients on every solve and calls cfx_solve().  All entry
 * points take plain pointers and sizes; labels are int32 (WM_LABEL_SIZE=32)
 * and scalars double (WM_DP).  Every function returns a cfx_status.
 *
 * Reference interfaces replaced (paths relative to the OpenFOAM-dev tree):
 *   lduAddressing                src/OpenFOAM/matrices/lduMatrix/lduAddressing/lduAddressing.H:172-194
 *   lduMatrix coefficients       src/OpenFOAM/matrices/lduMatrix/lduMatrix/lduMatrix.H:86-87
 *   lduMatrix::solver::New/solve src/OpenFOAM/matrices/lduMatrix/lduMatrix/lduMatrix.H:187-255,
 *                                src/OpenFOAM/matrices/lduMatrix/lduMatrix/lduMatrixSolver.C:40-130
 *   SolverPerformance            src/OpenFOAM/matrices/LduMatrix/LduMatrix/SolverPerformance.H:79-304
 *   lduMatrix::Amul / residual   src/OpenFOAM/matrices/lduMatrix/lduMatrix/lduMatrixATmul.C:34-92, 203-280
 *   preconditioner::precondition src/OpenFOAM/matrices/lduMatrix/lduMatrix/lduMatrix.H:420-430
 *   smoother::smooth             src/OpenFOAM/matrices/lduMatrix/lduMatrix/lduMatrix.H:316-330
 *   GAMGAgglomeration            src/OpenFOAM/matrices/lduMatrix/solvers/GAMG/GAMGAgglomerations/
 *                                GAMGAgglomeration/GAMGAgglomeration.H:325-380
 */
#ifndef CFX_H
#define CFX_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    CFX_OK = 0,
    CFX_ERR_ARG = -1,         /* bad argument (null pointer, size, enum) */
    CFX_ERR_ADDRESSING = -2,  /* l/u not upper-triangular, out of range */
    CFX_ERR_CUDA = -3,        /* CUDA runtime error (message: cfx_last_error) */
    CFX_ERR_NOMEM = -4,       /* device allocation failed */
    CFX_ERR_ADMISSION = -5,   /* request exceeds the server's HBM budget */
    CFX_ERR_TIMEOUT = -6,     /* a bounded device wait expired */
    CFX_ERR_CONFIG = -7,      /* unknown solver/preconditioner/smoother name */
    CFX_ERR_STATE = -8,       /* call out of order (e.g. GAMG without levels) */
    CFX_ERR_FATAL = -9        /* the reference's FatalError (e.g. "Singular matrix") */
} cfx_status;

typedef struct cfx_ctx cfx_ctx;        /* device, stream, scratch */
typedef struct cfx_mesh cfx_mesh;      /* resident addressing + schedules + GAMG levels */
typedef struct cfx_matrix cfx_matrix;  /* coefficients on a mesh */

/* SolverPerformance<scalar> (SolverPerformance.H:79-304) */
typedef struct {
    char solverName[32];   /* e.g. "DICPCG", "DILUPBiCGStab", "GAMG" */
    double initialResidual;
    double finalResidual;
    int nIterations;
    int converged;
    int singular;
    int status;            /* cfx_status of the solve */
    int nOuter;            /* mixed precision: refinement steps; else 0 */
    int pad;
} cfx_perf;

/* CFX_SOLVER_SMOOTH: smoothSolver (smoothSolver.C:77-196); CFX_SOLVER_PBICG:
 * PBiCG (PBiCG.C:65-220, asymmetric matrices; preconditioners with a
 * preconditionT: none, diagonal, DILU) */
enum { CFX_SOLVER_PCG = 0, CFX_SOLVER_PBICGSTAB = 1, CFX_SOLVER_GAMG = 2, CFX_SOLVER_SMOOTH = 3,
       CFX_SOLVER_PBICG = 4 };
/* CFX_PRE_GAMG: GAMGPreconditioner (GAMGPreconditioner.C:81-148), nVcycles
 * V-cycles with the controls' GAMG fields (smoother, sweeps) from w = 0; the
 * mesh needs GAMG levels */
/* CFX_PRE_FDIC: FDICPreconditioner (FDICPreconditioner.C:40-137, symmetric):
 * its cached rD[u]*upper products are the ones DIC forms, so it runs the DIC
 * sweeps and reports "FDIC<solver>" */
enum { CFX_PRE_NONE = 0, CFX_PRE_DIAGONAL = 1, CFX_PRE_DIC = 2, CFX_PRE_DILU = 3, CFX_PRE_GAMG = 4,
       CFX_PRE_FDIC = 5 };
/* lduMatrix::smoother run-time table (GAMG's smoother, smoothSolver's):
 * GaussSeidel, DIC (symmetric), symGaussSeidel, DILU (asymmetric),
 * DICGaussSeidel (symmetric), DILUGaussSeidel (asymmetric), FDIC (symmetric;
 * the DIC smoother's arithmetic, FDICSmoother.C:40-160) and
 * nonBlockingGaussSeidel (GaussSeidel's arithmetic when there are no
 * coupled interfaces, nonBlockingGaussSeidelSmoother.C:92-233) */
enum { CFX_SMOOTH_GS = 0, CFX_SMOOTH_DIC = 1, CFX_SMOOTH_SYMGS = 2, CFX_SMOOTH_DILU = 3, CFX_SMOOTH_DICGS = 4,
       CFX_SMOOTH_DILUGS = 5, CFX_SMOOTH_FDIC = 6, CFX_SMOOTH_NBGS = 7 };
enum { CFX_FP64 = 0, CFX_MIXED = 1 };

/* Solver controls: lduMatrix::solver::readControls (lduMatrixSolver.C:158-164)
 * and GAMGSolver::readControls (GAMGSolver.C:348-388); use cfx_default_controls. */
typedef struct {
    int solver;            /* CFX_SOLVER_* */
    int preconditioner;    /* CFX_PRE_* (PCG, PBiCGStab) */
    double tolerance;      /* default 1e-6 */
    double relTol;         /* default 0 */
    int maxIter;           /* default 1000 */
    int minIter;           /* default 0 */
    /* GAMG */
    int smoother;          /* CFX_SMOOTH_* (default GaussSeidel; GAMG and smoothSolver) */
    int nPreSweeps, preSweepsLevelMultiplier, maxPreSweeps;       /* 0, 1, 4 */
    int nPostSweeps, postSweepsLevelMultiplier, maxPostSweeps;    /* 2, 1, 4 */
    int nFinestSweeps;     /* 2 */
    int scaleCorrection;   /* -1: default = matrix symmetric */
    int nCellsInCoarsestLevel; /* 10 */
    /* precision: CFX_FP64, or CFX_MIXED = FP32 inner solve in an FP64
     * iterative-refinement loop (outer residual, solution, normFactor and
     * convergence in FP64) */
    int precision;
    /* smoothSolver: sweeps between residual checks (default 1; negative: that
     * many sweeps and no residuals, smoothSolver.C:93-116) */
    int nSweeps;
    /* GAMG preconditioner: V-cycles per application (default 2) and its own
     * tolerance / relTol (its coarsest-level solves; defaults 1e-6, 0) */
    int nVcycles;
    /* GAMG: interpolateCorrection (GAMGSolverInterpolate.C:30-130; default 0) */
    int interpolateCorrection;
    double pcTolerance;
    double pcRelTol;
    /* GAMG: directSolveCoarsest - the coarsest level by a dense LU with
     * implicit partial pivoting (LUscalarMatrix, GAMGSolver.C:257-267;
     * default 0); a singular coarsest matrix is CFX_ERR_FATAL */
    int directSolveCoarsest;
    int reserved;
} cfx_controls;

void cfx_default_controls(cfx_controls* c);

/* Human-readable text of the last error on this thread. */
const char* cfx_last_error(void);
int cfx_version(void);

/* ---- context ------------------------------------------------------------
 * Handles are reference counted: a mesh holds its context and a matrix its
 * mesh (batches and servers hold their context), so the *_destroy calls may
 * come in any order; memory goes with the last handle that uses it.
 *
 * Stream order: a context enqueues on its own non-blocking stream.  Entry
 * points that take the caller's device pointers first order that stream
 * after the work already on the legacy default stream (where CUDA runtime
 * code and PyTorch produce arrays by default), and those that return before
 * their work completes (cfx_fvm_assemble, cfx_matrix_update_device, the
 * diagonal solve) order the default stream after it.  A caller producing or
 * consuming arrays on another stream synchronises that stream itself, or
 * enqueues on the context's stream (cfx_ctx_stream). */
cfx_status cfx_ctx_create(int device, cfx_ctx** ctx);
cfx_status cfx_ctx_destroy(cfx_ctx* ctx);
/* The cudaStream_t all work of this context is enqueued on. */
cfx_status cfx_ctx_stream(cfx_ctx* ctx, void** stream);
cfx_status cfx_ctx_synchronize(cfx_ctx* ctx);
/* Number of kernels this context has launched (for launch accounting). */
cfx_status cfx_ctx_launch_count(cfx_ctx* ctx, int64_t* count);

/* ---- mesh (lduAddressing) ----------------------------------------------- */
/* Validates that (l, u) is upper-triangular (l < u, sorted by l then u, as
 * lduPrimitiveMesh::checkUpperTriangular, lduPrimitiveMesh.C:60-95), builds
 * losort/ownerStart/losortStart and the forward/backward level schedules of
 * the lower/upper dependency DAG, and keeps them resident. */
cfx_status cfx_mesh_create(cfx_ctx* ctx, int nCells, int nFaces, const int32_t* l,
                           const int32_t* u, cfx_mesh** mesh);
cfx_status cfx_mesh_destroy(cfx_mesh* mesh);
/* Level-schedule depth of the forward (lower) DAG. */
cfx_status cfx_mesh_info(cfx_mesh* mesh, int* nFwdLevels, int* nBwdLevels);
/* The finest level's sliced ELL rows used by the A x products (no reference
 * counterpart: the reference's products loop over faces): slices of 32 rows,
 * how many are offset-pattern slices (no columns stored), and the entries
 * including padding.  slices 0: not built (a row with over 255 neighbours). */
cfx_status cfx_mesh_sell_info(cfx_mesh* mesh, int* slices, int* patternSlices, int64_t* entries);

/* faceAreaPair weights |(Sf/sqrt|Sf|) * (1, 1.01, 1.02)|
 * (faceAreaPairGAMGAgglomeration.C:55-80) from face-area vectors Sf[nFaces*3]. */
cfx_status cfx_face_area_pair_weights(int nFaces, const double* Sf, double* weights);

/* GAMG level hierarchy by pairwise agglomeration of the given face weights
 * (pairGAMGAgglomerate.C:31-301, GAMGAgglomerateLduAddressing.C:32-222) on
 * the host, then uploaded.  forwardStart is the initial cell-loop direction
 * (pairGAMGAgglomeration::forward_, true in a fresh process). */
cfx_status cfx_gamg_agglomerate(cfx_mesh* mesh, const double* faceWeights,
                                int nCellsInCoarsestLevel, int forwardStart);
/* Same, from an agglomeration computed by the caller (e.g. the reference's
 * own cached GAMGAgglomeration): restrictAddr[i] has the cell count of level
 * i (level 0 = this mesh) and maps to nCoarseCells[i] cells. */
cfx_status cfx_gamg_set_levels(cfx_mesh* mesh, int nLevels, const int32_t* const* restrictAddr,
                               const int32_t* nCoarseCells);
/* Level sizes; restrictAddr/coarse l,u of level i copied out when non-null. */
cfx_status cfx_gamg_level_info(cfx_mesh* mesh, int level, int* nCells, int* nFaces,
                               int32_t* restrictAddr, int32_t* faceRestrict, int32_t* faceFlip,
                               int32_t* coarseL, int32_t* coarseU);
cfx_status cfx_gamg_n_levels(cfx_mesh* mesh, int* nLevels);
/* GAMG's coarse cyclic interfaces of one level, on the host
 * (cyclicGAMGInterface.C:87-151; GAMGAgglomerateLduAddressing.C:250-340
 * creates them): from the finer level's interfaces (nPatches patches of
 * patchSize faces in patch order, their cells and partner cells) and the
 * restriction map, each patch's faces grouped by (coarse cell, coarse partner
 * cell) in order of first appearance.  Out: the coarse patch sizes
 * [nPatches], coarse face cells and partner cells [sum of patchSize at
 * most], each fine face's coarse face (patch-order index) and the coarse
 * face count.  cfx_mesh_set_interfaces' GAMG levels are built this way. */
cfx_status cfx_gamg_coarse_interfaces(int32_t nFineCells, const int32_t* restrictAddr, int32_t nPatches,
                                      const int32_t* patchSize, const int32_t* faceCells,
                                      const int32_t* nbrCells, int32_t* coarsePatchSize,
                                      int32_t* coarseFaceCells, int32_t* coarseNbrCells,
                                      int32_t* fineToCoarse, int32_t* nCoarseFaces);

/* ---- matrix (lduMatrix coefficients) ------------------------------------ */
/* Host coefficients; lower == NULL means symmetric (lduMatrix::symmetric()).
 * upper == lower == NULL is a diagonal matrix (lduMatrix::diagonal()): every
 * solve of it is diagonalSolver's psi = source/diag ("diagonal", 0
 * iterations, converged), whatever solver the controls name, as
 * lduMatrix::solver::New selects it (lduMatrixSolver.C:52-66,
 * diagonalSolver.C:62-81). */
cfx_status cfx_matrix_create(cfx_mesh* mesh, const double* diag, const double* upper,
                             const double* lower, cfx_matrix** mat);
/* Re-upload coefficients (a new fvMatrix on the same mesh, every solve). */
cfx_status cfx_matrix_update(cfx_matrix* mat, const double* diag, const double* upper,
                             const double* lower);
/* Coupled (cyclic) interfaces of the mesh (lduInterfaceFieldPtrsList with
 * cyclic fields): nPatches patches, faces concatenated in patch order, for
 * each face the cell on this side (faceCells) and the neighbour patch's cell
 * (nbrFaceCells).  Amul, Tmul, residual, sumA/normFactor and the
 * Gauss-Seidel smoothers then add the interface terms as
 * lduMatrix::updateMatrixInterfaces does with cyclicFvPatchField
 * (cyclicFvPatchField.C:150-174: result[faceCells] -= coeffs*psi[nbr]);
 * the DIC/DILU factorisations ignore them, as the reference's do.  PCG,
 * PBiCGStab, PBiCG, smoothSolver and GAMG (cyclicGAMGInterface levels, and
 * GAMG as PCG's preconditioner) solve such systems, FP64 and mixed; the
 * direct coarsest-level solve also needs cfx_mesh_set_interface_partners;
 * the nonBlockingGaussSeidel smoother is refused.  nPatches = 0 removes
 * them.  Set the interfaces before the matrices' interface coefficients. */
cfx_status cfx_mesh_set_interfaces(cfx_mesh* mesh, int32_t nPatches, const int32_t* patchSize,
                                   const int32_t* faceCells, const int32_t* nbrFaceCells);
/* Each interface patch's partner patch (cyclicLduInterface::nbrPatchIndex,
 * cyclicLduInterface.H, in the numbering of cfx_mesh_set_interfaces), which
 * LUscalarMatrix::convert (LUscalarMatrix.C:205-265) reads for the direct
 * coarsest-level solve: it subtracts the partner's interfaceBouCoeffs.  A
 * partner must have as many faces.  Needed only by directSolveCoarsest with
 * interfaces; cfx_mesh_set_interfaces forgets it. */
cfx_status cfx_mesh_set_interface_partners(cfx_mesh* mesh, const int32_t* nbrPatch);
/* interfaceBouCoeffs and interfaceIntCoeffs (host, faces concatenated in patch
 * order; intCoeffs NULL: the same as bouCoeffs). */
cfx_status cfx_matrix_set_interface_coeffs(cfx_matrix* mat, const double* bouCoeffs, const double* intCoeffs);

/* A matrix of zero coefficients (symmetric: no lower triangle), to be filled
 * on the device by cfx_fvm_assemble or cfx_matrix_update_device. */
cfx_status cfx_matrix_create_empty(cfx_mesh* mesh, int symmetric, cfx_matrix** mat);

/* ---- finite-volume assembly on the device ------------------------------- */
/* Face geometry of the fvMesh behind an lduMesh, uploaded once (host
 * arrays): per internal face (lduAddressing order) magSf, the snGrad
 * scheme's deltaCoeffs and the linear interpolation weights (may be NULL
 * when no linear div term is assembled); per cell V; per boundary face, in
 * patch order, its cell, magSf and deltaCoeffs. */
cfx_status cfx_fv_geometry(cfx_mesh* mesh, const double* magSf, const double* deltaCoeffs, const double* weights,
                           const double* V, int32_t nBoundaryFaces, const int32_t* boundaryCells,
                           const double* magSfB, const double* deltaCoeffsB);

enum { CFX_DIV_UPWIND = 0, CFX_DIV_LINEAR = 1 };
enum { CFX_BC_ZERO_GRADIENT = 0, CFX_BC_FIXED_VALUE = 1, CFX_BC_FIXED_GRADIENT = 2, CFX_BC_CYCLIC = 3 };

/* fvm::ddt(psi) + fvm::div(phi, psi) + lapSign*fvm::laplacian(gamma, psi)
 * == su, every pointer a device array, every term optional:
 *   ddt (Euler, EulerDdtScheme.C:466-497) when rDeltaT > 0, psi0 = old psi;
 *   div (gaussConvectionScheme.C:121-152) when phi != NULL: face fluxes of
 *     the internal faces and phiB of the boundary faces; divScheme
 *     CFX_DIV_UPWIND (pos0(phi)) or CFX_DIV_LINEAR (the mesh weights);
 *   laplacian (gaussLaplacianScheme.C:47-89) when lapSign = +1 or -1:
 *     gamma/gammaB per face, or gammaUniform when gamma == NULL;
 *   su (NULL: none): operator==, source += V*su.
 * psi's boundary conditions per boundary face: bcType CFX_BC_* and bcValue
 * (the fixed value or the fixed gradient).  CFX_BC_CYCLIC marks a face of a
 * cyclic patch (cyclicFvPatchField): the coupled patch coefficients
 * (coupledFvPatchField.C:157-205: value w, 1 - w with the upwind weight;
 * gradient -deltaCoeffs, deltaCoeffs with deltaCoeffsB of that face the
 * snGrad scheme's, nonOrthDeltaCoeffs), internalCoeffs added to the
 * diagonal, boundaryCoeffs kept out of the source, and both written as the
 * matrix's interface coefficients; the cyclic faces, in boundary order, must
 * be the faces given to cfx_mesh_set_interfaces, in their order (else
 * CFX_ERR_ARG), and a div term with them must be upwind. */
typedef struct {
    double rDeltaT;
    const double* psi0;
    const double* phi;
    const double* phiB;
    int divScheme;
    int lapSign;
    double gammaUniform;
    const double* gamma;
    const double* gammaB;
    const int32_t* bcType;
    const double* bcValue;
    const double* su;
} cfx_fvm_terms;

/* Assembles the equation into mat's coefficients (on the device; as
 * fvMatrix::solveSegregated hands them to the solver, boundary diagonal
 * included) and its source into d_source (device, nCells).  A div term makes
 * the matrix asymmetric: mat must then have been created asymmetric. */
cfx_status cfx_fvm_assemble(cfx_matrix* mat, const cfx_fvm_terms* terms, double* d_source);

/* Same with device pointers (coefficients already in HBM). */
cfx_status cfx_matrix_update_device(cfx_matrix* mat, const double* d_diag, const double* d_upper,
                                    const double* d_lower);
cfx_status cfx_matrix_destroy(cfx_matrix* mat);
/* Coefficients of level `level` copied out: 0 the matrix itself (e.g. after
 * cfx_fvm_assemble), >= 1 the coarse levels assembled on the device. */
cfx_status cfx_matrix_coarse(cfx_matrix* mat, int level, double* diag, double* upper, double* lower);

/* ---- solve (lduMatrix::solver::solve) ------------------------------------ */
/* psi (in/out) and source are host arrays of nCells doubles. */
cfx_status cfx_solve(cfx_matrix* mat, const cfx_controls* ctl, double* psi, const double* source,
                     cfx_perf* perf);
/* Same with device pointers: nothing crosses PCIe/C2C except the perf record. */
cfx_status cfx_solve_device(cfx_matrix* mat, const cfx_controls* ctl, double* d_psi,
                            const double* d_source, cfx_perf* perf);

/* ---- tuning (process-wide knobs; no reference counterpart) ---------------
 * How triangular sweeps run, by mesh size.  A mesh whose vector fits one
 * CTA's shared memory sweeps in one CTA; one that fits a cluster's
 * distributed shared memory sweeps in one cluster; otherwise:
 *   CFX_TUNE_SMALL_SWEEP    <= this many cells: one CTA, vector in global
 *                           memory (default 0)
 *   CFX_TUNE_CLUSTER_GLOBAL <= this many cells: one cluster, vector in global
 *                           memory, cluster barriers between levels
 *   larger: the persistent grid-wide level scheduler.
 *   CFX_TUNE_CLUSTER_SIZE   CTAs per cluster (16 or 8 as the GPU allows; 0,
 *                           the default, disables the cluster forms: on GB300
 *                           the grid form sweeps mid-size levels faster). */
enum { CFX_TUNE_SMALL_SWEEP = 0, CFX_TUNE_CLUSTER_GLOBAL = 1, CFX_TUNE_CLUSTER_SIZE = 2,
       /* FP32 inner solves of mixed-precision batches (cfx_batch_*) reduce
        * the residual by 10^-value (default 3) per refinement step */
       CFX_TUNE_BATCH_INNER_DIGITS = 3,
       /* bytes of the swept vector one CTA may hold in shared memory (the
        * single-CTA form and a cluster CTA's share); default the device's
        * opt-in limit less the kernels' static use; 0 forces global forms */
       CFX_TUNE_SMEM_BYTES = 4,
       /* grid form: 1 = wavefront, each 32-slot group waits only for the
        * groups it reads; 0 (default) = whole-level counters, faster on GB300
        * for the fused multi-sweep Gauss-Seidel of the coarse levels */
       CFX_TUNE_GRID_WAVE = 5,
       /* CTAs per cluster for the DIC/DILU forward/backward sweeps when
        * CFX_TUNE_CLUSTER_SIZE is 0: a vector that fits the cluster's shared
        * memory is swept there (default 16 where the GPU allows it: PCG+DIC
        * 64^3 1.5x faster than the grid form); 0 keeps the grid */
       CFX_TUNE_CLUSTER_PRE = 6,
       CFX_TUNE_FLOW = 7,
       /* dataflow form: warps launched for this many levels of the
        * schedule's average width (default 4; 1..64) */
       CFX_TUNE_FLOW_AHEAD = 8,
       /* A x products (Amul, residual, the solvers' fused products): 0
        * gathers each row through losort/ownerStart; 1 and 2 (default) read
        * it from the level's sliced ELL copy, 2 with the slices whose rows
        * share at most 8 neighbour offsets stored without columns (1 or 2
        * is read when a mesh is created).  The results are identical */
       CFX_TUNE_AMUL_SELL = 9,
       /* level-counter grid form of the sweeps: the spacing of the per-level
        * completion counters in ints (1..32; 32 puts each in its own 128-byte
        * line) and the back-off of the waiting CTAs' polls in ns (0..1000) */
       CFX_TUNE_GRID_STRIDE = 10, CFX_TUNE_GRID_POLL_NS = 11,
       /* groups of 32 slots per chunk of the level-counter grid form (1..8,
        * default 2), read when a level's schedule is built: smaller chunks
        * spread a DAG level's arithmetic over more SMs */
       CFX_TUNE_CHUNK_GROUPS = 12,
       /* single-CTA form in FP32: hold 32 (1, default) or 16 (0) entries per
        * slot in registers when a schedule's slots have more than 16 (256^3
        * mixed GAMG 1.77 -> 1.71 s; in FP64 the larger set spills) */
       CFX_TUNE_CTA_XL = 13,
       /* Gauss-Seidel smoothing order: 0 the reference's cell order
        * everywhere; 1 (default) a multicolour order (a greedy colouring of
        * each level's cells, smaller colours first: about sweeps x colours
        * dependent steps instead of the cell order's thousands) in the FP32
        * inner cycles of mixed-precision solves, whose FP64 refinement still
        * reaches the FP64 tolerance; the FP64 solves keep the reference's
        * order bit for bit; 2 the multicolour order everywhere (tests) */
       CFX_TUNE_COLORED_GS = 14,
       /* DIC / DILU order (preconditioners and smoothers): 0 the
        * reference's everywhere; 1 (default) DIC (symmetric matrices) in the
        * FP32 inner solves of mixed-precision solves takes the incomplete
        * factorisation and its sweeps in the multicolour order (a cell's
        * smaller-coloured neighbours are its forward entries, the
        * larger-coloured its backward ones): a few dependent steps per sweep
        * instead of hundreds; 2 DILU there too (on convection-dominated
        * systems the multicolour DILU is a much weaker preconditioner); 3
        * both everywhere (tests).  The FP64 solves and the coarsest level's
        * one-CTA solve keep the reference's order */
       CFX_TUNE_COLORED_PRE = 15,
       /* schedules of at most this many DAG levels (0..128, default 96)
        * whose vector does not fit one CTA's shared memory run level by
        * level, one ordinary launch per level with no waits: the multicolour
        * schedules, whose levels are few and wide; 0: never */
       CFX_TUNE_LEVEL_LAUNCH = 16 };
cfx_status cfx_tune_set(int key, int value);
cfx_status cfx_tune_get(int key, int* value);

/* ---- batched solves of many small systems --------------------------------
 * No counterpart in the reference: many independent lduMatrix systems (an
 * ensemble of small cases, a parameter sweep) solved by one kernel launch,
 * one CTA per system.  Each system follows lduMatrix::solver::solve exactly
 * as cfx_solve does (PCG with symmetric, PBiCGStab with either matrix; any
 * preconditioner of cfx_controls), or, with precision CFX_MIXED, FP32 inner
 * solves inside FP64 iterative refinement (normFactor, residuals and the
 * convergence test in FP64).  The launch hands systems to persistent CTAs
 * largest first and is replayed from a CUDA graph.  Systems are numbered in
 * creation order; psi and source vectors are the systems' vectors
 * concatenated in that order (offsets: prefix sums of nCells). */
typedef struct cfx_batch cfx_batch;
/* l[i], u[i]: addressing of system i (as cfx_mesh_create). */
cfx_status cfx_batch_create(cfx_ctx* ctx, int nSystems, const int32_t* nCells, const int32_t* nFaces,
                            const int32_t* const* l, const int32_t* const* u, cfx_batch** batch);
cfx_status cfx_batch_destroy(cfx_batch* batch);
/* Host coefficients of system i; lower == NULL means symmetric. */
cfx_status cfx_batch_set_matrix(cfx_batch* batch, int i, const double* diag, const double* upper,
                                const double* lower);
/* psi (in/out) and source: host arrays of sum(nCells) doubles; perf[nSystems]. */
cfx_status cfx_batch_solve(cfx_batch* batch, const cfx_controls* ctl, double* psi, const double* source,
                           cfx_perf* perf);
/* The batch's resident device vectors (psi, source, each sum(nCells)
 * doubles) and the nSystems+1 cell offsets; any pointer may be NULL. */
cfx_status cfx_batch_vectors(cfx_batch* batch, double** d_psi, double** d_source, int64_t* offsets);
/* Solve with the resident device vectors; only perf crosses to the host. */
cfx_status cfx_batch_solve_device(cfx_batch* batch, const cfx_controls* ctl, cfx_perf* perf);
/* Start and end of each system's solve in the last launch, in ms from the
 * first start (device clock), creation order; arrays of nSystems. */
cfx_status cfx_batch_timings(cfx_batch* batch, double* startMs, double* endMs);
/* Persistent CTAs per SM (0: as many as fit). */
cfx_status cfx_batch_set_ctas_per_sm(cfx_batch* batch, int ctasPerSm);
/* Large systems on thread-block clusters: systems of at least bigCells cells
 * are each solved by a whole cluster of clusterSize CTAs (2..16), the rest
 * by one CTA each; clusterSize 0 turns clusters off (the default).  A
 * system's result depends on whether it ran on a cluster (the sums' order
 * changes), not on the rest of the batch. */
cfx_status cfx_batch_set_groups(cfx_batch* batch, int clusterSize, int bigCells);
cfx_status cfx_batch_get_groups(cfx_batch* batch, int* clusterSize, int* nBig, int* ctasPerSm);
/* Autotuned packing: times resident solves from the current psi (restored
 * afterwards) with one CTA per system, then with the systems whose solve
 * outlasted half the balanced share of the batch on clusters of 4, 8 and 16
 * CTAs, and keeps the fastest.  best = chosen cluster size (0: none);
 * bestMs = its time.  Either may be NULL. */
cfx_status cfx_batch_tune(cfx_batch* batch, const cfx_controls* ctl, int* best, float* bestMs);

/* ---- solve server ----------------------------------------------------------
 * No counterpart in the reference: an in-process server for many clients
 * (solver instances of several cases, a parametric study driver, a service
 * front end).  Matrices are registered once and stay resident in HBM;
 * requests bring a right-hand side (and initial psi) for a resident matrix,
 * so re-solving one (a PISO corrector) uploads two vectors.  Requests on
 * small matrices are solved together in persistent launches (continuous
 * batching: up to `lanes` launches run at once, each on its own stream and
 * taking the queued requests of one precision and one size class, at most one
 * request per matrix at a time, up to maxBatch), so a request that arrives
 * while a launch runs starts on an idle lane at once; requests on large
 * matrices (more than largeCells cells) run alone through the whole-GPU
 * drivers, with cudaGAMG when the matrix was registered with face weights,
 * yielding the GPU to the lanes between V-cycles.  Admission: resident matrices and the
 * requests' device vectors count against hbmBudget bytes; a matrix that does
 * not fit, or a request that alone exceeds the budget, is refused with
 * CFX_ERR_ADMISSION; a request that does not fit now blocks the submitting
 * thread until completions free space.  All functions are thread-safe. */
typedef struct cfx_server cfx_server;
typedef struct {
    int64_t hbmBudget;          /* bytes (default 150e9) */
    int largeCells;             /* larger matrices are solved alone (default 1,000,000) */
    int maxBatch;               /* systems per launch (default 1024) */
    int nCellsInCoarsestLevel;  /* GAMG agglomeration of large matrices (default 10) */
    int groupCells;             /* small matrices of at least this many cells are solved by */
    int groupSize;              /* a thread-block cluster of groupSize CTAs (defaults 100,000 and 4;
                                 * 0: one CTA each); a result depends on its matrix only, never on
                                 * the rest of the launch */
    int lanes;                  /* batch launches that may run at once, each on its own stream
                                 * (default 8, 1..16) */
} cfx_server_config;
typedef struct {
    int64_t submitted, completed, cancelled, failed, refused;
    int64_t batches, batchedSolves, largeSolves;
    int64_t queueDepth, running, residentMatrices;
    int64_t hbmInUse, hbmBudget;
    double elapsedS, solvesPerS;   /* since creation or the last reset */
    double p50Ms, p99Ms, meanMs, maxMs;  /* submit-to-completion latency */
    int64_t largeYields;           /* times a large solve yielded the GPU to a batch */
    double queueP50Ms, queueP99Ms; /* submit to start of its launch or solve */
    double runP50Ms, runP99Ms;     /* start to completion */
} cfx_server_stats_t;
void cfx_server_default_config(cfx_server_config* cfg);
/* cfg NULL: defaults.  The server runs on ctx's device. */
cfx_status cfx_server_create(cfx_ctx* ctx, const cfx_server_config* cfg, cfx_server** server);
/* Stops the worker after the running launch; frees everything. */
cfx_status cfx_server_destroy(cfx_server* server);
/* Registers a matrix (host arrays; lower NULL = symmetric; faceWeights
 * [nFaces] or NULL: large matrices given weights get a faceAreaPair GAMG
 * hierarchy).  matrixId identifies it in requests. */
cfx_status cfx_server_add_matrix(cfx_server* server, int nCells, int nFaces, const int32_t* l, const int32_t* u,
                                 const double* diag, const double* upper, const double* lower,
                                 const double* faceWeights, int64_t* matrixId);
/* Frees the matrix once no request uses it. */
cfx_status cfx_server_remove_matrix(cfx_server* server, int64_t matrixId);
/* Queues a solve (psi0 NULL: zero initial guess); the host arrays are copied
 * before the call returns. */
cfx_status cfx_server_submit(cfx_server* server, int64_t matrixId, const cfx_controls* ctl, const double* psi0,
                             const double* source, int64_t* requestId);
/* Waits up to timeoutMs (< 0: forever) for a request, copies psi (if non-NULL)
 * and perf out and frees the request.  CFX_ERR_TIMEOUT leaves it pending;
 * a cancelled request returns CFX_ERR_STATE. */
cfx_status cfx_server_wait(cfx_server* server, int64_t requestId, int timeoutMs, double* psi, cfx_perf* perf);
/* Removes a queued request (its wait returns CFX_ERR_STATE); CFX_ERR_STATE if
 * it is already running or finished. */
cfx_status cfx_server_cancel(cfx_server* server, int64_t requestId);
/* The client gives the request up (disconnect): queued -> cancelled;
 * running -> freed when it completes; finished -> freed now. */
cfx_status cfx_server_release(cfx_server* server, int64_t requestId);
cfx_status cfx_server_stats(cfx_server* server, cfx_server_stats_t* stats);
cfx_status cfx_server_reset_stats(cfx_server* server);

/* ---- single operations, device pointers (parity tests, building blocks) -- */
cfx_status cfx_amul(cfx_matrix* mat, const double* d_x, double* d_y);
cfx_status cfx_tmul(cfx_matrix* mat, const double* d_x, double* d_y);
cfx_status cfx_residual(cfx_matrix* mat, const double* d_x, const double* d_b, double* d_r);
cfx_status cfx_sumA(cfx_matrix* mat, double* d_s);
/* which: 0 sum, 1 sumMag, 2 sumSqr, 3 sumProd(a, b) -> *out (host). */
cfx_status cfx_reduce(cfx_ctx* ctx, int which, int n, const double* d_a, const double* d_b, double* out);
cfx_status cfx_norm_factor(cfx_matrix* mat, const double* d_psi, const double* d_b, double* out);
/* kind CFX_PRE_*; transpose != 0 applies DILU preconditionT. */
cfx_status cfx_precondition(cfx_matrix* mat, int kind, int transpose, const double* d_r, double* d_w);
cfx_status cfx_reciprocal_d(cfx_matrix* mat, int kind, double* d_rD);
cfx_status cfx_smooth(cfx_matrix* mat, int kind, double* d_psi, const double* d_b, int nSweeps);

/* ---- reduction that allocates nothing ------------------------------------
 * No counterpart in the reference: an extra entry point for callers that
 * cannot call cudaMalloc (a host application whose own memory pool reserves
 * the whole GPU, or one held to a fixed device-memory budget).  Same
 * operations as cfx_reduce (which: 0 sum, 1 sumMag, 2 sumSqr, 3 sumProd), no
 * context: d_a, d_b (device, n doubles) in, the result to the device double
 * d_out, enqueued on `stream` (a cudaStream_t; NULL = the default stream)
 * without synchronizing.  Its only scratch is a static device array of 4096
 * block partials, so n <= 33,554,432 (larger n returns CFX_ERR_ARG).  The
 * first call on a device looks up that array's address (make it before any
 * stream capture); calls on one device share the array, so calls that
 * overlap on the GPU race. */
cfx_status cfx_reduce_noalloc(int which, int n, const double* d_a, const double* d_b, double* d_out,
                              void* stream);

/* ---- diagnostics (no reference counterpart) -------------------------------
 * Exercises the failure path of the bounded device waits without any fault:
 * one Gauss-Seidel sweep of the matrix in the persistent grid form with the
 * level-0 completion count started one short, so level 1 waits on a count
 * nothing will reach.  Each wait gives up after timeoutMs (1..10000), the
 * kernel raises its abort flag, every CTA returns, and *status receives the
 * device status (CFX_ERR_TIMEOUT).  The context and the matrix stay usable;
 * the matrix needs at least two forward levels. */
cfx_status cfx_diag_sweep_stall(cfx_matrix* mat, int timeoutMs, int* status);

/* The smoothing the FP32 inner cycles of a mixed-precision GAMG solve apply
 * to a level, on its own: nSweeps sweeps of smoother `kind` (the cfx_smooth
 * kinds GaussSeidel, DIC, DILU and their GaussSeidel combinations) on the
 * matrix's FP32 coefficient copy, psi and b device FP32 vectors of nCells,
 * in the order the inner cycles use (CFX_TUNE_COLORED_GS /
 * CFX_TUNE_COLORED_PRE).  *form (may be NULL) receives the execution form of
 * the Gauss-Seidel schedule (DIC / DILU: of the forward schedule): 0 one CTA
 * (vector in shared memory), 1 a cluster (distributed shared memory), 2 one
 * CTA (vector in global memory),
 * 3 a cluster (global memory), 4 the persistent grid, 5 the dataflow form,
 * 6 one launch per level.  For timing and profiling. */
cfx_status cfx_diag_smooth_f32(cfx_matrix* mat, int kind, float* psi, const float* b, int nSweeps, int* form);

#ifdef __cplusplus
}
#endif

#endif
