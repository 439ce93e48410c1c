/*
 * ldu_oracle.h - CPU restatement of OpenFOAM-dev's lduMatrix solver path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the CUDA solver library is
 * compared against; nothing in the product links or calls it.  Each function
 * follows the reference loop it cites (file:line relative to the OpenFOAM-dev
 * tree) with the same operation order, so that compiled with
 * -ffp-contract=off it reproduces the reference's x86-64 build bit for bit.
 * It is pinned against the reference itself (oracle/_ref, built from source
 * by oracle/build_ref.py) through the golden vectors in tests/golden/.
 *
 * Labels are int32 (WM_LABEL_SIZE=32), scalars double (WM_DP).
 */
#ifndef LDU_ORACLE_H
#define LDU_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int nCells, nFaces;
    const int *l, *u;            /* lowerAddr, upperAddr */
    const double *diag, *upper;  /* lower == NULL -> symmetric */
    const double *lower;
    int *ownerStart;             /* [nCells+1] */
    int *losort;                 /* [nFaces] */
    int *losortStart;            /* [nCells+1] */
    /* coupled (cyclic) interfaces, faces concatenated in patch order: the
     * cell on this side, the neighbour patch's cell, interfaceBouCoeffs and
     * interfaceIntCoeffs (nIf = 0: none) */
    int nIf;
    const int *ifCell, *ifNbr;
    const double *ifBou, *ifInt;
    /* the interfaces' patch sizes (GAMG groups each patch's faces on its
     * own); nIfPatch = 0 with nIf > 0: one patch of nIf faces */
    int nIfPatch;
    const int* ifPatchSize;
    /* each patch's partner patch (cyclicLduInterface::nbrPatchIndex), or
     * NULL: needed only by the direct coarsest-level solve */
    const int* ifNbrPatch;
} ldu_matrix;

typedef struct {
    double initialResidual, finalResidual;
    int nIterations, converged, singular;
} ldu_perf;

typedef struct {
    double tolerance, relTol;
    int maxIter, minIter;
} ldu_controls;

/* lduAddressing.C:32-170 (losort, ownerStart, losortStart).  Allocates the
 * three derived arrays inside m; release with ldu_free_addr. */
int ldu_init_addr(ldu_matrix* m);
void ldu_free_addr(ldu_matrix* m);

/* lduMatrixATmul.C */
void ldu_amul(const ldu_matrix* m, const double* x, double* y);
void ldu_tmul(const ldu_matrix* m, const double* x, double* y);
void ldu_sumA(const ldu_matrix* m, double* s);
void ldu_residual(const ldu_matrix* m, const double* x, const double* b, double* r);

/* FieldReductionFunctions.C */
double ldu_sum(int n, const double* a);
double ldu_sum_mag(int n, const double* a);
double ldu_sum_sqr(int n, const double* a);
double ldu_sum_prod(int n, const double* a, const double* b);
double ldu_average(int n, const double* a);

/* lduMatrixSolver.C:174-197 */
double ldu_norm_factor(const ldu_matrix* m, const double* psi, const double* b,
                       const double* Apsi, double* tmp);

/* Preconditioners: 0 none, 1 diagonal, 2 DIC, 3 DILU */
enum { LDU_PRE_NONE = 0, LDU_PRE_DIAGONAL = 1, LDU_PRE_DIC = 2, LDU_PRE_DILU = 3 };
void ldu_dic_rD(const ldu_matrix* m, double* rD);
void ldu_dic_precondition(const ldu_matrix* m, const double* rD, const double* r, double* w);
void ldu_dilu_rD(const ldu_matrix* m, double* rD);
void ldu_dilu_precondition(const ldu_matrix* m, const double* rD, const double* r, double* w);
void ldu_dilu_preconditionT(const ldu_matrix* m, const double* rD, const double* r, double* w);

/* Smoothers: 0 GaussSeidel, 1 DIC */
enum { LDU_SMOOTH_GS = 0, LDU_SMOOTH_DIC = 1 };
void ldu_gs_smooth(const ldu_matrix* m, double* psi, const double* b, int nSweeps);
void ldu_dic_smooth(const ldu_matrix* m, const double* rD, double* psi, const double* b, int nSweeps);
void ldu_symgs_smooth(const ldu_matrix* m, double* psi, const double* b, int nSweeps);
void ldu_dilu_smooth(const ldu_matrix* m, const double* rD, double* psi, const double* b, int nSweeps);
/* smoothers beyond GaussSeidel and DIC (the values above) */
enum { LDU_SMOOTH_SYMGS = 2, LDU_SMOOTH_DILU = 3, LDU_SMOOTH_DICGS = 4, LDU_SMOOTH_DILUGS = 5 };
/* the named smoother, nSweeps sweeps (DIC/DILU pivots computed inside) */
void ldu_smooth(const ldu_matrix* m, int smoother, double* psi, const double* b, int nSweeps);
int ldu_smooth_solve(const ldu_matrix* m, double* psi, const double* b, const ldu_controls* c, int smoother,
                     int nSweeps, ldu_perf* perf);

/* PCG.C:65-193, PBiCGStab.C:68-254.  Return 0 or a negative error. */
int ldu_pcg(const ldu_matrix* m, double* psi, const double* b, const ldu_controls* c,
            int precond, ldu_perf* perf);
/* PBiCG::solve (PBiCG.C:65-220; asymmetric matrices): precond LDU_PRE_NONE,
 * DIAGONAL or DILU, with the preconditioner's preconditionT on the
 * transpose residual.  Returns -2 when the iteration count passes
 * max(1000, maxIter) (the reference's FatalError). */
int ldu_pbicg(const ldu_matrix* m, double* psi, const double* b, const ldu_controls* c, int precond,
              ldu_perf* perf);
int ldu_pbicgstab(const ldu_matrix* m, double* psi, const double* b, const ldu_controls* c,
                  int precond, ldu_perf* perf);

/* pairGAMGAgglomerate.C:123-301: one level of pairwise agglomeration.
 * *forward is the direction flag (pairGAMGAgglomeration::forward_), toggled
 * on return.  Returns nCoarseCells. */
int ldu_pair_agglomerate(int nCells, int nFaces, const int* l, const int* u,
                         const double* weights, int* forward, int* restrictMap);

/* GAMGAgglomerateLduAddressing.C:32-197: coarse l/u, faceRestrictAddr and
 * faceFlipMap of one level.  cl/cu must hold nFaces entries.  Returns
 * nCoarseFaces. */
int ldu_agglomerate_addressing(int nCells, int nFaces, const int* l, const int* u,
                               const int* restrictMap, int nCoarseCells, int* cl, int* cu,
                               int* faceRestrict, int* faceFlip);

/* GAMG agglomeration hierarchy (pairGAMGAgglomerate.C:31-118 with
 * mergeLevels 1, GAMGAgglomeration.C:205-230 stop rule, maxLevels 50). */
typedef struct {
    int nLevels;                 /* number of coarse levels */
    int nCells[50], nFaces[50];  /* coarse sizes per level */
    int* restrictAddr[50];       /* [fine nCells of level i] */
    int* faceRestrict[50];       /* [fine nFaces of level i] */
    int* faceFlip[50];
    int* cl[50];                 /* coarse lowerAddr [nFaces[i]] */
    int* cu[50];
} ldu_agglomeration;

int ldu_gamg_agglomerate(int nCells, int nFaces, const int* l, const int* u,
                         const double* weights, int nCellsInCoarsestLevel, int forwardStart,
                         ldu_agglomeration* agg);
void ldu_gamg_free(ldu_agglomeration* agg);

/* One GAMG level's coarse cyclic interfaces (cyclicGAMGInterface.C:87-151)
 * and summed coefficients (GAMGInterface.C:90-115) from the finer level's
 * (patch order) and restriction map R; returns the coarse face count. */
int ldu_gamg_coarse_interfaces(const int* R, int nPatch, const int* patchSize, const int* faceCells,
                               const int* nbrCells, const double* bou, int* coarsePatchSize, int* coarseFaceCells,
                               int* coarseNbrCells, double* coarseBou, int* toCoarse);

/* faceAreaPairGAMGAgglomeration.C:55-80 weights from face-area vectors. */
void ldu_face_area_pair_weights(int nFaces, const double* Sf, double* w);

/* GAMGSolverAgglomerateMatrix.C:33-193: coarse diag/upper/lower of level i. */
void ldu_gamg_coarse_matrix(int nFineCells, int nFineFaces, const double* fdiag,
                            const double* fupper, const double* flower,
                            const int* restrictAddr, const int* faceRestrict, const int* faceFlip,
                            int nCoarseCells, int nCoarseFaces, double* cdiag, double* cupper,
                            double* clower);

typedef struct {
    int nPreSweeps, preSweepsLevelMultiplier, maxPreSweeps;
    int nPostSweeps, postSweepsLevelMultiplier, maxPostSweeps;
    int nFinestSweeps;
    int scaleCorrection;  /* -1: default (= symmetric) */
    int smoother;         /* LDU_SMOOTH_* */
    int interpolateCorrection; /* GAMGSolverInterpolate.C:30-130 (default 0) */
    int directSolveCoarsest;   /* LU of the coarsest level (GAMGSolver.C:257-267; default 0) */
} ldu_gamg_controls;

/* LUDecompose (scalarMatrices.C:77-180): in-place Crout factorisation with
 * implicit partial pivoting of the row-major n x n matrix A; piv[n].
 * Returns -1 for a matrix with an all-zero row ("Singular matrix"). */
int ldu_lu_decompose(int n, double* A, int* piv);
/* LUBacksubstitute (scalarMatricesTemplates.C:117-163): x = A^-1 x. */
void ldu_lu_backsubstitute(int n, const double* LU, const int* piv, double* x);

void ldu_gamg_default_controls(ldu_gamg_controls* g);

/* GAMGSolverSolve.C:31-552 with GAMGSolverScale.C:31-76.  The agglomeration
 * must have been built for m's addressing.  Returns -1 without coarse levels,
 * -2 when the direct coarsest solve meets a singular matrix. */
int ldu_gamg(const ldu_matrix* m, const ldu_agglomeration* agg, double* psi, const double* b,
             const ldu_controls* c, const ldu_gamg_controls* g, ldu_perf* perf);
/* PCG with the GAMG preconditioner; pc: the preconditioner dictionary's
 * tolerance/relTol */
int ldu_pcg_gamg(const ldu_matrix* m, const ldu_agglomeration* agg, double* psi, const double* b,
                 const ldu_controls* c, const ldu_gamg_controls* g, const ldu_controls* pc, int nVcycles,
                 ldu_perf* perf);

/* ---- finite-volume assembly (fvMatrix of a scalar transport equation) ----
 * Face geometry of an fvMesh: internal faces (lowerAddr/upperAddr = owner /
 * neighbour) with magSf, the snGrad scheme's deltaCoeffs and the linear
 * interpolation weights; boundary faces in patch order with their cell,
 * magSf and deltaCoeffs; cell volumes. */
typedef struct {
    int nCells, nFaces, nBoundary;
    const int *l, *u;
    const double *magSf, *deltaCoeffs, *weights, *V;
    const int* bCell;
    const double *magSfB, *deltaCoeffsB;
} ldu_fv_geom;

enum { LDU_DIV_UPWIND = 0, LDU_DIV_LINEAR = 1 };
enum { LDU_BC_ZERO_GRADIENT = 0, LDU_BC_FIXED_VALUE = 1, LDU_BC_FIXED_GRADIENT = 2, LDU_BC_CYCLIC = 3 };

/* fvm::ddt(psi) + fvm::div(phi, psi) + lapSign*fvm::laplacian(gamma, psi)
 * == su, each term optional: ddt when rDeltaT > 0 (Euler: psi0 the old
 * value), div when phi != NULL (upwind or linear weights), laplacian when
 * lapSign != 0 (gamma per face, or gammaUniform when gamma == NULL); psi's
 * boundary conditions per boundary face (type, value or gradient). */
typedef struct {
    double rDeltaT;
    const double* psi0;
    const double *phi, *phiB;
    int divScheme;
    int lapSign;
    double gammaUniform;
    const double *gamma, *gammaB;
    const int* bcType;
    const double* bcValue;
    const double* su;
} ldu_fvm_terms;

/* The lduMatrix and source fvMatrix::solveSegregated hands to the solver:
 * each term built as EulerDdtScheme.C:466-497, gaussConvectionScheme.C:
 * 121-152 and gaussLaplacianScheme.C:47-89 build it, combined with
 * fvMatrix::operator+=/-= (fvMatrix.C:1094-1148, lduMatrixOperations.C:
 * 140-318), operator==(fvMatrix, field) adding V*su (fvMatrix.C:1705-1715),
 * then addBoundaryDiag / addBoundarySource (fvMatrix.C:112-174).  lower is
 * written when the result is asymmetric (a div term).  Returns -1 when no
 * term is given. */
int ldu_fvm_assemble(const ldu_fv_geom* g, const ldu_fvm_terms* t, double* diag, double* upper, double* lower,
                     double* source);
/* The same with cyclic (coupled) boundary faces (bcType LDU_BC_CYCLIC): their
 * internalCoeffs join the diagonal (addBoundaryDiag), their boundaryCoeffs
 * stay out of the source (addBoundarySource(source, false)), and both are
 * returned, in boundary-face order, as the solver's interfaceBouCoeffs
 * (ifBou) and interfaceIntCoeffs (ifInt).  Coupled patches take the
 * coupledFvPatchField coefficients (coupledFvPatchField.C:157-205): value
 * (w, 1 - w) with the upwind weight pos0(phi), gradient (-deltaCoeffs,
 * deltaCoeffs) with the snGrad scheme's deltaCoeffs in deltaCoeffsB.
 * Returns -1 when no term is given, -2 for linear div with cyclic faces
 * (the patch weights are not given). */
int ldu_fvm_assemble_coupled(const ldu_fv_geom* g, const ldu_fvm_terms* t, double* diag, double* upper,
                             double* lower, double* source, double* ifBou, double* ifInt);

#ifdef __cplusplus
}
#endif

#endif
