/*
 * ldu_oracle.c - CPU restatement of OpenFOAM-dev's lduMatrix solver path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker; see ldu_oracle.h).  Compile with
 * -ffp-contract=off: every loop keeps the reference's operation order so the
 * results equal the reference's x86-64 (non-FMA) build bit for bit.
 */
#include "ldu_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* OpenFOAM doubleScalar constants (src/OpenFOAM/primitives/Scalar/doubleScalar/doubleScalar.H:55-66)
 * and SolverPerformance great_/small_/vsmall_ (SolverPerformance.H:285-291). */
#define VSMALL DBL_MIN
#define GREAT (1.0 / DBL_EPSILON)
#define SP_GREAT 1e20
#define SP_SMALL 1e-20

static void* xmalloc(size_t n) { return malloc(n ? n : 1); }

/* ---------------------------------------------------------------- addressing */

/* lduAddressing::calcLosort (lduAddressing.C:32-90): faces grouped by
 * neighbour (upperAddr), each group in face order.  losortStart is the
 * group offset array (calcLosortStart, lduAddressing.C:130-170).
 * calcOwnerStart (lduAddressing.C:93-127): offsets of the owner-sorted faces. */
int ldu_init_addr(ldu_matrix* m) {
    const int n = m->nCells, nf = m->nFaces;
    m->ownerStart = (int*)xmalloc(sizeof(int) * (n + 1));
    m->losort = (int*)xmalloc(sizeof(int) * nf);
    m->losortStart = (int*)xmalloc(sizeof(int) * (n + 1));
    int* cnt = (int*)calloc(n + 1, sizeof(int));
    for (int f = 0; f < nf; ++f) cnt[m->u[f] + 1]++;
    m->losortStart[0] = 0;
    for (int c = 0; c < n; ++c) m->losortStart[c + 1] = m->losortStart[c] + cnt[c + 1];
    memset(cnt, 0, sizeof(int) * (n + 1));
    for (int f = 0; f < nf; ++f) {
        const int c = m->u[f];
        m->losort[m->losortStart[c] + cnt[c]++] = f;
    }
    for (int c = 0; c <= n; ++c) m->ownerStart[c] = nf;
    m->ownerStart[0] = 0;
    int nOwnStart = 0, i = 1;
    for (int f = 0; f < nf; ++f) {
        const int curOwn = m->l[f];
        if (curOwn > nOwnStart) {
            while (i <= curOwn) m->ownerStart[i++] = f;
            nOwnStart = curOwn;
        }
    }
    free(cnt);
    return 0;
}

void ldu_free_addr(ldu_matrix* m) {
    free(m->ownerStart);
    free(m->losort);
    free(m->losortStart);
    m->ownerStart = m->losort = m->losortStart = NULL;
}

static const double* lowerOf(const ldu_matrix* m) { return m->lower ? m->lower : m->upper; }

/* lduMatrix::updateMatrixInterfaces (lduMatrixUpdateMatrixInterfaces.C:96-
 * 266) with cyclic interfaces (cyclicFvPatchField.C:150-174, a scalar field:
 * no transform): result[faceCells] -= coeffs*psi[nbrFaceCells], patch by
 * patch.  neg: the callers that pass the negated coefficients (residual,
 * the Gauss-Seidel smoothers' mBouCoeffs). */
static void update_interfaces(const ldu_matrix* m, const double* coeffs, int neg, const double* psi,
                              double* result) {
    for (int k = 0; k < m->nIf; ++k) {
        const double c = neg ? -coeffs[k] : coeffs[k];
        result[m->ifCell[k]] -= c * psi[m->ifNbr[k]];
    }
}

/* ------------------------------------------------------------- matrix ops */

/* lduMatrix::Amul, lduMatrixATmul.C:34-92 */
void ldu_amul(const ldu_matrix* m, const double* x, double* y) {
    const double* lo = lowerOf(m);
    for (int c = 0; c < m->nCells; ++c) y[c] = m->diag[c] * x[c];
    for (int f = 0; f < m->nFaces; ++f) {
        y[m->u[f]] += lo[f] * x[m->l[f]];
        y[m->l[f]] += m->upper[f] * x[m->u[f]];
    }
    update_interfaces(m, m->ifBou, 0, x, y);
}

/* lduMatrix::Tmul, lduMatrixATmul.C:95-151 */
void ldu_tmul(const ldu_matrix* m, const double* x, double* y) {
    const double* lo = lowerOf(m);
    for (int c = 0; c < m->nCells; ++c) y[c] = m->diag[c] * x[c];
    for (int f = 0; f < m->nFaces; ++f) {
        y[m->u[f]] += m->upper[f] * x[m->l[f]];
        y[m->l[f]] += lo[f] * x[m->u[f]];
    }
    update_interfaces(m, m->ifInt, 0, x, y);
}

/* lduMatrix::sumA, lduMatrixATmul.C:154-200 */
void ldu_sumA(const ldu_matrix* m, double* s) {
    const double* lo = lowerOf(m);
    for (int c = 0; c < m->nCells; ++c) s[c] = m->diag[c];
    for (int f = 0; f < m->nFaces; ++f) {
        s[m->u[f]] += lo[f];
        s[m->l[f]] += m->upper[f];
    }
    for (int k = 0; k < m->nIf; ++k) s[m->ifCell[k]] -= m->ifBou[k];
}

/* lduMatrix::residual, lduMatrixATmul.C:203-280 */
void ldu_residual(const ldu_matrix* m, const double* x, const double* b, double* r) {
    const double* lo = lowerOf(m);
    for (int c = 0; c < m->nCells; ++c) r[c] = b[c] - m->diag[c] * x[c];
    for (int f = 0; f < m->nFaces; ++f) {
        r[m->u[f]] -= lo[f] * x[m->l[f]];
        r[m->l[f]] -= m->upper[f] * x[m->u[f]];
    }
    update_interfaces(m, m->ifBou, 1, x, r);
}

/* ------------------------------------------------------------- reductions */
/* FieldReductionFunctions.C: sequential sums in index order (serial reduce is
 * a no-op, src/Pstream/dummy/UPstream.C). */
double ldu_sum(int n, const double* a) {
    double s = 0;
    for (int i = 0; i < n; ++i) s += a[i];
    return s;
}
double ldu_sum_mag(int n, const double* a) {
    double s = 0;
    for (int i = 0; i < n; ++i) s += fabs(a[i]);
    return s;
}
double ldu_sum_sqr(int n, const double* a) {
    double s = 0;
    for (int i = 0; i < n; ++i) s += a[i] * a[i];
    return s;
}
double ldu_sum_prod(int n, const double* a, const double* b) {
    double s = 0;
    for (int i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}
/* gAverage, FieldReductionFunctions.C:334-357 */
double ldu_average(int n, const double* a) { return n > 0 ? ldu_sum(n, a) / n : 0.0; }

/* lduMatrix::solver::normFactor, lduMatrixSolver.C:174-197 */
double ldu_norm_factor(const ldu_matrix* m, const double* psi, const double* b,
                       const double* Apsi, double* tmp) {
    const int n = m->nCells;
    ldu_sumA(m, tmp);
    const double avg = ldu_average(n, psi);
    for (int i = 0; i < n; ++i) tmp[i] *= avg;
    double s = 0;
    for (int i = 0; i < n; ++i) s += fabs(Apsi[i] - tmp[i]) + fabs(b[i] - tmp[i]);
    return s + SP_SMALL;
}

/* --------------------------------------------------------- preconditioners */

/* DICPreconditioner::calcReciprocalD, DICPreconditioner.C:57-84 (rD = diag on entry
 * in the reference ctor, :40-54) */
void ldu_dic_rD(const ldu_matrix* m, double* rD) {
    for (int c = 0; c < m->nCells; ++c) rD[c] = m->diag[c];
    for (int f = 0; f < m->nFaces; ++f)
        rD[m->u[f]] -= m->upper[f] * m->upper[f] / rD[m->l[f]];
    for (int c = 0; c < m->nCells; ++c) rD[c] = 1.0 / rD[c];
}

/* DICPreconditioner::precondition, DICPreconditioner.C:87-123 */
void ldu_dic_precondition(const ldu_matrix* m, const double* rD, const double* r, double* w) {
    for (int c = 0; c < m->nCells; ++c) w[c] = rD[c] * r[c];
    for (int f = 0; f < m->nFaces; ++f)
        w[m->u[f]] -= rD[m->u[f]] * m->upper[f] * w[m->l[f]];
    for (int f = m->nFaces - 1; f >= 0; --f)
        w[m->l[f]] -= rD[m->l[f]] * m->upper[f] * w[m->u[f]];
}

/* DILUPreconditioner::calcReciprocalD, DILUPreconditioner.C:57-85 */
void ldu_dilu_rD(const ldu_matrix* m, double* rD) {
    const double* lo = lowerOf(m);
    for (int c = 0; c < m->nCells; ++c) rD[c] = m->diag[c];
    for (int f = 0; f < m->nFaces; ++f)
        rD[m->u[f]] -= m->upper[f] * lo[f] / rD[m->l[f]];
    for (int c = 0; c < m->nCells; ++c) rD[c] = 1.0 / rD[c];
}

/* DILUPreconditioner::precondition, DILUPreconditioner.C:88-135 */
void ldu_dilu_precondition(const ldu_matrix* m, const double* rD, const double* r, double* w) {
    const double* lo = lowerOf(m);
    for (int c = 0; c < m->nCells; ++c) w[c] = rD[c] * r[c];
    for (int k = 0; k < m->nFaces; ++k) {
        const int f = m->losort[k];
        w[m->u[f]] -= rD[m->u[f]] * lo[f] * w[m->l[f]];
    }
    for (int f = m->nFaces - 1; f >= 0; --f)
        w[m->l[f]] -= rD[m->l[f]] * m->upper[f] * w[m->u[f]];
}

/* DILUPreconditioner::preconditionT, DILUPreconditioner.C:138-185 */
void ldu_dilu_preconditionT(const ldu_matrix* m, const double* rD, const double* r, double* w) {
    const double* lo = lowerOf(m);
    for (int c = 0; c < m->nCells; ++c) w[c] = rD[c] * r[c];
    for (int f = 0; f < m->nFaces; ++f)
        w[m->u[f]] -= rD[m->u[f]] * m->upper[f] * w[m->l[f]];
    for (int k = m->nFaces - 1; k >= 0; --k) {
        const int f = m->losort[k];
        w[m->l[f]] -= rD[m->l[f]] * lo[f] * w[m->u[f]];
    }
}

typedef struct {
    int kind;
    double* rD;
} precon;

static void precon_init(precon* p, const ldu_matrix* m, int kind) {
    p->kind = kind;
    p->rD = NULL;
    if (kind == LDU_PRE_NONE) return;
    p->rD = (double*)xmalloc(sizeof(double) * m->nCells);
    if (kind == LDU_PRE_DIAGONAL) {
        /* diagonalPreconditioner.C ctor: rD = 1/diag */
        for (int c = 0; c < m->nCells; ++c) p->rD[c] = 1.0 / m->diag[c];
    } else if (kind == LDU_PRE_DIC) {
        ldu_dic_rD(m, p->rD);
    } else {
        ldu_dilu_rD(m, p->rD);
    }
}

static void precon_apply(const precon* p, const ldu_matrix* m, double* w, const double* r) {
    switch (p->kind) {
        case LDU_PRE_NONE:
            memcpy(w, r, sizeof(double) * m->nCells);
            break;
        case LDU_PRE_DIAGONAL:
            for (int c = 0; c < m->nCells; ++c) w[c] = p->rD[c] * r[c];
            break;
        case LDU_PRE_DIC:
            ldu_dic_precondition(m, p->rD, r, w);
            break;
        default:
            ldu_dilu_precondition(m, p->rD, r, w);
            break;
    }
}

/* --------------------------------------------------------------- smoothers */

/* GaussSeidelSmoother::smooth, GaussSeidelSmoother.C:66-187 (no interfaces) */
void ldu_gs_smooth(const ldu_matrix* m, double* psi, const double* b, int nSweeps) {
    const int n = m->nCells;
    const double* lo = lowerOf(m);
    double* bPrime = (double*)xmalloc(sizeof(double) * n);
    for (int sweep = 0; sweep < nSweeps; ++sweep) {
        memcpy(bPrime, b, sizeof(double) * n);
        update_interfaces(m, m->ifBou, 1, psi, bPrime);  /* the Jacobi interface term */
        int fEnd = m->ownerStart[0];
        for (int c = 0; c < n; ++c) {
            const int fStart = fEnd;
            fEnd = m->ownerStart[c + 1];
            double psii = bPrime[c];
            for (int f = fStart; f < fEnd; ++f) psii -= m->upper[f] * psi[m->u[f]];
            psii /= m->diag[c];
            for (int f = fStart; f < fEnd; ++f) bPrime[m->u[f]] -= lo[f] * psii;
            psi[c] = psii;
        }
    }
    free(bPrime);
}

/* DICSmoother::smooth, DICSmoother.C:67-116 */
void ldu_dic_smooth(const ldu_matrix* m, const double* rD, double* psi, const double* b, int nSweeps) {
    const int n = m->nCells;
    double* rA = (double*)xmalloc(sizeof(double) * n);
    for (int sweep = 0; sweep < nSweeps; ++sweep) {
        ldu_residual(m, psi, b, rA);
        for (int c = 0; c < n; ++c) rA[c] *= rD[c];
        for (int f = 0; f < m->nFaces; ++f) {
            const int u = m->u[f];
            rA[u] -= rD[u] * m->upper[f] * rA[m->l[f]];
        }
        for (int f = m->nFaces - 1; f >= 0; --f) {
            const int l = m->l[f];
            rA[l] -= rD[l] * m->upper[f] * rA[m->u[f]];
        }
        for (int c = 0; c < n; ++c) psi[c] += rA[c];
    }
    free(rA);
}

/* symGaussSeidelSmoother::smooth, symGaussSeidelSmoother.C:66-204 (no
 * interfaces): per sweep bPrime = source, a forward pass as GaussSeidel, then
 * a backward pass over the cells in reverse order that starts from the bPrime
 * the forward pass left (the lower contributions of the forward values). */
void ldu_symgs_smooth(const ldu_matrix* m, double* psi, const double* b, int nSweeps) {
    const int n = m->nCells;
    const double* lo = lowerOf(m);
    double* bPrime = (double*)xmalloc(sizeof(double) * n);
    for (int sweep = 0; sweep < nSweeps; ++sweep) {
        memcpy(bPrime, b, sizeof(double) * n);
        update_interfaces(m, m->ifBou, 1, psi, bPrime);  /* the Jacobi interface term */
        int fEnd = m->ownerStart[0];
        for (int c = 0; c < n; ++c) {
            const int fStart = fEnd;
            fEnd = m->ownerStart[c + 1];
            double psii = bPrime[c];
            for (int f = fStart; f < fEnd; ++f) psii -= m->upper[f] * psi[m->u[f]];
            psii /= m->diag[c];
            for (int f = fStart; f < fEnd; ++f) bPrime[m->u[f]] -= lo[f] * psii;
            psi[c] = psii;
        }
        int fStart = m->ownerStart[n];
        for (int c = n - 1; c >= 0; --c) {
            const int fE = fStart;
            fStart = m->ownerStart[c];
            double psii = bPrime[c];
            for (int f = fStart; f < fE; ++f) psii -= m->upper[f] * psi[m->u[f]];
            psii /= m->diag[c];
            for (int f = fStart; f < fE; ++f) bPrime[m->u[f]] -= lo[f] * psii;
            psi[c] = psii;
        }
    }
    free(bPrime);
}

/* DILUSmoother::smooth, DILUSmoother.C:67-118 */
void ldu_dilu_smooth(const ldu_matrix* m, const double* rD, double* psi, const double* b, int nSweeps) {
    const int n = m->nCells;
    const double* lo = lowerOf(m);
    double* rA = (double*)xmalloc(sizeof(double) * n);
    for (int sweep = 0; sweep < nSweeps; ++sweep) {
        ldu_residual(m, psi, b, rA);
        for (int c = 0; c < n; ++c) rA[c] *= rD[c];
        for (int f = 0; f < m->nFaces; ++f) {
            const int u = m->u[f];
            rA[u] -= rD[u] * lo[f] * rA[m->l[f]];
        }
        for (int f = m->nFaces - 1; f >= 0; --f) {
            const int l = m->l[f];
            rA[l] -= rD[l] * m->upper[f] * rA[m->u[f]];
        }
        for (int c = 0; c < n; ++c) psi[c] += rA[c];
    }
    free(rA);
}

/* lduMatrix::smoother by name: GaussSeidel, symGaussSeidel, DIC (symmetric),
 * DILU (asymmetric), DICGaussSeidel and DILUGaussSeidel
 * (DICGaussSeidelSmoother.C:79-92, DILUGaussSeidelSmoother.C:79-92: the
 * incomplete-factorisation smoother's sweeps, then Gauss-Seidel's).  rD: the
 * DIC/DILU reciprocal diagonal (unused otherwise). */
static void smoother_apply(const ldu_matrix* m, int smoother, const double* rD, double* psi, const double* b,
                           int nSweeps) {
    switch (smoother) {
        case LDU_SMOOTH_GS: ldu_gs_smooth(m, psi, b, nSweeps); break;
        case LDU_SMOOTH_SYMGS: ldu_symgs_smooth(m, psi, b, nSweeps); break;
        case LDU_SMOOTH_DIC: ldu_dic_smooth(m, rD, psi, b, nSweeps); break;
        case LDU_SMOOTH_DILU: ldu_dilu_smooth(m, rD, psi, b, nSweeps); break;
        case LDU_SMOOTH_DICGS:
            ldu_dic_smooth(m, rD, psi, b, nSweeps);
            ldu_gs_smooth(m, psi, b, nSweeps);
            break;
        default:
            ldu_dilu_smooth(m, rD, psi, b, nSweeps);
            ldu_gs_smooth(m, psi, b, nSweeps);
            break;
    }
}

static double* smoother_rD(const ldu_matrix* m, int smoother) {
    if (smoother == LDU_SMOOTH_GS || smoother == LDU_SMOOTH_SYMGS) return NULL;
    double* rD = (double*)xmalloc(sizeof(double) * m->nCells);
    if (smoother == LDU_SMOOTH_DIC || smoother == LDU_SMOOTH_DICGS)
        ldu_dic_rD(m, rD);
    else
        ldu_dilu_rD(m, rD);
    return rD;
}

void ldu_smooth(const ldu_matrix* m, int smoother, double* psi, const double* b, int nSweeps) {
    double* rD = smoother_rD(m, smoother);
    smoother_apply(m, smoother, rD, psi, b, nSweeps);
    free(rD);
}

/* ----------------------------------------------------------------- solvers */

/* SolverPerformance::checkConvergence, SolverPerformance.C:60-92 */
static int check_convergence(ldu_perf* p, const ldu_controls* c) {
    p->converged = (p->finalResidual < c->tolerance ||
                    (c->relTol > SP_SMALL && p->finalResidual < c->relTol * p->initialResidual));
    return p->converged;
}

/* SolverPerformance::checkSingularity, SolverPerformance.C:32-44 */
static int check_singularity(ldu_perf* p, double v) {
    p->singular = v < VSMALL;
    return p->singular;
}

/* PCG::solve, PCG.C:65-193 */
int ldu_pcg(const ldu_matrix* m, double* psi, const double* b, const ldu_controls* c,
            int precond, ldu_perf* perf) {
    const int n = m->nCells;
    double* pA = (double*)xmalloc(sizeof(double) * n);
    double* wA = (double*)xmalloc(sizeof(double) * n);
    double* rA = (double*)xmalloc(sizeof(double) * n);
    memset(perf, 0, sizeof(*perf));
    double wArA = SP_GREAT, wArAold = wArA;
    ldu_amul(m, psi, wA);
    for (int i = 0; i < n; ++i) rA[i] = b[i] - wA[i];
    const double normFactor = ldu_norm_factor(m, psi, b, wA, pA);
    perf->initialResidual = ldu_sum_mag(n, rA) / normFactor;
    perf->finalResidual = perf->initialResidual;
    if (c->minIter > 0 || !check_convergence(perf, c)) {
        precon P;
        precon_init(&P, m, precond);
        do {
            wArAold = wArA;
            precon_apply(&P, m, wA, rA);
            wArA = ldu_sum_prod(n, wA, rA);
            if (perf->nIterations == 0) {
                for (int i = 0; i < n; ++i) pA[i] = wA[i];
            } else {
                const double beta = wArA / wArAold;
                for (int i = 0; i < n; ++i) pA[i] = wA[i] + beta * pA[i];
            }
            ldu_amul(m, pA, wA);
            const double wApA = ldu_sum_prod(n, wA, pA);
            if (check_singularity(perf, fabs(wApA) / normFactor)) break;
            const double alpha = wArA / wApA;
            for (int i = 0; i < n; ++i) {
                psi[i] += alpha * pA[i];
                rA[i] -= alpha * wA[i];
            }
            perf->finalResidual = ldu_sum_mag(n, rA) / normFactor;
        } while ((++perf->nIterations < c->maxIter && !check_convergence(perf, c)) ||
                 perf->nIterations < c->minIter);
        free(P.rD);
    }
    free(pA);
    free(wA);
    free(rA);
    return 0;
}

/* DILUPreconditioner::preconditionT, DILUPreconditioner.C:138-185: forward
 * over the faces in order with the upper coefficients, backward over the
 * faces in reverse losort order with the lower ones. */
static void dilu_precondition_t(const ldu_matrix* m, const double* rD, const double* r, double* w) {
    const int n = m->nCells, nf = m->nFaces;
    const double* lo = lowerOf(m);
    for (int c = 0; c < n; ++c) w[c] = rD[c] * r[c];
    for (int f = 0; f < nf; ++f) w[m->u[f]] -= rD[m->u[f]] * m->upper[f] * w[m->l[f]];
    for (int f = nf - 1; f >= 0; --f) {
        const int sf = m->losort[f];
        w[m->l[sf]] -= rD[m->l[sf]] * lo[sf] * w[m->u[sf]];
    }
}

/* preconditionT of none / diagonal is precondition (noPreconditioner.H:89-97,
 * diagonalPreconditioner.H:97-105) */
static void precon_apply_t(const precon* p, const ldu_matrix* m, double* w, const double* r) {
    if (p->kind == LDU_PRE_DILU)
        dilu_precondition_t(m, p->rD, r, w);
    else
        precon_apply(p, m, w, r);
}

int ldu_pbicg(const ldu_matrix* m, double* psi, const double* b, const ldu_controls* c, int precond,
              ldu_perf* perf) {
    const int n = m->nCells;
    double* pA = (double*)xmalloc(sizeof(double) * n);
    double* wA = (double*)xmalloc(sizeof(double) * n);
    double* rA = (double*)xmalloc(sizeof(double) * n);
    memset(perf, 0, sizeof(*perf));
    ldu_amul(m, psi, wA);
    for (int i = 0; i < n; ++i) rA[i] = b[i] - wA[i];
    const double normFactor = ldu_norm_factor(m, psi, b, wA, pA);
    perf->initialResidual = ldu_sum_mag(n, rA) / normFactor;
    perf->finalResidual = perf->initialResidual;
    if (c->minIter > 0 || !check_convergence(perf, c)) {
        double* pT = (double*)calloc(n ? n : 1, sizeof(double));
        double* wT = (double*)xmalloc(sizeof(double) * n);
        double* rT = (double*)xmalloc(sizeof(double) * n);
        ldu_tmul(m, psi, wT);
        for (int i = 0; i < n; ++i) rT[i] = b[i] - wT[i];
        double wArT = 0;
        precon P;
        precon_init(&P, m, precond);
        do {
            const double wArTold = wArT;
            precon_apply(&P, m, wA, rA);
            precon_apply_t(&P, m, wT, rT);
            wArT = ldu_sum_prod(n, wA, rT);
            if (perf->nIterations == 0) {
                for (int i = 0; i < n; ++i) {
                    pA[i] = wA[i];
                    pT[i] = wT[i];
                }
            } else {
                const double beta = wArT / wArTold;
                for (int i = 0; i < n; ++i) {
                    pA[i] = wA[i] + beta * pA[i];
                    pT[i] = wT[i] + beta * pT[i];
                }
            }
            ldu_amul(m, pA, wA);
            ldu_tmul(m, pT, wT);
            const double wApT = ldu_sum_prod(n, wA, pT);
            if (check_singularity(perf, fabs(wApT) / normFactor)) break;
            const double alpha = wArT / wApT;
            for (int i = 0; i < n; ++i) {
                psi[i] += alpha * pA[i];
                rA[i] -= alpha * wA[i];
                rT[i] -= alpha * wT[i];
            }
            perf->finalResidual = ldu_sum_mag(n, rA) / normFactor;
        } while ((++perf->nIterations < c->maxIter && !check_convergence(perf, c)) ||
                 perf->nIterations < c->minIter);
        free(P.rD);
        free(pT);
        free(wT);
        free(rT);
    }
    free(pA);
    free(wA);
    free(rA);
    const int lim = c->maxIter > 1000 ? c->maxIter : 1000;
    return perf->nIterations > lim ? -2 : 0;
}

/* PBiCGStab::solve, PBiCGStab.C:68-254 */
int ldu_pbicgstab(const ldu_matrix* m, double* psi, const double* b, const ldu_controls* c,
                  int precond, ldu_perf* perf) {
    const int n = m->nCells;
    double* pA = (double*)xmalloc(sizeof(double) * n);
    double* yA = (double*)xmalloc(sizeof(double) * n);
    double* rA = (double*)xmalloc(sizeof(double) * n);
    memset(perf, 0, sizeof(*perf));
    ldu_amul(m, psi, yA);
    for (int i = 0; i < n; ++i) rA[i] = b[i] - yA[i];
    const double normFactor = ldu_norm_factor(m, psi, b, yA, pA);
    perf->initialResidual = ldu_sum_mag(n, rA) / normFactor;
    perf->finalResidual = perf->initialResidual;
    if (c->minIter > 0 || !check_convergence(perf, c)) {
        double* AyA = (double*)xmalloc(sizeof(double) * n);
        double* sA = (double*)xmalloc(sizeof(double) * n);
        double* zA = (double*)xmalloc(sizeof(double) * n);
        double* tA = (double*)xmalloc(sizeof(double) * n);
        double* rA0 = (double*)xmalloc(sizeof(double) * n);
        memcpy(rA0, rA, sizeof(double) * n);
        double rA0rA = 0, alpha = 0, omega = 0;
        precon P;
        precon_init(&P, m, precond);
        do {
            const double rA0rAold = rA0rA;
            rA0rA = ldu_sum_prod(n, rA0, rA);
            if (check_singularity(perf, fabs(rA0rA))) break;
            if (perf->nIterations == 0) {
                for (int i = 0; i < n; ++i) pA[i] = rA[i];
            } else {
                if (check_singularity(perf, fabs(omega))) break;
                const double beta = (rA0rA / rA0rAold) * (alpha / omega);
                for (int i = 0; i < n; ++i) pA[i] = rA[i] + beta * (pA[i] - omega * AyA[i]);
            }
            precon_apply(&P, m, yA, pA);
            ldu_amul(m, yA, AyA);
            const double rA0AyA = ldu_sum_prod(n, rA0, AyA);
            alpha = rA0rA / rA0AyA;
            for (int i = 0; i < n; ++i) sA[i] = rA[i] - alpha * AyA[i];
            perf->finalResidual = ldu_sum_mag(n, sA) / normFactor;
            if (++perf->nIterations >= c->minIter && check_convergence(perf, c)) {
                for (int i = 0; i < n; ++i) psi[i] += alpha * yA[i];
                break;
            }
            precon_apply(&P, m, zA, sA);
            ldu_amul(m, zA, tA);
            const double tAtA = ldu_sum_sqr(n, tA);
            omega = ldu_sum_prod(n, tA, sA) / tAtA;
            for (int i = 0; i < n; ++i) {
                psi[i] += alpha * yA[i] + omega * zA[i];
                rA[i] = sA[i] - omega * tA[i];
            }
            perf->finalResidual = ldu_sum_mag(n, rA) / normFactor;
        } while ((perf->nIterations < c->maxIter && !check_convergence(perf, c)) ||
                 perf->nIterations < c->minIter);
        free(P.rD);
        free(AyA);
        free(sA);
        free(zA);
        free(tA);
        free(rA0);
    }
    free(pA);
    free(yA);
    free(rA);
    return 0;
}

/* smoothSolver::solve, smoothSolver.C:77-196.  nSweeps < 0: that many sweeps,
 * no residuals, nIterations = -nSweeps. */
int ldu_smooth_solve(const ldu_matrix* m, double* psi, const double* b, const ldu_controls* c, int smoother,
                     int nSweeps, ldu_perf* perf) {
    const int n = m->nCells;
    memset(perf, 0, sizeof(*perf));
    if (nSweeps < 0) {
        ldu_smooth(m, smoother, psi, b, -nSweeps);
        perf->nIterations -= nSweeps;
        return 0;
    }
    double* Apsi = (double*)xmalloc(sizeof(double) * n);
    double* tmp = (double*)xmalloc(sizeof(double) * n);
    ldu_amul(m, psi, Apsi);
    const double normFactor = ldu_norm_factor(m, psi, b, Apsi, tmp);
    double s = 0;
    for (int i = 0; i < n; ++i) s += fabs(b[i] - Apsi[i]);
    perf->initialResidual = s / normFactor;
    perf->finalResidual = perf->initialResidual;
    if (c->minIter > 0 || !check_convergence(perf, c)) {
        double* rD = smoother_rD(m, smoother);
        do {
            smoother_apply(m, smoother, rD, psi, b, nSweeps);
            ldu_residual(m, psi, b, tmp);
            perf->finalResidual = ldu_sum_mag(n, tmp) / normFactor;
        } while (((perf->nIterations += nSweeps) < c->maxIter && !check_convergence(perf, c)) ||
                 perf->nIterations < c->minIter);
        free(rD);
    }
    free(Apsi);
    free(tmp);
    return 0;
}

/* ------------------------------------------------------------ agglomeration */

/* pairGAMGAgglomeration::agglomerate (one level), pairGAMGAgglomerate.C:123-301 */
int ldu_pair_agglomerate(int nFine, int nFaces, const int* l, const int* u,
                         const double* w, int* forward, int* map) {
    int* off = (int*)calloc(nFine + 1, sizeof(int));
    int* cnt = (int*)calloc(nFine + 1, sizeof(int));
    int* cellFaces = (int*)xmalloc(sizeof(int) * 2 * (size_t)nFaces);
    for (int f = 0; f < nFaces; ++f) cnt[u[f]]++;
    for (int f = 0; f < nFaces; ++f) cnt[l[f]]++;
    off[0] = 0;
    for (int c = 0; c < nFine; ++c) off[c + 1] = off[c] + cnt[c];
    memset(cnt, 0, sizeof(int) * (nFine + 1));
    for (int f = 0; f < nFaces; ++f) cellFaces[off[u[f]] + cnt[u[f]]++] = f;
    for (int f = 0; f < nFaces; ++f) cellFaces[off[l[f]] + cnt[l[f]]++] = f;

    for (int c = 0; c < nFine; ++c) map[c] = -1;
    int nCoarse = 0;
    const int fwd = *forward;
    for (int cf = 0; cf < nFine; ++cf) {
        const int c = fwd ? cf : nFine - cf - 1;
        if (map[c] >= 0) continue;
        int match = -1;
        double maxW = -GREAT;
        for (int k = off[c]; k < off[c + 1]; ++k) {
            const int f = cellFaces[k];
            if (map[u[f]] < 0 && map[l[f]] < 0 && w[f] > maxW) {
                match = f;
                maxW = w[f];
            }
        }
        if (match >= 0) {
            map[u[match]] = nCoarse;
            map[l[match]] = nCoarse;
            nCoarse++;
        } else {
            int cmatch = -1;
            double cmax = -GREAT;
            for (int k = off[c]; k < off[c + 1]; ++k) {
                const int f = cellFaces[k];
                if (w[f] > cmax) {
                    cmatch = f;
                    cmax = w[f];
                }
            }
            if (cmatch >= 0) {
                const int a = map[u[cmatch]], b = map[l[cmatch]];
                map[c] = a > b ? a : b;
            }
        }
    }
    for (int cf = 0; cf < nFine; ++cf) {
        const int c = fwd ? cf : nFine - cf - 1;
        if (map[c] < 0) map[c] = nCoarse++;
    }
    if (!fwd) {
        nCoarse--;
        for (int c = 0; c < nFine; ++c) map[c] = nCoarse - map[c];
        nCoarse++;
    }
    *forward = !fwd;
    free(off);
    free(cnt);
    free(cellFaces);
    return nCoarse;
}

/* GAMGAgglomeration::agglomerateLduAddressing, GAMGAgglomerateLduAddressing.C:32-222 */
int ldu_agglomerate_addressing(int nCells, int nFaces, const int* l, const int* u,
                               const int* rm, int nCoarse, int* cl, int* cu,
                               int* fra, int* flip) {
    (void)nCells;
    int maxNnbrs = 10;
    int* cCellnFaces = (int*)calloc(nCoarse, sizeof(int));
    int* cCellFaces = (int*)xmalloc(sizeof(int) * (size_t)maxNnbrs * nCoarse);
    int* initNeighb = (int*)xmalloc(sizeof(int) * nFaces);
    int nCoarseFaces = 0;
    for (int f = 0; f < nFaces; ++f) {
        const int rU = rm[u[f]], rL = rm[l[f]];
        if (rU == rL) {
            fra[f] = -(rU + 1);
            continue;
        }
        int cOwn = rU, cNei = rL;
        if (rU > rL) {
            cOwn = rL;
            cNei = rU;
        }
        int* cc = &cCellFaces[(size_t)maxNnbrs * cOwn];
        int found = 0;
        for (int i = 0; i < cCellnFaces[cOwn]; ++i) {
            if (initNeighb[cc[i]] == cNei) {
                found = 1;
                fra[f] = cc[i];
                break;
            }
        }
        if (!found) {
            if (cCellnFaces[cOwn] >= maxNnbrs) {
                const int oldMax = maxNnbrs;
                maxNnbrs *= 2;
                int* grown = (int*)xmalloc(sizeof(int) * (size_t)maxNnbrs * nCoarse);
                for (int i = 0; i < nCoarse; ++i)
                    for (int j = 0; j < cCellnFaces[i]; ++j)
                        grown[(size_t)maxNnbrs * i + j] = cCellFaces[(size_t)oldMax * i + j];
                free(cCellFaces);
                cCellFaces = grown;
                cc = &cCellFaces[(size_t)maxNnbrs * cOwn];
            }
            cc[cCellnFaces[cOwn]] = nCoarseFaces;
            initNeighb[nCoarseFaces] = cNei;
            fra[f] = nCoarseFaces;
            cCellnFaces[cOwn]++;
            nCoarseFaces++;
        }
    }
    /* renumber into upper-triangular order */
    int* coarseFaceMap = (int*)xmalloc(sizeof(int) * (nCoarseFaces ? nCoarseFaces : 1));
    int cf = 0;
    for (int cc = 0; cc < nCoarse; ++cc) {
        const int* faces = &cCellFaces[(size_t)maxNnbrs * cc];
        for (int i = 0; i < cCellnFaces[cc]; ++i) {
            cl[cf] = cc;
            cu[cf] = initNeighb[faces[i]];
            coarseFaceMap[faces[i]] = cf;
            cf++;
        }
    }
    for (int f = 0; f < nFaces; ++f)
        if (fra[f] >= 0) fra[f] = coarseFaceMap[fra[f]];
    for (int f = 0; f < nFaces; ++f) {
        flip[f] = 0;
        const int c = fra[f];
        if (c >= 0) {
            const int rU = rm[u[f]], rL = rm[l[f]];
            if (cl[c] == rU && cu[c] == rL) flip[f] = 1;
        }
    }
    free(cCellnFaces);
    free(cCellFaces);
    free(initNeighb);
    free(coarseFaceMap);
    return nCoarseFaces;
}

/* faceAreaPairGAMGAgglomeration.C:55-80: mag(cmptMultiply(Sf/sqrt(magSf), (1,1.01,1.02)))
 * with magSf = max(mag(Sf), rootVSmall) (primitiveMeshFaceCentresAndAreas.C:93). */
void ldu_face_area_pair_weights(int nFaces, const double* Sf, double* w) {
    const double rootVSmall = sqrt(DBL_MIN);
    for (int f = 0; f < nFaces; ++f) {
        const double x = Sf[3 * f], y = Sf[3 * f + 1], z = Sf[3 * f + 2];
        double m = sqrt(x * x + y * y + z * z);
        if (m < rootVSmall) m = rootVSmall;
        const double s = sqrt(m);
        const double a = (x / s) * 1.0, b = (y / s) * 1.01, c = (z / s) * 1.02;
        w[f] = sqrt(a * a + b * b + c * c);
    }
}

/* pairGAMGAgglomeration::agglomerate(mesh, weights), pairGAMGAgglomerate.C:31-118,
 * with continueAgglomerating (GAMGAgglomeration.C:205-230) and restrictFaceField
 * (GAMGAgglomerationTemplates.C:138-167). */
int ldu_gamg_agglomerate(int nCells, int nFaces, const int* l, const int* u,
                         const double* weights, int nCellsInCoarsestLevel, int forwardStart,
                         ldu_agglomeration* agg) {
    memset(agg, 0, sizeof(*agg));
    const int maxLevels = 50;
    int forward = forwardStart;
    int fn = nCells, fnf = nFaces;
    const int *fl = l, *fu = u;
    double* fw = (double*)xmalloc(sizeof(double) * nFaces);
    memcpy(fw, weights, sizeof(double) * nFaces);
    int nCreated = 0;
    while (nCreated < maxLevels - 1) {
        int* map = (int*)xmalloc(sizeof(int) * fn);
        const int nCoarse = ldu_pair_agglomerate(fn, fnf, fl, fu, fw, &forward, map);
        if (!(nCoarse >= nCellsInCoarsestLevel && nCoarse < fn)) {
            free(map);
            break;
        }
        int* cl = (int*)xmalloc(sizeof(int) * (fnf ? fnf : 1));
        int* cu = (int*)xmalloc(sizeof(int) * (fnf ? fnf : 1));
        int* fra = (int*)xmalloc(sizeof(int) * (fnf ? fnf : 1));
        int* flip = (int*)xmalloc(sizeof(int) * (fnf ? fnf : 1));
        const int ncf = ldu_agglomerate_addressing(fn, fnf, fl, fu, map, nCoarse, cl, cu, fra, flip);
        double* cw = (double*)calloc(ncf ? ncf : 1, sizeof(double));
        for (int f = 0; f < fnf; ++f)
            if (fra[f] >= 0) cw[fra[f]] += fw[f];
        free(fw);
        fw = cw;
        agg->nCells[nCreated] = nCoarse;
        agg->nFaces[nCreated] = ncf;
        agg->restrictAddr[nCreated] = map;
        agg->faceRestrict[nCreated] = fra;
        agg->faceFlip[nCreated] = flip;
        agg->cl[nCreated] = cl;
        agg->cu[nCreated] = cu;
        fn = nCoarse;
        fnf = ncf;
        fl = cl;
        fu = cu;
        nCreated++;
    }
    free(fw);
    agg->nLevels = nCreated;
    return nCreated > 0 ? 0 : -1;
}

void ldu_gamg_free(ldu_agglomeration* agg) {
    for (int i = 0; i < agg->nLevels; ++i) {
        free(agg->restrictAddr[i]);
        free(agg->faceRestrict[i]);
        free(agg->faceFlip[i]);
        free(agg->cl[i]);
        free(agg->cu[i]);
    }
    agg->nLevels = 0;
}

/* GAMGSolver::agglomerateMatrix, GAMGSolverAgglomerateMatrix.C:33-193 */
void ldu_gamg_coarse_matrix(int nFineCells, int nFineFaces, const double* fdiag,
                            const double* fupper, const double* flower,
                            const int* ra, const int* fra, const int* flip,
                            int nCoarseCells, int nCoarseFaces, double* cdiag, double* cupper,
                            double* clower) {
    for (int c = 0; c < nCoarseCells; ++c) cdiag[c] = 0;
    for (int i = 0; i < nFineCells; ++i) cdiag[ra[i]] += fdiag[i];
    for (int f = 0; f < nCoarseFaces; ++f) cupper[f] = 0;
    if (flower) {
        for (int f = 0; f < nCoarseFaces; ++f) clower[f] = 0;
        for (int f = 0; f < nFineFaces; ++f) {
            const int c = fra[f];
            if (c >= 0) {
                if (!flip[f]) {
                    cupper[c] += fupper[f];
                    clower[c] += flower[f];
                } else {
                    cupper[c] += flower[f];
                    clower[c] += fupper[f];
                }
            } else {
                cdiag[-1 - c] += fupper[f] + flower[f];
            }
        }
    } else {
        for (int f = 0; f < nFineFaces; ++f) {
            const int c = fra[f];
            if (c >= 0)
                cupper[c] += fupper[f];
            else
                cdiag[-1 - c] += 2 * fupper[f];
        }
    }
}

/* -------------------------------------------------------------------- GAMG */

void ldu_gamg_default_controls(ldu_gamg_controls* g) {
    /* GAMGSolver.C:70-80 */
    g->nPreSweeps = 0;
    g->preSweepsLevelMultiplier = 1;
    g->maxPreSweeps = 4;
    g->nPostSweeps = 2;
    g->postSweepsLevelMultiplier = 1;
    g->maxPostSweeps = 4;
    g->nFinestSweeps = 2;
    g->scaleCorrection = -1;
    g->smoother = LDU_SMOOTH_GS;
    g->interpolateCorrection = 0;
    g->directSolveCoarsest = 0;
}

typedef struct {
    ldu_matrix m;
    double* diag;
    double* upper;
    double* lower;
    double* rD; /* DIC smoother */
    /* the level's coupled interfaces (cyclicGAMGInterface) */
    int *ifCell, *ifNbr, *ifPatchSize;
    double *ifBou, *ifInt;
} level_matrix;

/* Coarse cyclic interfaces of one GAMG level from the finer level's and its
 * restriction map R: cyclicGAMGInterface's constructor
 * (cyclicGAMGInterface.C:87-151) groups each patch's faces by the pair
 * (coarse cell, coarse neighbour cell) in order of first appearance, the
 * neighbour cells coming from the partner patch (internalFieldTransfer of
 * the restrict map, cyclicGAMGInterface.C:172-189: the same pair read from
 * the other side); the coefficients are summed over each coarse face's fine
 * faces in face order (GAMGSolverAgglomerateMatrix.C:196-268 restrictField,
 * GAMGInterface.C:90-115). */
static void coarse_interfaces(const ldu_matrix* fine, const int* R, level_matrix* L, int* toCoarse) {
    const int nIf = fine->nIf;
    const int nP = fine->nIfPatch > 0 ? fine->nIfPatch : 1;
    L->ifCell = (int*)xmalloc(sizeof(int) * nIf);
    L->ifNbr = (int*)xmalloc(sizeof(int) * nIf);
    L->ifBou = (double*)xmalloc(sizeof(double) * nIf);
    L->ifInt = (double*)xmalloc(sizeof(double) * nIf);
    L->ifPatchSize = (int*)xmalloc(sizeof(int) * nP);
    int off = 0, nc = 0;
    for (int p = 0; p < nP; ++p) {
        const int np = fine->nIfPatch > 0 ? fine->ifPatchSize[p] : nIf;
        const int c0 = nc;
        for (int k = off; k < off + np; ++k) {
            const int a = R[fine->ifCell[k]], b = R[fine->ifNbr[k]];
            int j = c0;
            while (j < nc && !(L->ifCell[j] == a && L->ifNbr[j] == b)) ++j;
            if (j == nc) {
                L->ifCell[nc] = a;
                L->ifNbr[nc] = b;
                L->ifBou[nc] = 0.0;
                L->ifInt[nc] = 0.0;
                ++nc;
            }
            L->ifBou[j] += fine->ifBou[k];
            L->ifInt[j] += fine->ifInt ? fine->ifInt[k] : fine->ifBou[k];
            if (toCoarse) toCoarse[k] = j;
        }
        L->ifPatchSize[p] = nc - c0;
        off += np;
    }
    L->m.nIf = nc;
    L->m.ifCell = L->ifCell;
    L->m.ifNbr = L->ifNbr;
    L->m.ifBou = L->ifBou;
    L->m.ifInt = L->ifInt;
    L->m.nIfPatch = nP;
    L->m.ifPatchSize = L->ifPatchSize;
    L->m.ifNbrPatch = fine->nIfPatch > 0 ? fine->ifNbrPatch : NULL;  /* the same patches */
}

/* GAMG's smoother on one level (any smoother of the table; rD as smoother_rD) */
static void smooth(const ldu_matrix* m, const double* rD, int kind, double* psi, const double* b, int n) {
    smoother_apply(m, kind, rD, psi, b, n);
}

/* GAMGSolver::scale, GAMGSolverScale.C:31-76 */
static void gamg_scale(const ldu_matrix* A, double* field, double* Acf, const double* source) {
    const int n = A->nCells;
    ldu_amul(A, field, Acf);
    double num = 0, den = 0;
    for (int i = 0; i < n; ++i) {
        num += source[i] * field[i];
        den += Acf[i] * field[i];
    }
    /* stabilise(den, vSmall), src/OpenFOAM/primitives/Scalar/Scalar.H:367-377 */
    const double st = den >= 0 ? den + VSMALL : den - VSMALL;
    const double sf = num / st;
    for (int i = 0; i < n; ++i) field[i] = sf * field[i] + (source[i] - sf * Acf[i]) / A->diag[i];
}

static int imin(int a, int b) { return a < b ? a : b; }

int ldu_gamg_coarse_interfaces(const int* R, int nPatch, const int* patchSize, const int* faceCells,
                               const int* nbrCells, const double* bou, int* coarsePatchSize, int* coarseFaceCells,
                               int* coarseNbrCells, double* coarseBou, int* toCoarse) {
    ldu_matrix f;
    memset(&f, 0, sizeof(f));
    int nIf = 0;
    for (int p = 0; p < nPatch; ++p) nIf += patchSize[p];
    f.nIf = nIf;
    f.ifCell = faceCells;
    f.ifNbr = nbrCells;
    f.ifBou = bou;
    f.ifInt = bou;
    f.nIfPatch = nPatch;
    f.ifPatchSize = patchSize;
    level_matrix L;
    memset(&L, 0, sizeof(L));
    if (nIf) coarse_interfaces(&f, R, &L, toCoarse);
    const int nc = L.m.nIf;
    for (int p = 0; p < nPatch && nIf; ++p) coarsePatchSize[p] = L.ifPatchSize[p];
    for (int j = 0; j < nc; ++j) {
        coarseFaceCells[j] = L.ifCell[j];
        coarseNbrCells[j] = L.ifNbr[j];
        coarseBou[j] = L.ifBou[j];
    }
    free(L.ifCell);
    free(L.ifNbr);
    free(L.ifPatchSize);
    free(L.ifBou);
    free(L.ifInt);
    return nc;
}

/* The GAMG hierarchy of one solve: coarse matrices (GAMGSolver ctor,
 * GAMGSolver.C:204-206), the smoothers' reciprocal diagonals and the coarse
 * correction and source fields (initVcycle, GAMGSolverSolve.C:446-517). */
int ldu_lu_decompose(int n, double* A, int* piv) {
    double* vv = (double*)xmalloc(sizeof(double) * (n ? n : 1));
    /* implicit scaling: 1 / the largest magnitude of each row */
    for (int i = 0; i < n; ++i) {
        double big = 0.0;
        for (int j = 0; j < n; ++j) {
            const double t = fabs(A[(size_t)i * n + j]);
            if (t > big) big = t;
        }
        if (big == 0.0) {
            free(vv);
            return -1;
        }
        vv[i] = 1.0 / big;
    }
    for (int j = 0; j < n; ++j) {
        /* U above the diagonal of column j, rows in ascending order */
        for (int i = 0; i < j; ++i) {
            double sum = A[(size_t)i * n + j];
            for (int k = 0; k < i; ++k) sum -= A[(size_t)i * n + k] * A[(size_t)k * n + j];
            A[(size_t)i * n + j] = sum;
        }
        /* the rest of the column; pivot: the last row of largest scaled magnitude */
        int iMax = 0;
        double big = 0.0;
        for (int i = j; i < n; ++i) {
            double sum = A[(size_t)i * n + j];
            for (int k = 0; k < j; ++k) sum -= A[(size_t)i * n + k] * A[(size_t)k * n + j];
            A[(size_t)i * n + j] = sum;
            const double t = vv[i] * fabs(sum);
            if (t >= big) {
                big = t;
                iMax = i;
            }
        }
        piv[j] = iMax;
        if (j != iMax) {
            for (int k = 0; k < n; ++k) {
                const double t = A[(size_t)j * n + k];
                A[(size_t)j * n + k] = A[(size_t)iMax * n + k];
                A[(size_t)iMax * n + k] = t;
            }
            vv[iMax] = vv[j];
        }
        if (A[(size_t)j * n + j] == 0.0) A[(size_t)j * n + j] = DBL_EPSILON;
        if (j != n - 1) {
            const double rDiag = 1.0 / A[(size_t)j * n + j];
            for (int i = j + 1; i < n; ++i) A[(size_t)i * n + j] *= rDiag;
        }
    }
    free(vv);
    return 0;
}

void ldu_lu_backsubstitute(int n, const double* LU, const int* piv, double* x) {
    /* forward: unit-lower L with the row interchanges; the first nonzero
     * entry starts the sums (ii) */
    int ii = 0;
    for (int i = 0; i < n; ++i) {
        const int ip = piv[i];
        double sum = x[ip];
        x[ip] = x[i];
        if (ii != 0) {
            for (int j = ii - 1; j < i; ++j) sum -= LU[(size_t)i * n + j] * x[j];
        } else if (sum != 0.0) {
            ii = i + 1;
        }
        x[i] = sum;
    }
    for (int i = n - 1; i >= 0; --i) {
        double sum = x[i];
        for (int j = i + 1; j < n; ++j) sum -= LU[(size_t)i * n + j] * x[j];
        x[i] = sum / LU[(size_t)i * n + i];
    }
}

typedef struct {
    const ldu_matrix* m;
    const ldu_agglomeration* agg;
    const ldu_gamg_controls* gc;
    int nl, coarsest, sym, scaleCorrection, maxSize;
    level_matrix* lv;
    double **corr, **src;
    double* rD0;
    double* lu; /* directSolveCoarsest: the factorised coarsest matrix */
    int* piv;
    int singular;
} gamg_hier;

/* LUscalarMatrix::convert (LUscalarMatrix.C:205-266, no interfaces): the
 * dense row-major matrix of an LDU matrix (lower = upper when symmetric). */
/* The direct coarsest solve takes interfaces when every patch names a
 * partner patch with as many faces (at most 64 patches). */
static int lu_interfaces_ok(const ldu_matrix* m) {
    if (!m->nIf) return 1;
    if (m->nIfPatch <= 0 || m->nIfPatch > 64 || !m->ifNbrPatch) return 0;
    for (int p = 0; p < m->nIfPatch; ++p) {
        const int q = m->ifNbrPatch[p];
        if (q < 0 || q >= m->nIfPatch || m->ifPatchSize[q] != m->ifPatchSize[p]) return 0;
    }
    return 1;
}

/* LUscalarMatrix::convert (LUscalarMatrix.C:205-265): the dense matrix,
 * then per cyclic patch p and face f, A[faceCells_p[f]][faceCells_q[f]] -=
 * interfaceBouCoeffs_q[f] with q the partner patch (the partner's
 * coefficient, as the reference takes it), in patch then face order. */
static void lu_dense(const ldu_matrix* m, double* A) {
    const int n = m->nCells;
    const double* lower = m->lower ? m->lower : m->upper;
    memset(A, 0, sizeof(double) * (size_t)n * n);
    for (int c = 0; c < n; ++c) A[(size_t)c * n + c] = m->diag[c];
    for (int f = 0; f < m->nFaces; ++f) {
        A[(size_t)m->u[f] * n + m->l[f]] = lower[f];
        A[(size_t)m->l[f] * n + m->u[f]] = m->upper[f];
    }
    if (!m->nIf || !lu_interfaces_ok(m)) return;
    int off[64];
    for (int p = 0, o = 0; p < m->nIfPatch && p < 64; ++p) {
        off[p] = o;
        o += m->ifPatchSize[p];
    }
    for (int p = 0; p < m->nIfPatch; ++p) {
        const int q = m->ifNbrPatch[p];
        for (int f = 0; f < m->ifPatchSize[p]; ++f)
            A[(size_t)m->ifCell[off[p] + f] * n + m->ifCell[off[q] + f]] -= m->ifBou[off[q] + f];
    }
}



static void gamg_setup(gamg_hier* H, const ldu_matrix* m, const ldu_agglomeration* agg,
                       const ldu_gamg_controls* gc) {
    const int n = m->nCells;
    const int nl = agg->nLevels;
    H->m = m;
    H->agg = agg;
    H->gc = gc;
    H->nl = nl;
    H->coarsest = nl - 1;
    H->sym = m->lower == NULL;
    H->scaleCorrection = gc->scaleCorrection < 0 ? H->sym : gc->scaleCorrection;
    H->lv = (level_matrix*)calloc(nl, sizeof(level_matrix));
    const ldu_matrix* fine = m;
    int maxSize = n;
    for (int i = 0; i < nl; ++i) {
        const int nc = agg->nCells[i], ncf = agg->nFaces[i];
        if (nc > maxSize) maxSize = nc;
        level_matrix* L = &H->lv[i];
        L->diag = (double*)xmalloc(sizeof(double) * nc);
        L->upper = (double*)xmalloc(sizeof(double) * (ncf ? ncf : 1));
        L->lower = H->sym ? NULL : (double*)xmalloc(sizeof(double) * (ncf ? ncf : 1));
        ldu_gamg_coarse_matrix(fine->nCells, fine->nFaces, fine->diag, fine->upper,
                               H->sym ? NULL : fine->lower, agg->restrictAddr[i], agg->faceRestrict[i],
                               agg->faceFlip[i], nc, ncf, L->diag, L->upper, L->lower);
        L->m.nCells = nc;
        L->m.nFaces = ncf;
        L->m.l = agg->cl[i];
        L->m.u = agg->cu[i];
        L->m.diag = L->diag;
        L->m.upper = L->upper;
        L->m.lower = L->lower;
        if (fine->nIf) coarse_interfaces(fine, agg->restrictAddr[i], L, NULL);
        ldu_init_addr(&L->m);
        fine = &L->m;
    }
    H->maxSize = maxSize;
    H->corr = (double**)calloc(nl, sizeof(double*));
    H->src = (double**)calloc(nl, sizeof(double*));
    H->rD0 = smoother_rD(m, gc->smoother);
    for (int i = 0; i < nl; ++i) {
        H->corr[i] = (double*)xmalloc(sizeof(double) * agg->nCells[i]);
        H->src[i] = (double*)xmalloc(sizeof(double) * agg->nCells[i]);
        H->lv[i].rD = smoother_rD(&H->lv[i].m, gc->smoother);
    }
    H->lu = NULL;
    H->piv = NULL;
    H->singular = 0;
    if (gc->directSolveCoarsest) {
        const level_matrix* L = &H->lv[nl - 1];
        const int nc = L->m.nCells;
        H->lu = (double*)xmalloc(sizeof(double) * ((size_t)nc * nc + 1));
        H->piv = (int*)xmalloc(sizeof(int) * (nc + 1));
        lu_dense(&L->m, H->lu);
        H->singular = ldu_lu_decompose(nc, H->lu, H->piv) != 0;
    }
}

static void gamg_free(gamg_hier* H) {
    for (int i = 0; i < H->nl; ++i) {
        free(H->corr[i]);
        free(H->src[i]);
        free(H->lv[i].rD);
        free(H->lv[i].diag);
        free(H->lv[i].upper);
        free(H->lv[i].lower);
        free(H->lv[i].ifCell);
        free(H->lv[i].ifNbr);
        free(H->lv[i].ifPatchSize);
        free(H->lv[i].ifBou);
        free(H->lv[i].ifInt);
        ldu_free_addr(&H->lv[i].m);
    }
    free(H->corr);
    free(H->src);
    free(H->rD0);
    free(H->lv);
    free(H->lu);
    free(H->piv);
}

/* GAMGSolver::interpolate, GAMGSolverInterpolate.C:30-127: one Jacobi step
 * psi = -(A - D) psi / D (the off-diagonal product from zero, in face
 * order), then every coarse cell's diagonal-weighted mean of psi is replaced
 * by psiC (ra: this level's restriction map, nCC coarse cells).  Apsi:
 * scratch of m's size. */
static void gamg_interpolate(const ldu_matrix* m, double* psi, double* Apsi, const int* ra, const double* psiC,
                             int nCC) {
    const int n = m->nCells;
    const double* lower = m->lower ? m->lower : m->upper;
    for (int c = 0; c < n; ++c) Apsi[c] = 0;
    for (int f = 0; f < m->nFaces; ++f) {
        Apsi[m->u[f]] += lower[f] * psi[m->l[f]];
        Apsi[m->l[f]] += m->upper[f] * psi[m->u[f]];
    }
    /* the interfaces' updateMatrixInterfaces (GAMGSolverInterpolate.C:60-67) */
    update_interfaces(m, m->ifBou, 0, psi, Apsi);
    for (int c = 0; c < n; ++c) psi[c] = -Apsi[c] / m->diag[c];
    double* corrC = (double*)calloc(nCC ? nCC : 1, sizeof(double));
    double* diagC = (double*)calloc(nCC ? nCC : 1, sizeof(double));
    for (int c = 0; c < n; ++c) {
        corrC[ra[c]] += m->diag[c] * psi[c];
        diagC[ra[c]] += m->diag[c];
    }
    for (int k = 0; k < nCC; ++k) corrC[k] = psiC[k] - corrC[k] / diagC[k];
    for (int c = 0; c < n; ++c) psi[c] += corrC[ra[c]];
    free(corrC);
    free(diagC);
}

/* GAMGSolver::Vcycle, GAMGSolverSolve.C:148-443: psi += the coarse-grid
 * correction of finestResidual, then the finest level's smoothing against
 * source b.  Apsi, finestCorrection: scratch of maxSize.  cc: the coarsest
 * level solve's tolerances (the GAMG object's own). */
static void gamg_vcycle(gamg_hier* H, double* psi, const double* b, double* Apsi, double* finestCorrection,
                        const double* finestResidual, const ldu_controls* cc) {
    const ldu_matrix* m = H->m;
    const ldu_agglomeration* agg = H->agg;
    const ldu_gamg_controls* gc = H->gc;
    const int n = m->nCells, coarsest = H->coarsest, scaleCorrection = H->scaleCorrection;
    level_matrix* lv = H->lv;
    double** corr = H->corr;
    double** src = H->src;
    double* scratch1 = Apsi;
    double* scratch2 = finestCorrection;
    /* restrictField(coarseSources[0], finestResidual, 0) */
    for (int k = 0; k < agg->nCells[0]; ++k) src[0][k] = 0;
    for (int k = 0; k < n; ++k) src[0][agg->restrictAddr[0][k]] += finestResidual[k];
    for (int li = 0; li < coarsest; ++li) {
        const int nc = agg->nCells[li];
        if (gc->nPreSweeps) {
            for (int k = 0; k < nc; ++k) corr[li][k] = 0;
            smooth(&lv[li].m, lv[li].rD, gc->smoother, corr[li], src[li],
                   imin(gc->nPreSweeps + gc->preSweepsLevelMultiplier * li, gc->maxPreSweeps));
            if (scaleCorrection && li < coarsest - 1) gamg_scale(&lv[li].m, corr[li], scratch1, src[li]);
            ldu_amul(&lv[li].m, corr[li], scratch1);
            for (int k = 0; k < nc; ++k) src[li][k] -= scratch1[k];
        }
        const int nn = agg->nCells[li + 1];
        for (int k = 0; k < nn; ++k) src[li + 1][k] = 0;
        for (int k = 0; k < nc; ++k) src[li + 1][agg->restrictAddr[li + 1][k]] += src[li][k];
    }
    /* solveCoarsestLevel, GAMGSolverSolve.C:520-552 */
    if (H->lu) {
        /* LUscalarMatrix::solve: x = source, then the back-substitution */
        memcpy(corr[coarsest], src[coarsest], sizeof(double) * agg->nCells[coarsest]);
        ldu_lu_backsubstitute(agg->nCells[coarsest], H->lu, H->piv, corr[coarsest]);
    } else {
        ldu_perf cp;
        for (int k = 0; k < agg->nCells[coarsest]; ++k) corr[coarsest][k] = 0;
        if (H->sym)
            ldu_pcg(&lv[coarsest].m, corr[coarsest], src[coarsest], cc, LDU_PRE_DIC, &cp);
        else
            ldu_pbicgstab(&lv[coarsest].m, corr[coarsest], src[coarsest], cc, LDU_PRE_DILU, &cp);
    }
    for (int li = coarsest - 1; li >= 0; --li) {
        const int nc = agg->nCells[li];
        double* pre = scratch2;
        if (gc->nPreSweeps) memcpy(pre, corr[li], sizeof(double) * nc);
        for (int k = 0; k < nc; ++k) corr[li][k] = corr[li + 1][agg->restrictAddr[li + 1][k]];
        if (gc->interpolateCorrection)
            gamg_interpolate(&lv[li].m, corr[li], scratch1, agg->restrictAddr[li + 1], corr[li + 1],
                             agg->nCells[li + 1]);
        if (scaleCorrection && (gc->interpolateCorrection || li < coarsest - 1))
            gamg_scale(&lv[li].m, corr[li], scratch1, src[li]);
        if (gc->nPreSweeps)
            for (int k = 0; k < nc; ++k) corr[li][k] += pre[k];
        smooth(&lv[li].m, lv[li].rD, gc->smoother, corr[li], src[li],
               imin(gc->nPostSweeps + gc->postSweepsLevelMultiplier * li, gc->maxPostSweeps));
    }
    for (int k = 0; k < n; ++k) finestCorrection[k] = corr[0][agg->restrictAddr[0][k]];
    if (gc->interpolateCorrection)
        gamg_interpolate(m, finestCorrection, Apsi, agg->restrictAddr[0], corr[0], agg->nCells[0]);
    if (scaleCorrection) gamg_scale(m, finestCorrection, Apsi, finestResidual);
    for (int k = 0; k < n; ++k) psi[k] += finestCorrection[k];
    smooth(m, H->rD0, gc->smoother, psi, b, gc->nFinestSweeps);
}

/* GAMGSolver::solve / Vcycle / initVcycle / solveCoarsestLevel,
 * GAMGSolverSolve.C:31-552, with the coupled interfaces agglomerated level
 * by level (coarse_interfaces).  directSolveCoarsest with interfaces needs
 * each patch's partner (ifNbrPatch); without it returns -3. */
int ldu_gamg(const ldu_matrix* m, const ldu_agglomeration* agg, double* psi, const double* b,
             const ldu_controls* c, const ldu_gamg_controls* gc, ldu_perf* perf) {
    const int n = m->nCells;
    if (agg->nLevels < 1) return -1;
    if (m->nIf && gc->directSolveCoarsest && !lu_interfaces_ok(m)) return -3;
    memset(perf, 0, sizeof(*perf));
    gamg_hier H;
    gamg_setup(&H, m, agg, gc);
    if (H.singular) {
        gamg_free(&H);
        return -2;
    }
    double* Apsi = (double*)xmalloc(sizeof(double) * H.maxSize);
    double* finestCorrection = (double*)xmalloc(sizeof(double) * H.maxSize);
    double* finestResidual = (double*)xmalloc(sizeof(double) * n);
    ldu_amul(m, psi, Apsi);
    const double normFactor = ldu_norm_factor(m, psi, b, Apsi, finestCorrection);
    for (int i = 0; i < n; ++i) finestResidual[i] = b[i] - Apsi[i];
    perf->initialResidual = ldu_sum_mag(n, finestResidual) / normFactor;
    perf->finalResidual = perf->initialResidual;
    if (c->minIter > 0 || !check_convergence(perf, c)) {
        ldu_controls cc = {c->tolerance, c->relTol, 1000, 0};
        do {
            gamg_vcycle(&H, psi, b, Apsi, finestCorrection, finestResidual, &cc);
            ldu_amul(m, psi, Apsi);
            for (int k = 0; k < n; ++k) finestResidual[k] = b[k] - Apsi[k];
            perf->finalResidual = ldu_sum_mag(n, finestResidual) / normFactor;
        } while ((++perf->nIterations < c->maxIter && !check_convergence(perf, c)) ||
                 perf->nIterations < c->minIter);
    }
    gamg_free(&H);
    free(Apsi);
    free(finestCorrection);
    free(finestResidual);
    return 0;
}

/* PCG::solve (PCG.C:65-193) with GAMGPreconditioner::precondition
 * (GAMGPreconditioner.C:81-148): wA = 0, nVcycles V-cycles on A wA = rA, the
 * finest residual rA - A wA recomputed between them.  pc: the preconditioner
 * dictionary's tolerance/relTol (its coarsest-level solves). */
int ldu_pcg_gamg(const ldu_matrix* m, const ldu_agglomeration* agg, double* psi, const double* b,
                 const ldu_controls* c, const ldu_gamg_controls* gc, const ldu_controls* pc, int nVcycles,
                 ldu_perf* perf) {
    const int n = m->nCells;
    if (agg->nLevels < 1) return -1;
    if (m->nIf && gc->directSolveCoarsest && !lu_interfaces_ok(m)) return -3;
    double* pA = (double*)xmalloc(sizeof(double) * n);
    double* wA = (double*)xmalloc(sizeof(double) * n);
    double* rA = (double*)xmalloc(sizeof(double) * n);
    memset(perf, 0, sizeof(*perf));
    double wArA = SP_GREAT, wArAold = wArA;
    ldu_amul(m, psi, wA);
    for (int i = 0; i < n; ++i) rA[i] = b[i] - wA[i];
    const double normFactor = ldu_norm_factor(m, psi, b, wA, pA);
    perf->initialResidual = ldu_sum_mag(n, rA) / normFactor;
    perf->finalResidual = perf->initialResidual;
    if (c->minIter > 0 || !check_convergence(perf, c)) {
        gamg_hier H;
        gamg_setup(&H, m, agg, gc);
        double* AwA = (double*)xmalloc(sizeof(double) * H.maxSize);
        double* fcorr = (double*)xmalloc(sizeof(double) * H.maxSize);
        double* fres = (double*)xmalloc(sizeof(double) * n);
        const ldu_controls cc = {pc->tolerance, pc->relTol, 1000, 0};
        do {
            wArAold = wArA;
            memset(wA, 0, sizeof(double) * n);
            memcpy(fres, rA, sizeof(double) * n);
            for (int cycle = 0; cycle < nVcycles; ++cycle) {
                gamg_vcycle(&H, wA, rA, AwA, fcorr, fres, &cc);
                if (cycle < nVcycles - 1) {
                    ldu_amul(m, wA, AwA);
                    for (int i = 0; i < n; ++i) fres[i] = rA[i] - AwA[i];
                }
            }
            wArA = ldu_sum_prod(n, wA, rA);
            if (perf->nIterations == 0) {
                for (int i = 0; i < n; ++i) pA[i] = wA[i];
            } else {
                const double beta = wArA / wArAold;
                for (int i = 0; i < n; ++i) pA[i] = wA[i] + beta * pA[i];
            }
            ldu_amul(m, pA, wA);
            const double wApA = ldu_sum_prod(n, wA, pA);
            if (check_singularity(perf, fabs(wApA) / normFactor)) break;
            const double alpha = wArA / wApA;
            for (int i = 0; i < n; ++i) {
                psi[i] += alpha * pA[i];
                rA[i] -= alpha * wA[i];
            }
            perf->finalResidual = ldu_sum_mag(n, rA) / normFactor;
        } while ((++perf->nIterations < c->maxIter && !check_convergence(perf, c)) ||
                 perf->nIterations < c->minIter);
        gamg_free(&H);
        free(AwA);
        free(fcorr);
        free(fres);
    }
    free(pA);
    free(wA);
    free(rA);
    return 0;
}

/* ------------------------------------------------ finite-volume assembly */

/* An fvMatrix under construction: lduMatrix coefficient arrays (NULL while
 * unallocated, lduMatrix.C:168-212), the source and the patch
 * internal/boundary coefficients (zero-initialised, as fvMatrix's
 * constructor does). */
typedef struct {
    int nCells, nFaces, nB;
    double *diag, *upper, *lower;
    double *src, *ic, *bc;
} fvm_mat;

static void fvm_init(fvm_mat* m, const ldu_fv_geom* g) {
    m->nCells = g->nCells;
    m->nFaces = g->nFaces;
    m->nB = g->nBoundary;
    m->diag = m->upper = m->lower = NULL;
    m->src = (double*)calloc(g->nCells ? g->nCells : 1, sizeof(double));
    m->ic = (double*)calloc(g->nBoundary ? g->nBoundary : 1, sizeof(double));
    m->bc = (double*)calloc(g->nBoundary ? g->nBoundary : 1, sizeof(double));
}

static void fvm_free(fvm_mat* m) {
    free(m->diag);
    free(m->upper);
    free(m->lower);
    free(m->src);
    free(m->ic);
    free(m->bc);
}

static double* dup_or_zero(const double* a, int n) {
    double* p = (double*)calloc(n ? n : 1, sizeof(double));
    if (a) memcpy(p, a, sizeof(double) * n);
    return p;
}

/* lduMatrix::diag() / upper() / lower(): allocate on first use (a copy of
 * the other triangle when it exists) */
static double* fvm_diag(fvm_mat* m) {
    if (!m->diag) m->diag = dup_or_zero(NULL, m->nCells);
    return m->diag;
}
static double* fvm_upper(fvm_mat* m) {
    if (!m->upper) m->upper = dup_or_zero(m->lower, m->nFaces);
    return m->upper;
}
static double* fvm_lower(fvm_mat* m) {
    if (!m->lower) m->lower = dup_or_zero(m->upper, m->nFaces);
    return m->lower;
}

/* lduMatrix::negSumDiag, lduMatrixOperations.C:55-74 */
static void fvm_neg_sum_diag(fvm_mat* m, const ldu_fv_geom* g) {
    if (!m->lower && !m->upper) return;
    const double* Lower = m->lower ? m->lower : m->upper;
    const double* Upper = m->upper ? m->upper : m->lower;
    double* d = fvm_diag(m);
    for (int f = 0; f < g->nFaces; ++f) {
        d[g->l[f]] -= Lower[f];
        d[g->u[f]] -= Upper[f];
    }
}

/* fvMatrix::negate, fvMatrix.C:1079-1090 */
static void fvm_negate(fvm_mat* m) {
    if (m->lower)
        for (int f = 0; f < m->nFaces; ++f) m->lower[f] = -m->lower[f];
    if (m->upper)
        for (int f = 0; f < m->nFaces; ++f) m->upper[f] = -m->upper[f];
    if (m->diag)
        for (int c = 0; c < m->nCells; ++c) m->diag[c] = -m->diag[c];
    for (int c = 0; c < m->nCells; ++c) m->src[c] = -m->src[c];
    for (int b = 0; b < m->nB; ++b) {
        m->ic[b] = -m->ic[b];
        m->bc[b] = -m->bc[b];
    }
}

static void axpy_sign(int n, double s, const double* a, double* y) {
    if (s > 0)
        for (int i = 0; i < n; ++i) y[i] += a[i];
    else
        for (int i = 0; i < n; ++i) y[i] -= a[i];
}

/* fvMatrix::operator+= / -= (s = +1 / -1): lduMatrix::operator+=/-=
 * (lduMatrixOperations.C:159-318) on the coefficients, then the source and
 * the patch coefficients */
static void fvm_add(fvm_mat* C, const fvm_mat* A, double s) {
    const int nf = C->nFaces;
    if (A->diag) axpy_sign(C->nCells, s, A->diag, fvm_diag(C));
    const int cSym = C->diag && !C->lower && C->upper, cAsym = C->diag && C->lower && C->upper;
    const int cDiagonal = C->diag && !C->lower && !C->upper;
    const int aSym = A->diag && !A->lower && A->upper, aAsym = A->diag && A->lower && A->upper;
    if (cSym && aSym) {
        axpy_sign(nf, s, A->upper, fvm_upper(C));
    } else if (cSym && aAsym) {
        fvm_lower(C);
        axpy_sign(nf, s, A->upper, fvm_upper(C));
        axpy_sign(nf, s, A->lower, fvm_lower(C));
    } else if (cAsym && aSym) {
        const double* a = A->upper ? A->upper : A->lower;
        axpy_sign(nf, s, a, fvm_lower(C));
        axpy_sign(nf, s, a, fvm_upper(C));
    } else if (cAsym && aAsym) {
        axpy_sign(nf, s, A->lower, fvm_lower(C));
        axpy_sign(nf, s, A->upper, fvm_upper(C));
    } else if (cDiagonal) {
        if (A->upper) {
            double* u = fvm_upper(C);
            for (int f = 0; f < nf; ++f) u[f] = s > 0 ? A->upper[f] : -A->upper[f];
        }
        if (A->lower) {
            double* l = fvm_lower(C);
            for (int f = 0; f < nf; ++f) l[f] = s > 0 ? A->lower[f] : -A->lower[f];
        }
    }
    axpy_sign(C->nCells, s, A->src, C->src);
    axpy_sign(C->nB, s, A->ic, C->ic);
    axpy_sign(C->nB, s, A->bc, C->bc);
}

/* EulerDdtScheme::fvmDdt, EulerDdtScheme.C:466-497 (static mesh) */
static void fvm_ddt(fvm_mat* m, const ldu_fv_geom* g, double rDeltaT, const double* psi0) {
    double* d = fvm_diag(m);
    for (int c = 0; c < g->nCells; ++c) {
        d[c] = rDeltaT * g->V[c];
        m->src[c] = rDeltaT * psi0[c] * g->V[c];
    }
}

/* gaussConvectionScheme::fvmDiv, gaussConvectionScheme.C:121-152, with the
 * upwind (upwind.H: pos0(faceFlux)) or linear (mesh weights) interpolation
 * weights; the patch value coefficients of fixedValue (0, value),
 * zeroGradient (1, 0) and fixedGradient (1, gradient/deltaCoeffs) */
static void fvm_div(fvm_mat* m, const ldu_fv_geom* g, const ldu_fvm_terms* t) {
    double* lo = fvm_lower(m);
    for (int f = 0; f < g->nFaces; ++f) {
        const double w = t->divScheme == LDU_DIV_UPWIND ? (t->phi[f] >= 0.0 ? 1.0 : 0.0) : g->weights[f];
        lo[f] = -w * t->phi[f];
    }
    double* up = fvm_upper(m);
    for (int f = 0; f < g->nFaces; ++f) up[f] = lo[f] + t->phi[f];
    fvm_neg_sum_diag(m, g);
    for (int b = 0; b < g->nBoundary; ++b) {
        const int type = t->bcType[b];
        if (type == LDU_BC_CYCLIC) {
            /* coupledFvPatchField::valueInternalCoeffs / valueBoundaryCoeffs:
             * (w, 1 - w), upwind w = pos0(phi) */
            const double w = t->phiB[b] >= 0.0 ? 1.0 : 0.0;
            m->ic[b] = t->phiB[b] * (1.0 * w);
            m->bc[b] = -t->phiB[b] * (1.0 * (1.0 - w));
            continue;
        }
        const double vic = type == LDU_BC_FIXED_VALUE ? 0.0 : 1.0;
        const double vbc = type == LDU_BC_FIXED_VALUE ? t->bcValue[b]
                           : type == LDU_BC_FIXED_GRADIENT ? t->bcValue[b] / g->deltaCoeffsB[b]
                                                           : 0.0;
        m->ic[b] = t->phiB[b] * vic;
        m->bc[b] = -t->phiB[b] * vbc;
    }
}

/* gaussLaplacianScheme::fvmLaplacian (gaussLaplacianSchemes.C:35-90) with
 * fvmLaplacianUncorrected (gaussLaplacianScheme.C:47-89): gammaMagSf =
 * gamma*magSf; the patch gradient coefficients of fixedValue
 * (-deltaCoeffs, deltaCoeffs*value), zeroGradient (0, 0) and fixedGradient
 * (0, gradient) */
static void fvm_laplacian(fvm_mat* m, const ldu_fv_geom* g, const ldu_fvm_terms* t) {
    double* up = fvm_upper(m);
    for (int f = 0; f < g->nFaces; ++f) {
        const double gms = (t->gamma ? t->gamma[f] : t->gammaUniform) * g->magSf[f];
        up[f] = g->deltaCoeffs[f] * gms;
    }
    fvm_neg_sum_diag(m, g);
    for (int b = 0; b < g->nBoundary; ++b) {
        const double gms = (t->gammaB ? t->gammaB[b] : t->gammaUniform) * g->magSfB[b];
        const int type = t->bcType[b];
        /* coupled: gradientInternalCoeffs(deltaCoeffs) = -deltaCoeffs,
         * gradientBoundaryCoeffs = minus that */
        const double gic = type == LDU_BC_FIXED_VALUE || type == LDU_BC_CYCLIC ? -1.0 * g->deltaCoeffsB[b] : 0.0;
        const double gbc = type == LDU_BC_CYCLIC ? -gic
                           : type == LDU_BC_FIXED_VALUE ? g->deltaCoeffsB[b] * t->bcValue[b]
                           : type == LDU_BC_FIXED_GRADIENT ? t->bcValue[b]
                                                           : 0.0;
        m->ic[b] = gms * gic;
        m->bc[b] = -gms * gbc;
    }
}

int ldu_fvm_assemble(const ldu_fv_geom* g, const ldu_fvm_terms* t, double* diag, double* upper, double* lower,
                     double* source) {
    return ldu_fvm_assemble_coupled(g, t, diag, upper, lower, source, NULL, NULL);
}

int ldu_fvm_assemble_coupled(const ldu_fv_geom* g, const ldu_fvm_terms* t, double* diag, double* upper,
                             double* lower, double* source, double* ifBou, double* ifInt) {
    fvm_mat C, A;
    int have = 0;
    if (t->phi && t->divScheme != LDU_DIV_UPWIND)
        for (int b = 0; b < g->nBoundary; ++b)
            if (t->bcType[b] == LDU_BC_CYCLIC) return -2;
    fvm_init(&C, g);
    if (t->rDeltaT > 0) {
        fvm_ddt(&C, g, t->rDeltaT, t->psi0);
        have = 1;
    }
    if (t->phi) {
        if (!have) {
            fvm_div(&C, g, t);
        } else {
            fvm_init(&A, g);
            fvm_div(&A, g, t);
            fvm_add(&C, &A, 1.0);
            fvm_free(&A);
        }
        have = 1;
    }
    if (t->lapSign) {
        if (!have) {
            fvm_laplacian(&C, g, t);
            if (t->lapSign < 0) fvm_negate(&C);
        } else {
            fvm_init(&A, g);
            fvm_laplacian(&A, g, t);
            fvm_add(&C, &A, t->lapSign > 0 ? 1.0 : -1.0);
            fvm_free(&A);
        }
        have = 1;
    }
    if (!have) {
        fvm_free(&C);
        return -1;
    }
    /* operator==(fvMatrix, field): source += V*su */
    if (t->su)
        for (int c = 0; c < g->nCells; ++c) C.src[c] += g->V[c] * t->su[c];
    /* fvMatrix::solveSegregated: addBoundarySource, addBoundaryDiag */
    memcpy(diag, fvm_diag(&C), sizeof(double) * g->nCells);
    memcpy(source, C.src, sizeof(double) * g->nCells);
    int k = 0;
    for (int b = 0; b < g->nBoundary; ++b) {
        diag[g->bCell[b]] += C.ic[b];
        if (t->bcType[b] != LDU_BC_CYCLIC) {
            source[g->bCell[b]] += C.bc[b];
        } else {
            if (ifBou) ifBou[k] = C.bc[b];
            if (ifInt) ifInt[k] = C.ic[b];
            ++k;
        }
    }
    const double* U = C.upper ? C.upper : C.lower;
    if (U) memcpy(upper, U, sizeof(double) * g->nFaces);
    if (lower && C.lower) memcpy(lower, C.lower, sizeof(double) * g->nFaces);
    fvm_free(&C);
    return 0;
}
