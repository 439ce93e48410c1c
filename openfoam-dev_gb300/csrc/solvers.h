// solvers.h - fused solver kernels (launchers) used by the host drivers.
#pragma once

#include "internal.h"

namespace cfx {

// Single-CTA whole-solve system description (coarsest GAMG level, batches).
template <class T>
struct BlockSys {
    int n, nf;
    const int *ownerStart, *losortStart, *losortL, *u;
    const int *fwdCells, *fwdLevelStart, *bwdCells, *bwdLevelStart;
    int nFwd, nBwd;
    const T *diag, *lp, *upper, *rD;
    const T* upPerm;  // upper[losort] for the DILU reciprocal diagonal (null: lp)
    Iface<T> itf;     // the level's coupled interfaces (start null: none)
    const T* b;
    T* psi;
    T *r, *w, *p, *q, *s, *t, *r0;  // work vectors (s, t, r0: PBiCGStab)
    double tolerance, relTol;
    int maxIter, minIter;
    int precond;   // CFX_PRE_*
    int solver;    // CFX_SOLVER_PCG / CFX_SOLVER_PBICGSTAB
    // results
    double initialResidual, finalResidual;
    int nIterations, converged, singular, pad;
};

template <class T>
struct Kern {
    // st->red0 = sum(psi) must be set; computes r = b - Apsi, normFactor,
    // initial/final residual, convergence, done; r0 copy when non-null.
    static void norm_init(cudaStream_t s, Scratch& sc, const LevelMesh& m, const LevelCoeffs<T>& a,
                          const T* Apsi, const T* b, T* r, T* r0, SolveState* st);
    // w = r (none) / rD*r (diagonal), with the w.r dot partials
    static void precond_pointwise(cudaStream_t s, int n, const T* rD, const T* r, T* w, double* partials,
                                  const int* done);
    // PCG
    static void pcg_beta(cudaStream_t s, int nPartials, const double* partials, SolveState* st);
    static void pcg_p(cudaStream_t s, int n, const T* w, T* p, const SolveState* st);
    static void pcg_amul(cudaStream_t s, Scratch& sc, const LevelMesh& m, const LevelCoeffs<T>& a, const T* p,
                         T* wA, SolveState* st);
    static void pcg_update(cudaStream_t s, Scratch& sc, int n, const T* p, const T* wA, T* psi, T* r,
                           SolveState* st);
    // PBiCG (wArA holds wArT)
    static void pbicg_p(cudaStream_t s, int n, const T* w, const T* wT, T* p, T* pT, const SolveState* st);
    static void pbicg_tmul(cudaStream_t s, Scratch& sc, const LevelMesh& m, const LevelCoeffs<T>& a, const T* pT,
                           T* wT, const T* wA, SolveState* st);
    static void pbicg_update(cudaStream_t s, Scratch& sc, int n, const T* p, const T* wA, const T* wT, T* psi,
                             T* r, T* rT, SolveState* st);
    // PBiCGStab
    static void bicg_rho(cudaStream_t s, Scratch& sc, int n, const T* r0, const T* r, SolveState* st);
    static void bicg_p(cudaStream_t s, int n, const T* r, const T* AyA, T* p, const SolveState* st);
    static void bicg_amul_alpha(cudaStream_t s, Scratch& sc, const LevelMesh& m, const LevelCoeffs<T>& a,
                                const T* yA, T* AyA, const T* r0, SolveState* st);
    static void bicg_s(cudaStream_t s, Scratch& sc, int n, const T* r, const T* AyA, T* sA, SolveState* st);
    static void bicg_early(cudaStream_t s, int n, const T* yA, T* psi, SolveState* st);
    static void bicg_amul_omega(cudaStream_t s, Scratch& sc, const LevelMesh& m, const LevelCoeffs<T>& a,
                                const T* zA, T* tA, const T* sA, SolveState* st);
    static void bicg_update(cudaStream_t s, Scratch& sc, int n, const T* yA, const T* zA, const T* sA,
                            const T* tA, T* psi, T* r, SolveState* st);
    // GAMG
    // Acf = A*field; st->sf = (source.field)/stabilise(Acf.field, vSmall)
    static void gamg_scale_sf(cudaStream_t s, Scratch& sc, const LevelMesh& m, const LevelCoeffs<T>& a,
                              const T* field, T* Acf, const T* source, SolveState* st);
    // field = sf*field + (source - sf*Acf)/diag (+ pre when non-null)
    static void gamg_scale_apply(cudaStream_t s, int n, T* field, const T* Acf, const T* source, const T* diag,
                                 const T* pre, const SolveState* st);
    // r = b - A psi; final = sum|r|/normFactor; nIterations++; loop test.
    // inc > 0: r = lduMatrix::residual and nIterations += inc (smoothSolver)
    static void gamg_residual_check(cudaStream_t s, Scratch& sc, const LevelMesh& m, const LevelCoeffs<T>& a,
                                    const T* psi, const T* b, T* r, SolveState* st, int inc = 0);
    // single-CTA whole solve of one or more small systems (blockIdx = system)
    static void block_solve(cudaStream_t s, BlockSys<T>* d_sys, int nSys, const int* done);
    // y (+)= x, predicated
    static void axpy(cudaStream_t s, int n, T a, const T* x, T* y, const int* done);
    static void copy(cudaStream_t s, int n, const T* x, T* y, const int* done);
    static void fill(cudaStream_t s, int n, T v, T* y, const int* done);
};

// A system of a batch in slot order: slot p holds cell cellOf[p], slots
// ordered by forward (lower-DAG) level, so each level of the DIC/DILU
// forward sweep is a contiguous slot range.  Neighbours are kept in ELL
// form, column-major ([j*n + p], padded with p): the faces where the cell is
// the neighbour (losort order; lower coefficients) and the faces it owns
// (face order; upper coefficients).  cnt[p] = nLower | nUpper << 16.  The
// operator and every per-cell face order are the reference's; only the
// storage order of the vectors differs.
template <class T>
struct SlotSys {
    int n, wLo, wUp, nFwd, nBwd;
    int bwdMirror;  // backward level L = forward level nFwd-1-L, same order
    const int *cnt, *loSrc, *upSrc, *cellOf;
    const int *fwdLevelStart, *bwdSlot, *bwdLevelStart;
    const T *diag, *lo, *up;  // slot order; lo/up [w*n]
    const T* upLo;            // upper[losort] in lo layout (asymmetric DILU pivots; null: lo)
    T* rD;
    T *b, *psi;               // slot order
    T *r, *w, *p, *q, *s, *t, *r0;
    const double* bCell;      // cell order (FP64 record): source in,
    double* psiCell;          // solution in/out
    double tolerance, relTol;
    int maxIter, minIter;
    int precond, solver;
    double initialResidual, finalResidual;
    int nIterations, converged, singular, nOuter;
    unsigned long long tStart, tEnd;  // %globaltimer at the system's start / end (ns)
};

// A system's result as the batch kernels publish it, when asked, to
// host-mapped memory the moment the system finishes: the fields, then a
// system-scope fence, then flag = 1 (so the system's psiCell and the fields
// are visible once the host sees the flag), letting a host thread complete
// the system while the launch runs on.  The host zeroes the flags before
// the launch.
struct BatchDone {
    double initialResidual, finalResidual;
    int nIterations, converged, singular, nOuter;
    unsigned flag, pad;
};

// Batched solves of independent systems: nCta persistent CTAs take systems
// in array order from the counter next[1] (zero at launch), one CTA per
// system.  Preconditioner set-up runs in the kernel.  mixed: FP32 inner
// solves in FP64 iterative refinement (nOuter = refinement steps).  done
// (device view of host-mapped memory, [nSys], or null): per-system results
// published as each system finishes.
void launch_batch(cudaStream_t s, SlotSys<double>* s64, SlotSys<float>* s32, int nSys, int nCta, int mixed,
                  double innerRelTol, int maxOuter, unsigned* next, BatchDone* done = nullptr);
// resident batch CTAs per SM (occupancy of the batch kernel)
int batch_ctas_per_sm();
// Cluster form: the first nBig systems (in array order) are solved by whole
// clusters of clusterSize CTAs, the rest by single CTAs; nClusters
// persistent clusters; next[0], next[1] zero at launch.
cudaError_t launch_batch_cluster(cudaStream_t s, SlotSys<double>* s64, SlotSys<float>* s32, int nSys, int nBig,
                                 int clusterSize, int nClusters, int mixed, double innerRelTol, int maxOuter,
                                 unsigned* next, BatchDone* done = nullptr);
// co-resident clusters of the cluster form (0: clusters unavailable)
int batch_max_clusters(int clusterSize);

// Mixed precision: e (float) -> psi (double) += e; r64 -> r32.
void launch_add_f2d(cudaStream_t s, int n, const float* e, double* psi, const int* done);
void launch_cast_pred(cudaStream_t s, int n, const double* in, float* out, const int* done);

// increments a process-wide kernel-launch counter
void count_launch(int k = 1);
int64_t launch_count();

}  // namespace cfx
