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
    // r = b - A psi; final = sum|r|/normFactor; nIterations++; loop test
    static void gamg_residual_check(cudaStream_t s, Scratch& sc, const LevelMesh& m, const LevelCoeffs<T>& a,
                                    const T* psi, const T* b, T* r, SolveState* st);
    // single-CTA whole solve of one or more small systems (blockIdx = system)
    static void block_solve(cudaStream_t s, BlockSys<T>* d_sys, int nSys, const int* done);
    // y (+)= x, predicated
    static void axpy(cudaStream_t s, int n, T a, const T* x, T* y, const int* done);
    static void copy(cudaStream_t s, int n, const T* x, T* y, const int* done);
    static void fill(cudaStream_t s, int n, T v, T* y, const int* done);
};

// Mixed precision: e (float) -> psi (double) += e; r64 -> r32.
void launch_add_f2d(cudaStream_t s, int n, const float* e, double* psi, const int* done);
void launch_cast_pred(cudaStream_t s, int n, const double* in, float* out, const int* done);

// increments a process-wide kernel-launch counter
void count_launch(int k = 1);
int64_t launch_count();

}  // namespace cfx
