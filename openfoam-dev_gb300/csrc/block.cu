// block.cu - whole solves by one CTA: the coarsest GAMG level.
//
// Every solve follows the reference's loop with the reference's scalar logic:
//   PCG::solve              src/OpenFOAM/matrices/lduMatrix/solvers/PCG/PCG.C:65-193
//   PBiCGStab::solve        src/OpenFOAM/matrices/lduMatrix/solvers/PBiCGStab/PBiCGStab.C:68-254
//   solver::normFactor      src/OpenFOAM/matrices/lduMatrix/lduMatrix/lduMatrixSolver.C:174-197
//   DIC / DILU              src/OpenFOAM/matrices/lduMatrix/preconditioners/DICPreconditioner/DICPreconditioner.C:57-126,
//                           src/OpenFOAM/matrices/lduMatrix/preconditioners/DILUPreconditioner/DILUPreconditioner.C:57-136
// The CTA's threads stride over the cells; the triangular sweeps of DIC/DILU
// run level by level (cells of one level are independent) with a barrier
// between levels; sums are fixed-order trees.

#include <cooperative_groups.h>

#include "device.cuh"
#include "groups.cuh"
#include "solvers.h"

namespace cfx {

namespace {

template <class G, class T>
__device__ void blk_amul(G& g, const BlockSys<T>& S, const T* x, T* y) {
    // Amul with the interfaces (lduMatrixATmul.C:34-92): internal faces,
    // then each interface face's -coeffs*x[nbr]
    for (int c = g.rank(); c < S.n; c += g.size())
        y[c] = iface_sub(S.itf, c, x,
                         row_amul<T>(c, S.ownerStart, S.losortStart, S.losortL, S.u, S.diag, S.lp, S.upper, x));
    g.sync();
}

// w = M^-1 r (DICPreconditioner.C:87-126, DILUPreconditioner.C:88-136):
// forward then backward level sweeps, or the pointwise forms.
template <class G, class T>
__device__ void blk_precondition(G& g, const BlockSys<T>& S, const T* r, T* w) {
    if (S.precond == CFX_PRE_DIC || S.precond == CFX_PRE_DILU) {
        for (int L = 0; L < S.nFwd; ++L) {
            for (int i = S.fwdLevelStart[L] + g.rank(); i < S.fwdLevelStart[L + 1]; i += g.size()) {
                const int c = S.fwdCells[i];
                const T rDc = S.rD[c];
                T v = rDc * r[c];
                for (int k = S.losortStart[c]; k < S.losortStart[c + 1]; ++k) v -= (rDc * S.lp[k]) * w[S.losortL[k]];
                w[c] = v;
            }
            g.sync();
        }
        for (int L = 0; L < S.nBwd; ++L) {
            for (int i = S.bwdLevelStart[L] + g.rank(); i < S.bwdLevelStart[L + 1]; i += g.size()) {
                const int c = S.bwdCells[i];
                const T rDc = S.rD[c];
                T v = w[c];
                for (int f = S.ownerStart[c + 1] - 1; f >= S.ownerStart[c]; --f) v -= (rDc * S.upper[f]) * w[S.u[f]];
                w[c] = v;
            }
            g.sync();
        }
    } else {
        for (int c = g.rank(); c < S.n; c += g.size()) w[c] = S.precond == CFX_PRE_DIAGONAL ? S.rD[c] * r[c] : r[c];
        g.sync();
    }
}

template <class T>
__device__ __forceinline__ bool blk_check(const BlockSys<T>& S, double fin, double ini) {
    return fin < S.tolerance || (S.relTol > SP_SMALL && fin < S.relTol * ini);
}

// DIC / DILU reciprocal diagonal: pivots in forward level order (each cell's
// subtractions in face order, as the reference's face loop), then 1/D.
// up = upper in losort order (== lp when symmetric).
template <class G, class T>
__device__ void blk_rD(G& g, const BlockSys<T>& S, const T* up, T* rD) {
    for (int L = 0; L < S.nFwd; ++L) {
        for (int i = S.fwdLevelStart[L] + g.rank(); i < S.fwdLevelStart[L + 1]; i += g.size()) {
            const int c = S.fwdCells[i];
            T D = S.diag[c];
            for (int k = S.losortStart[c]; k < S.losortStart[c + 1]; ++k) D -= (up[k] * S.lp[k]) / rD[S.losortL[k]];
            rD[c] = D;
        }
        g.sync();
    }
    for (int c = g.rank(); c < S.n; c += g.size()) rD[c] = T(1) / rD[c];
    g.sync();
}

// diagonalPreconditioner: rD = 1/diag (diagonalPreconditioner.C:46-66).
template <class G, class T>
__device__ void blk_rdiag(G& g, const BlockSys<T>& S, T* rD) {
    for (int c = g.rank(); c < S.n; c += g.size()) rD[c] = T(1) / S.diag[c];
    g.sync();
}

template <class G, class T>
__device__ void blk_setup_precond(G& g, const BlockSys<T>& S) {
    if (S.precond == CFX_PRE_DIC || S.precond == CFX_PRE_DILU)
        blk_rD(g, S, S.upPerm ? S.upPerm : S.lp, const_cast<T*>(S.rD));
    else if (S.precond == CFX_PRE_DIAGONAL)
        blk_rdiag(g, S, const_cast<T*>(S.rD));
}

// One whole PCG / PBiCGStab solve of S by group g (PCG.C:65-193,
// PBiCGStab.C:68-254); S.rD must hold the preconditioner's reciprocal
// diagonal.
template <class G, class T>
__device__ void blk_solve(G& g, BlockSys<T>& S) {
    const int n = S.n;
    const int r0_ = g.rank(), st_ = g.size();
    T* psi = S.psi;
    double s0 = 0.0;
    for (int c = r0_; c < n; c += st_) s0 += double(psi[c]);
    const double avg = n > 0 ? g.sum(s0) / n : 0.0;
    blk_amul(g, S, psi, S.q);
    double nf = 0.0, mg = 0.0;
    for (int c = r0_; c < n; c += st_) {
        T sA = S.diag[c];
        for (int k = S.losortStart[c]; k < S.losortStart[c + 1]; ++k) sA += S.lp[k];
        for (int f = S.ownerStart[c]; f < S.ownerStart[c + 1]; ++f) sA += S.upper[f];
        // sumA's interface terms (lduMatrixATmul.C:238-254)
        if (S.itf.start)
            for (int j = S.itf.start[c]; j < S.itf.start[c + 1]; ++j) sA -= S.itf.coef[j];
        const T t = sA * T(avg);
        nf += double(fabs(S.q[c] - t) + fabs(S.b[c] - t));
        const T rc = S.b[c] - S.q[c];
        S.r[c] = rc;
        if (S.r0) S.r0[c] = rc;
        mg += fabs(double(rc));
    }
    const double normFactor = g.sum(nf) + SP_SMALL;
    const double initial = g.sum(mg) / normFactor;
    double fin = initial;
    int nIter = 0, converged = blk_check(S, fin, initial), singular = 0;
    if (S.minIter > 0 || !converged) {
        if (S.solver == CFX_SOLVER_PCG) {
            double wArA = SP_GREAT, wArAold;
            do {
                wArAold = wArA;
                blk_precondition(g, S, S.r, S.w);
                double d = 0.0;
                for (int c = r0_; c < n; c += st_) d += double(S.w[c]) * double(S.r[c]);
                wArA = g.sum(d);
                const T beta = T(wArA / wArAold);
                for (int c = r0_; c < n; c += st_) S.p[c] = nIter == 0 ? S.w[c] : S.w[c] + beta * S.p[c];
                g.sync();
                blk_amul(g, S, S.p, S.w);
                d = 0.0;
                for (int c = r0_; c < n; c += st_) d += double(S.w[c]) * double(S.p[c]);
                const double wApA = g.sum(d);
                singular = fabs(wApA) / normFactor < VSMALL;
                if (singular) break;
                const T alpha = T(wArA / wApA);
                mg = 0.0;
                for (int c = r0_; c < n; c += st_) {
                    psi[c] += alpha * S.p[c];
                    const T rc = S.r[c] - alpha * S.w[c];
                    S.r[c] = rc;
                    mg += fabs(double(rc));
                }
                fin = g.sum(mg) / normFactor;
                bool cont = false;
                if (++nIter < S.maxIter) {
                    converged = blk_check(S, fin, initial);
                    cont = !converged;
                }
                if (!(cont || nIter < S.minIter)) break;
            } while (true);
        } else {
            double rA0rA = 0.0, alpha = 0.0, omega = 0.0;
            do {
                const double rA0rAold = rA0rA;
                double d = 0.0;
                for (int c = r0_; c < n; c += st_) d += double(S.r0[c]) * double(S.r[c]);
                rA0rA = g.sum(d);
                singular = fabs(rA0rA) < VSMALL;
                if (singular) break;
                if (nIter == 0) {
                    for (int c = r0_; c < n; c += st_) S.p[c] = S.r[c];
                } else {
                    singular = fabs(omega) < VSMALL;
                    if (singular) break;
                    const T beta = T((rA0rA / rA0rAold) * (alpha / omega));
                    for (int c = r0_; c < n; c += st_) S.p[c] = S.r[c] + beta * (S.p[c] - T(omega) * S.q[c]);
                }
                g.sync();
                blk_precondition(g, S, S.p, S.w);  // yA = w
                blk_amul(g, S, S.w, S.q);          // AyA = q
                d = 0.0;
                for (int c = r0_; c < n; c += st_) d += double(S.r0[c]) * double(S.q[c]);
                alpha = rA0rA / g.sum(d);
                mg = 0.0;
                for (int c = r0_; c < n; c += st_) {
                    const T v = S.r[c] - T(alpha) * S.q[c];
                    S.s[c] = v;
                    mg += fabs(double(v));
                }
                fin = g.sum(mg) / normFactor;
                if (++nIter >= S.minIter && (converged = blk_check(S, fin, initial))) {
                    for (int c = r0_; c < n; c += st_) psi[c] += T(alpha) * S.w[c];
                    g.sync();
                    break;
                }
                blk_precondition(g, S, S.s, S.t);  // zA = t
                // tA = A zA, kept in r (r is rewritten below from s and tA)
                double tt = 0.0, ts = 0.0;
                for (int c = r0_; c < n; c += st_) {
                    const T v = iface_sub(S.itf, c, S.t,
                                          row_amul<T>(c, S.ownerStart, S.losortStart, S.losortL, S.u, S.diag, S.lp,
                                                      S.upper, S.t));
                    S.r[c] = v;
                    tt += double(v) * double(v);
                    ts += double(v) * double(S.s[c]);
                }
                const double tAtA = g.sum(tt);
                omega = g.sum(ts) / tAtA;
                mg = 0.0;
                for (int c = r0_; c < n; c += st_) {
                    psi[c] += T(alpha) * S.w[c] + T(omega) * S.t[c];
                    const T v = S.s[c] - T(omega) * S.r[c];
                    S.r[c] = v;
                    mg += fabs(double(v));
                }
                fin = g.sum(mg) / normFactor;
                bool cont = false;
                if (nIter < S.maxIter) {
                    converged = blk_check(S, fin, initial);
                    cont = !converged;
                }
                if (!(cont || nIter < S.minIter)) break;
            } while (true);
        }
    }
    if (g.leader()) {
        S.initialResidual = initial;
        S.finalResidual = fin;
        S.nIterations = nIter;
        S.converged = converged;
        S.singular = singular;
    }
    g.sync();
}

template <class T>
__global__ void __launch_bounds__(BLK_NT) block_solve_k(BlockSys<T>* systems, const int* done) {
    __shared__ double sh[BLK_NT / 32 + 1];
    if (done && *done) return;
    CtaGroup g{sh};
    blk_solve(g, systems[blockIdx.x]);
}

}  // namespace

template <class T>
void Kern<T>::block_solve(cudaStream_t s, BlockSys<T>* d_sys, int nSys, const int* done) {
    block_solve_k<T><<<nSys, BLK_NT, 0, s>>>(d_sys, done);
    count_launch();
}
template void Kern<double>::block_solve(cudaStream_t, BlockSys<double>*, int, const int*);
template void Kern<float>::block_solve(cudaStream_t, BlockSys<float>*, int, const int*);

}  // namespace cfx
