// solvers.cu - fused kernels of the Krylov and GAMG drivers.
//
// Every scalar of the iteration (normFactor, wArA, alpha, beta, omega, the
// residuals, nIterations, converged/singular) lives in a device SolveState;
// the last block of each reduction kernel finishes the reduction in a fixed
// order and applies the reference's scalar logic, so the host never waits
// inside an iteration.  Once `done` is set every later kernel returns at
// entry, which lets the host enqueue iterations ahead of the convergence test.
//
// Reference loops restated here (paths relative to the OpenFOAM-dev tree):
//   PCG::solve              src/OpenFOAM/matrices/lduMatrix/solvers/PCG/PCG.C:65-193
//   PBiCGStab::solve        src/OpenFOAM/matrices/lduMatrix/solvers/PBiCGStab/PBiCGStab.C:68-254
//   solver::normFactor      src/OpenFOAM/matrices/lduMatrix/lduMatrix/lduMatrixSolver.C:174-197
//   checkConvergence / checkSingularity
//                           src/OpenFOAM/matrices/LduMatrix/LduMatrix/SolverPerformance.C:32-92
//   GAMGSolver::scale       src/OpenFOAM/matrices/lduMatrix/solvers/GAMG/GAMGSolverScale.C:31-76
//   GAMGSolver::solve       src/OpenFOAM/matrices/lduMatrix/solvers/GAMG/GAMGSolverSolve.C:31-145

#include <atomic>
#include <cfloat>

#include "device.cuh"
#include "solvers.h"

namespace cfx {

namespace {

std::atomic<int64_t> g_launches{0};


inline int grid_for(int64_t n) {
    int64_t b = (n + RED_NT - 1) / RED_NT;
    if (b < 1) b = 1;
    if (b > RED_MAXB) b = RED_MAXB;
    return int(b);
}

__device__ __forceinline__ int check_convergence(SolveState* st) {
    const int c = st->finalResidual < st->tolerance ||
                  (st->relTol > SP_SMALL && st->finalResidual < st->relTol * st->initialResidual);
    st->converged = c;
    return c;
}

// do { ... } while ((++nIter < maxIter && !converged) || nIter < minIter)
__device__ __forceinline__ void loop_test(SolveState* st, int inc = 1) {
    st->nIterations += inc;
    bool cont = false;
    if (st->nIterations < st->maxIter) cont = !check_convergence(st);
    cont = cont || st->nIterations < st->minIter;
    if (!cont) st->done = 1;
}

// Two fixed-order partial sums per block, finished by the last block.
struct Red2 {
    double* partials;
    unsigned* counter;
};

template <int NT>
__device__ __forceinline__ bool reduce2(double a, double b, Red2 r, double& outA, double& outB) {
    __shared__ double sh[NT / 32];
    a = block_sum<NT>(a, sh);
    b = block_sum<NT>(b, sh);
    if (threadIdx.x == 0) {
        r.partials[blockIdx.x] = a;
        r.partials[RED_MAXB + blockIdx.x] = b;
    }
    if (!last_block(r.counter)) return false;
    double sa = 0.0, sb = 0.0;
    for (int i = threadIdx.x; i < gridDim.x; i += NT) {
        sa += __ldcg(r.partials + i);
        sb += __ldcg(r.partials + RED_MAXB + i);
    }
    sa = block_sum<NT>(sa, sh);
    sb = block_sum<NT>(sb, sh);
    outA = sa;
    outB = sb;
    return true;  // valid in thread 0
}


// normFactor (lduMatrixSolver.C:174-197): sumA*gAverage(psi), then
// sum(|Apsi - t| + |b - t|) + small_; also r = b - Apsi and sum|r|.
template <class T>
__global__ void __launch_bounds__(RED_NT) norm_init_k(int n, const int* os, const int* ls, const int* u,
                                                      const T* diag, const T* lp, const T* upper,
                                                      const T* __restrict__ Apsi, const T* __restrict__ b,
                                                      T* __restrict__ r, T* __restrict__ r0, SolveState* st,
                                                      Red2 red, Iface<T> itf) {
    const double avg = n > 0 ? st->red0 / n : 0.0;
    double nf = 0.0, mg = 0.0;
    for (int c = blockIdx.x * RED_NT + threadIdx.x; c < n; c += gridDim.x * RED_NT) {
        T sA = diag[c];
        for (int k = ls[c]; k < ls[c + 1]; ++k) sA += lp[k];
        for (int f = os[c]; f < os[c + 1]; ++f) sA += upper[f];
        if (itf.start)  // sumA's interface boundary coefficients
            for (int j = itf.start[c]; j < itf.start[c + 1]; ++j) sA -= itf.coef[j];
        const T t = sA * T(avg);
        nf += double(fabs(Apsi[c] - t) + fabs(b[c] - t));
        const T rc = b[c] - Apsi[c];
        r[c] = rc;
        if (r0) r0[c] = rc;
        mg += fabs(double(rc));
    }
    double snf, smg;
    if (reduce2<RED_NT>(nf, mg, red, snf, smg) && threadIdx.x == 0) {
        st->normFactor = snf + SP_SMALL;
        st->initialResidual = smg / st->normFactor;
        st->finalResidual = st->initialResidual;
        st->nIterations = 0;
        st->singular = 0;
        st->phase = 0;
        st->wArA = SP_GREAT;
        st->rA0rA = 0.0;
        st->alpha = 0.0;
        st->omega = 0.0;
        const int conv = check_convergence(st);
        st->done = !(st->minIter > 0 || !conv);
    }
}

template <class T>
__global__ void __launch_bounds__(RED_NT) precond_pointwise_k(int n, const T* __restrict__ rD,
                                                              const T* __restrict__ r, T* __restrict__ w,
                                                              double* partials, const int* done) {
    __shared__ double sh[RED_NT / 32];
    if (done && *done) return;
    double d = 0.0;
    for (int c = blockIdx.x * RED_NT + threadIdx.x; c < n; c += gridDim.x * RED_NT) {
        const T v = rD ? rD[c] * r[c] : r[c];
        w[c] = v;
        d += double(v) * double(r[c]);
    }
    d = block_sum<RED_NT>(d, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = d;
}

// wArAold = wArA; wArA = sum of the preconditioner's dot partials; beta.
__global__ void pcg_beta_k(int nPartials, const double* partials, SolveState* st) {
    __shared__ double sh[RED_NT / 32];
    if (st->done) return;
    double s = 0.0;
    for (int i = threadIdx.x; i < nPartials; i += RED_NT) s += partials[i];
    s = block_sum<RED_NT>(s, sh);
    if (threadIdx.x == 0) {
        st->wArAold = st->wArA;
        st->wArA = s;
        st->beta = st->wArA / st->wArAold;
    }
}

template <class T>
__global__ void pcg_p_k(int n, const T* __restrict__ w, T* __restrict__ p, const SolveState* st) {
    if (st->done) return;
    const bool first = st->nIterations == 0;
    const T beta = T(st->beta);
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x)
        p[c] = first ? w[c] : w[c] + beta * p[c];
}

template <class T>
__global__ void __launch_bounds__(RED_NT) pcg_amul_k(int n, const int* os, const int* ls, const int* lL,
                                                     const int* u, const T* diag, const T* lp, const T* upper, Sell<T> S,
                                                     const T* __restrict__ p, T* __restrict__ wA, SolveState* st,
                                                     Red2 red, Iface<T> itf) {
    if (st->done) return;
    double d = 0.0;
    for (int c = blockIdx.x * RED_NT + threadIdx.x; c < n; c += gridDim.x * RED_NT) {
        const T v = iface_sub(itf, c, p, row_ax<T>(c, os, ls, lL, u, diag, lp, upper, S, p));
        wA[c] = v;
        d += double(v) * double(p[c]);
    }
    double s, dummy;
    if (reduce2<RED_NT>(d, 0.0, red, s, dummy) && threadIdx.x == 0) {
        // PCG.C:161-168: singularity test, then alpha
        st->singular = fabs(s) / st->normFactor < VSMALL;
        if (st->singular) {
            st->done = 1;
        } else {
            st->alpha = st->wArA / s;
        }
    }
}

template <class T>
__global__ void __launch_bounds__(RED_NT) pcg_update_k(int n, const T* __restrict__ p, const T* __restrict__ wA,
                                                       T* __restrict__ psi, T* __restrict__ r, SolveState* st,
                                                       Red2 red) {
    if (st->done) return;
    const T alpha = T(st->alpha);
    double mg = 0.0;
    for (int c = blockIdx.x * RED_NT + threadIdx.x; c < n; c += gridDim.x * RED_NT) {
        psi[c] += alpha * p[c];
        const T rc = r[c] - alpha * wA[c];
        r[c] = rc;
        mg += fabs(double(rc));
    }
    double s, dummy;
    if (reduce2<RED_NT>(mg, 0.0, red, s, dummy) && threadIdx.x == 0) {
        st->finalResidual = s / st->normFactor;
        loop_test(st);
    }
}

// PBiCG.C:138-158: the search directions of the pair (first iteration: the
// preconditioned residuals)
template <class T>
__global__ void pbicg_p_k(int n, const T* __restrict__ w, const T* __restrict__ wT, T* __restrict__ p,
                          T* __restrict__ pT, const SolveState* st) {
    if (st->done) return;
    const bool first = st->nIterations == 0;
    const T beta = T(st->beta);
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        if (first) {
            p[c] = w[c];
            pT[c] = wT[c];
        } else {
            p[c] = w[c] + beta * p[c];
            pT[c] = wT[c] + beta * pT[c];
        }
    }
}

// PBiCG.C:160-172: wT = A^T pT (row gather, lduMatrix::Tmul's per-cell face
// order) fused with wApT = wA.pT, the singularity test and alpha.
template <class T>
__global__ void __launch_bounds__(RED_NT) pbicg_tmul_k(int n, const int* os, const int* ls, const int* lL,
                                                       const int* u, const T* diag, const T* upPerm, const T* lower,
                                                       const T* __restrict__ pT, T* __restrict__ wT,
                                                       const T* __restrict__ wA, SolveState* st, Red2 red,
                                                       Iface<T> itf) {
    if (st->done) return;
    double d = 0.0;
    for (int c = blockIdx.x * RED_NT + threadIdx.x; c < n; c += gridDim.x * RED_NT) {
        wT[c] = iface_sub(itf, c, pT, row_amul<T>(c, os, ls, lL, u, diag, upPerm, lower, pT));
        d += double(wA[c]) * double(pT[c]);
    }
    double s, dummy;
    if (reduce2<RED_NT>(d, 0.0, red, s, dummy) && threadIdx.x == 0) {
        st->singular = fabs(s) / st->normFactor < VSMALL;
        if (st->singular) {
            st->done = 1;
        } else {
            st->alpha = st->wArA / s;
        }
    }
}

// PBiCG.C:174-200: psi, rA and rT updates, |rA|/normFactor, loop test.
template <class T>
__global__ void __launch_bounds__(RED_NT) pbicg_update_k(int n, const T* __restrict__ p, const T* __restrict__ wA,
                                                         const T* __restrict__ wT, T* __restrict__ psi,
                                                         T* __restrict__ r, T* __restrict__ rT, SolveState* st,
                                                         Red2 red) {
    if (st->done) return;
    const T alpha = T(st->alpha);
    double mg = 0.0;
    for (int c = blockIdx.x * RED_NT + threadIdx.x; c < n; c += gridDim.x * RED_NT) {
        psi[c] += alpha * p[c];
        const T rc = r[c] - alpha * wA[c];
        r[c] = rc;
        rT[c] -= alpha * wT[c];
        mg += fabs(double(rc));
    }
    double s, dummy;
    if (reduce2<RED_NT>(mg, 0.0, red, s, dummy) && threadIdx.x == 0) {
        st->finalResidual = s / st->normFactor;
        loop_test(st);
    }
}

// PBiCGStab.C:141-171
template <class T>
__global__ void __launch_bounds__(RED_NT) bicg_rho_k(int n, const T* __restrict__ r0, const T* __restrict__ r,
                                                     SolveState* st, Red2 red) {
    if (st->done) return;
    double d = 0.0;
    for (int c = blockIdx.x * RED_NT + threadIdx.x; c < n; c += gridDim.x * RED_NT) d += double(r0[c]) * double(r[c]);
    double s, dummy;
    if (reduce2<RED_NT>(d, 0.0, red, s, dummy) && threadIdx.x == 0) {
        st->rA0rAold = st->rA0rA;
        st->rA0rA = s;
        st->singular = fabs(s) < VSMALL;
        if (st->singular) {
            st->done = 1;
            return;
        }
        if (st->nIterations > 0) {
            st->singular = fabs(st->omega) < VSMALL;
            if (st->singular) {
                st->done = 1;
                return;
            }
            st->beta = (st->rA0rA / st->rA0rAold) * (st->alpha / st->omega);
        }
    }
}

template <class T>
__global__ void bicg_p_k(int n, const T* __restrict__ r, const T* __restrict__ AyA, T* __restrict__ p,
                         const SolveState* st) {
    if (st->done) return;
    const bool first = st->nIterations == 0;
    const T beta = T(st->beta), omega = T(st->omega);
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x)
        p[c] = first ? r[c] : r[c] + beta * (p[c] - omega * AyA[c]);
}

template <class T>
__global__ void __launch_bounds__(RED_NT) bicg_amul_alpha_k(int n, const int* os, const int* ls, const int* lL,
                                                            const int* u, const T* diag, const T* lp,
                                                            const T* upper, Sell<T> S, const T* __restrict__ yA,
                                                            T* __restrict__ AyA, const T* __restrict__ r0,
                                                            SolveState* st, Red2 red, Iface<T> itf) {
    if (st->done) return;
    double d = 0.0;
    for (int c = blockIdx.x * RED_NT + threadIdx.x; c < n; c += gridDim.x * RED_NT) {
        const T v = iface_sub(itf, c, yA, row_ax<T>(c, os, ls, lL, u, diag, lp, upper, S, yA));
        AyA[c] = v;
        d += double(r0[c]) * double(v);
    }
    double s, dummy;
    if (reduce2<RED_NT>(d, 0.0, red, s, dummy) && threadIdx.x == 0) st->alpha = st->rA0rA / s;
}

template <class T>
__global__ void __launch_bounds__(RED_NT) bicg_s_k(int n, const T* __restrict__ r, const T* __restrict__ AyA,
                                                   T* __restrict__ sA, SolveState* st, Red2 red) {
    if (st->done) return;
    const T alpha = T(st->alpha);
    double mg = 0.0;
    for (int c = blockIdx.x * RED_NT + threadIdx.x; c < n; c += gridDim.x * RED_NT) {
        const T v = r[c] - alpha * AyA[c];
        sA[c] = v;
        mg += fabs(double(v));
    }
    double s, dummy;
    if (reduce2<RED_NT>(mg, 0.0, red, s, dummy) && threadIdx.x == 0) {
        st->finalResidual = s / st->normFactor;
        // if (++nIterations >= minIter && checkConvergence) { psi += alpha*yA; return }
        if (++st->nIterations >= st->minIter && check_convergence(st)) {
            st->phase = 1;
            st->done = 1;
        }
    }
}

template <class T>
__global__ void bicg_early_k(int n, const T* __restrict__ yA, T* __restrict__ psi, SolveState* st) {
    if (st->phase != 1) return;
    const T alpha = T(st->alpha);
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) psi[c] += alpha * yA[c];
}

__global__ void bicg_phase_k(SolveState* st) {
    if (st->phase == 1) st->phase = 2;
}

template <class T>
__global__ void __launch_bounds__(RED_NT) bicg_amul_omega_k(int n, const int* os, const int* ls, const int* lL,
                                                            const int* u, const T* diag, const T* lp,
                                                            const T* upper, Sell<T> S, const T* __restrict__ zA,
                                                            T* __restrict__ tA, const T* __restrict__ sA,
                                                            SolveState* st, Red2 red, Iface<T> itf) {
    if (st->done) return;
    double tt = 0.0, ts = 0.0;
    for (int c = blockIdx.x * RED_NT + threadIdx.x; c < n; c += gridDim.x * RED_NT) {
        const T v = iface_sub(itf, c, zA, row_ax<T>(c, os, ls, lL, u, diag, lp, upper, S, zA));
        tA[c] = v;
        tt += double(v) * double(v);
        ts += double(v) * double(sA[c]);
    }
    double stt, sts;
    if (reduce2<RED_NT>(tt, ts, red, stt, sts) && threadIdx.x == 0) {
        st->tAtA = stt;
        st->omega = sts / stt;
    }
}

template <class T>
__global__ void __launch_bounds__(RED_NT) bicg_update_k(int n, const T* __restrict__ yA, const T* __restrict__ zA,
                                                        const T* __restrict__ sA, const T* __restrict__ tA,
                                                        T* __restrict__ psi, T* __restrict__ r, SolveState* st,
                                                        Red2 red) {
    if (st->done) return;
    const T alpha = T(st->alpha), omega = T(st->omega);
    double mg = 0.0;
    for (int c = blockIdx.x * RED_NT + threadIdx.x; c < n; c += gridDim.x * RED_NT) {
        psi[c] += alpha * yA[c] + omega * zA[c];
        const T v = sA[c] - omega * tA[c];
        r[c] = v;
        mg += fabs(double(v));
    }
    double s, dummy;
    if (reduce2<RED_NT>(mg, 0.0, red, s, dummy) && threadIdx.x == 0) {
        st->finalResidual = s / st->normFactor;
        // while ((nIter < maxIter && !converged) || nIter < minIter)
        bool cont = false;
        if (st->nIterations < st->maxIter) cont = !check_convergence(st);
        cont = cont || st->nIterations < st->minIter;
        if (!cont) st->done = 1;
    }
}

// GAMGSolverScale.C:42-75
template <class T>
__global__ void __launch_bounds__(RED_NT) gamg_scale_sf_k(int n, const int* os, const int* ls, const int* lL,
                                                          const int* u, const T* diag, const T* lp, const T* upper, Sell<T> S,
                                                          const T* __restrict__ field, T* __restrict__ Acf,
                                                          const T* __restrict__ source, SolveState* st, Red2 red,
                                                          Iface<T> itf) {
    if (st->done) return;
    // a thread's partial sums in T (the FP32 inner cycles accumulate their
    // few cells in FP32 rather than on GB300's slow FP64 pipe), the block and
    // grid sums in double
    T num = T(0), den = T(0);
    for (int c = blockIdx.x * RED_NT + threadIdx.x; c < n; c += gridDim.x * RED_NT) {
        // Amul with the level's interfaces (GAMGSolverScale.C:42-50)
        const T v = iface_sub(itf, c, field, row_ax<T>(c, os, ls, lL, u, diag, lp, upper, S, field));
        Acf[c] = v;
        num += source[c] * field[c];
        den += v * field[c];
    }
    double sn, sd;
    if (reduce2<RED_NT>(double(num), double(den), red, sn, sd) && threadIdx.x == 0) {
        const double stab = sd >= 0 ? sd + VSMALL : sd - VSMALL;  // stabilise(den, vSmall)
        st->sf = sn / stab;
    }
}

template <class T>
__global__ void gamg_scale_apply_k(int n, T* __restrict__ field, const T* __restrict__ Acf,
                                   const T* __restrict__ source, const T* __restrict__ D, const T* __restrict__ pre,
                                   const SolveState* st) {
    if (st->done) return;
    const T sf = T(st->sf);
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        T v = sf * field[c] + (source[c] - sf * Acf[c]) / D[c];
        if (pre) v += pre[c];
        field[c] = v;
    }
}

// RES false: GAMG's finestResidual = source - Apsi (GAMGSolverSolve.C:116-118);
// RES true: lduMatrix::residual (lduMatrixATmul.C:203-280: source - diag psi,
// then minus the neighbour products), as smoothSolver checks it.  The loop
// counter advances by inc.
template <class T, bool RES>
__global__ void __launch_bounds__(RED_NT) gamg_residual_check_k(int n, const int* os, const int* ls, const int* lL,
                                                                const int* u, const T* diag, const T* lp,
                                                                const T* upper, Sell<T> S, const T* __restrict__ psi,
                                                                const T* __restrict__ b, T* __restrict__ r,
                                                                SolveState* st, Red2 red, int inc, Iface<T> itf) {
    if (st->done) return;
    double mg = 0.0;
    for (int c = blockIdx.x * RED_NT + threadIdx.x; c < n; c += gridDim.x * RED_NT) {
        T v;
        if (RES) {
            v = iface_sub_neg(itf, c, psi, row_res<T>(c, os, ls, lL, u, diag, lp, upper, S, psi, b));
        } else {
            v = b[c] - iface_sub(itf, c, psi, row_ax<T>(c, os, ls, lL, u, diag, lp, upper, S, psi));
        }
        r[c] = v;
        mg += fabs(double(v));
    }
    double s, dummy;
    if (reduce2<RED_NT>(mg, 0.0, red, s, dummy) && threadIdx.x == 0) {
        st->finalResidual = s / st->normFactor;
        loop_test(st, inc);
    }
}

template <class T>
__global__ void axpy_k(int n, T a, const T* __restrict__ x, T* __restrict__ y, const int* done) {
    if (done && *done) return;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) y[c] += a * x[c];
}

template <class T>
__global__ void copy_k(int n, const T* __restrict__ x, T* __restrict__ y, const int* done) {
    if (done && *done) return;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) y[c] = x[c];
}

template <class T>
__global__ void fill_k(int n, T v, T* __restrict__ y, const int* done) {
    if (done && *done) return;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) y[c] = v;
}

__global__ void add_f2d_k(int n, const float* __restrict__ e, double* __restrict__ psi, const int* done) {
    if (done && *done) return;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) psi[c] += double(e[c]);
}

__global__ void cast_pred_k(int n, const double* __restrict__ in, float* __restrict__ out, const int* done) {
    if (done && *done) return;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) out[c] = float(in[c]);
}


}  // namespace

void count_launch(int k) { g_launches += k; }
int64_t launch_count() { return g_launches.load(); }

template <class T>
void Kern<T>::norm_init(cudaStream_t s, Scratch& sc, const LevelMesh& m, const LevelCoeffs<T>& a, const T* Apsi,
                        const T* b, T* r, T* r0, SolveState* st) {
    norm_init_k<T><<<grid_for(m.n), RED_NT, 0, s>>>(m.n, m.ownerStart, m.losortStart, m.u, a.diag, a.lowerPerm,
                                                    a.upper, Apsi, b, r, r0, st, Red2{sc.partials, sc.counters},
                                                    if_bou(m, a));
    count_launch();
}

template <class T>
void Kern<T>::precond_pointwise(cudaStream_t s, int n, const T* rD, const T* r, T* w, double* partials,
                                const int* done) {
    precond_pointwise_k<T><<<grid_for(n), RED_NT, 0, s>>>(n, rD, r, w, partials, done);
    count_launch();
}

template <class T>
void Kern<T>::pcg_beta(cudaStream_t s, int nPartials, const double* partials, SolveState* st) {
    pcg_beta_k<<<1, RED_NT, 0, s>>>(nPartials, partials, st);
    count_launch();
}

template <class T>
void Kern<T>::pcg_p(cudaStream_t s, int n, const T* w, T* p, const SolveState* st) {
    pcg_p_k<T><<<grid_for(n), RED_NT, 0, s>>>(n, w, p, st);
    count_launch();
}

template <class T>
void Kern<T>::pcg_amul(cudaStream_t s, Scratch& sc, const LevelMesh& m, const LevelCoeffs<T>& a, const T* p, T* wA,
                       SolveState* st) {
    pcg_amul_k<T><<<grid_for(m.n), RED_NT, 0, s>>>(m.n, m.ownerStart, m.losortStart, m.losortL, m.u, a.diag,
                                                   a.lowerPerm, a.upper, sell_of(m, a), p, wA, st, Red2{sc.partials, sc.counters},
                                                   if_bou(m, a));
    count_launch();
}

template <class T>
void Kern<T>::pcg_update(cudaStream_t s, Scratch& sc, int n, const T* p, const T* wA, T* psi, T* r, SolveState* st) {
    pcg_update_k<T><<<grid_for(n), RED_NT, 0, s>>>(n, p, wA, psi, r, st, Red2{sc.partials, sc.counters});
    count_launch();
}

template <class T>
void Kern<T>::pbicg_p(cudaStream_t s, int n, const T* w, const T* wT, T* p, T* pT, const SolveState* st) {
    pbicg_p_k<T><<<grid_for(n), RED_NT, 0, s>>>(n, w, wT, p, pT, st);
    count_launch();
}

template <class T>
void Kern<T>::pbicg_tmul(cudaStream_t s, Scratch& sc, const LevelMesh& m, const LevelCoeffs<T>& a, const T* pT,
                         T* wT, const T* wA, SolveState* st) {
    pbicg_tmul_k<T><<<grid_for(m.n), RED_NT, 0, s>>>(m.n, m.ownerStart, m.losortStart, m.losortL, m.u, a.diag,
                                                     a.sym ? a.lowerPerm : a.upperPerm, a.sym ? a.upper : a.lower,
                                                     pT, wT, wA, st, Red2{sc.partials, sc.counters}, if_int(m, a));
    count_launch();
}

template <class T>
void Kern<T>::pbicg_update(cudaStream_t s, Scratch& sc, int n, const T* p, const T* wA, const T* wT, T* psi, T* r,
                           T* rT, SolveState* st) {
    pbicg_update_k<T><<<grid_for(n), RED_NT, 0, s>>>(n, p, wA, wT, psi, r, rT, st, Red2{sc.partials, sc.counters});
    count_launch();
}

template <class T>
void Kern<T>::bicg_rho(cudaStream_t s, Scratch& sc, int n, const T* r0, const T* r, SolveState* st) {
    bicg_rho_k<T><<<grid_for(n), RED_NT, 0, s>>>(n, r0, r, st, Red2{sc.partials, sc.counters});
    count_launch();
}

template <class T>
void Kern<T>::bicg_p(cudaStream_t s, int n, const T* r, const T* AyA, T* p, const SolveState* st) {
    bicg_p_k<T><<<grid_for(n), RED_NT, 0, s>>>(n, r, AyA, p, st);
    count_launch();
}

template <class T>
void Kern<T>::bicg_amul_alpha(cudaStream_t s, Scratch& sc, const LevelMesh& m, const LevelCoeffs<T>& a, const T* yA,
                              T* AyA, const T* r0, SolveState* st) {
    bicg_amul_alpha_k<T><<<grid_for(m.n), RED_NT, 0, s>>>(m.n, m.ownerStart, m.losortStart, m.losortL, m.u, a.diag,
                                                          a.lowerPerm, a.upper, sell_of(m, a), yA, AyA, r0, st,
                                                          Red2{sc.partials, sc.counters}, if_bou(m, a));
    count_launch();
}

template <class T>
void Kern<T>::bicg_s(cudaStream_t s, Scratch& sc, int n, const T* r, const T* AyA, T* sA, SolveState* st) {
    bicg_s_k<T><<<grid_for(n), RED_NT, 0, s>>>(n, r, AyA, sA, st, Red2{sc.partials, sc.counters});
    count_launch();
}

template <class T>
void Kern<T>::bicg_early(cudaStream_t s, int n, const T* yA, T* psi, SolveState* st) {
    bicg_early_k<T><<<grid_for(n), RED_NT, 0, s>>>(n, yA, psi, st);
    bicg_phase_k<<<1, 1, 0, s>>>(st);
    count_launch(2);
}

template <class T>
void Kern<T>::bicg_amul_omega(cudaStream_t s, Scratch& sc, const LevelMesh& m, const LevelCoeffs<T>& a, const T* zA,
                              T* tA, const T* sA, SolveState* st) {
    bicg_amul_omega_k<T><<<grid_for(m.n), RED_NT, 0, s>>>(m.n, m.ownerStart, m.losortStart, m.losortL, m.u, a.diag,
                                                          a.lowerPerm, a.upper, sell_of(m, a), zA, tA, sA, st,
                                                          Red2{sc.partials, sc.counters}, if_bou(m, a));
    count_launch();
}

template <class T>
void Kern<T>::bicg_update(cudaStream_t s, Scratch& sc, int n, const T* yA, const T* zA, const T* sA, const T* tA,
                          T* psi, T* r, SolveState* st) {
    bicg_update_k<T><<<grid_for(n), RED_NT, 0, s>>>(n, yA, zA, sA, tA, psi, r, st, Red2{sc.partials, sc.counters});
    count_launch();
}

template <class T>
void Kern<T>::gamg_scale_sf(cudaStream_t s, Scratch& sc, const LevelMesh& m, const LevelCoeffs<T>& a, const T* field,
                            T* Acf, const T* source, SolveState* st) {
    gamg_scale_sf_k<T><<<grid_for(m.n), RED_NT, 0, s>>>(m.n, m.ownerStart, m.losortStart, m.losortL, m.u, a.diag,
                                                        a.lowerPerm, a.upper, sell_of(m, a), field, Acf, source, st,
                                                        Red2{sc.partials, sc.counters}, if_bou(m, a));
    count_launch();
}

template <class T>
void Kern<T>::gamg_scale_apply(cudaStream_t s, int n, T* field, const T* Acf, const T* source, const T* diag,
                               const T* pre, const SolveState* st) {
    gamg_scale_apply_k<T><<<grid_for(n), RED_NT, 0, s>>>(n, field, Acf, source, diag, pre, st);
    count_launch();
}

template <class T>
void Kern<T>::gamg_residual_check(cudaStream_t s, Scratch& sc, const LevelMesh& m, const LevelCoeffs<T>& a,
                                  const T* psi, const T* b, T* r, SolveState* st, int inc) {
    if (inc > 0)
        gamg_residual_check_k<T, true><<<grid_for(m.n), RED_NT, 0, s>>>(
            m.n, m.ownerStart, m.losortStart, m.losortL, m.u, a.diag, a.lowerPerm, a.upper, sell_of(m, a), psi, b, r, st,
            Red2{sc.partials, sc.counters}, inc, if_bou(m, a));
    else
        gamg_residual_check_k<T, false><<<grid_for(m.n), RED_NT, 0, s>>>(
            m.n, m.ownerStart, m.losortStart, m.losortL, m.u, a.diag, a.lowerPerm, a.upper, sell_of(m, a), psi, b, r, st,
            Red2{sc.partials, sc.counters}, 1, if_bou(m, a));
    count_launch();
}

template <class T>
void Kern<T>::axpy(cudaStream_t s, int n, T a, const T* x, T* y, const int* done) {
    axpy_k<T><<<grid_for(n), RED_NT, 0, s>>>(n, a, x, y, done);
    count_launch();
}

template <class T>
void Kern<T>::copy(cudaStream_t s, int n, const T* x, T* y, const int* done) {
    copy_k<T><<<grid_for(n), RED_NT, 0, s>>>(n, x, y, done);
    count_launch();
}

template <class T>
void Kern<T>::fill(cudaStream_t s, int n, T v, T* y, const int* done) {
    fill_k<T><<<grid_for(n), RED_NT, 0, s>>>(n, v, y, done);
    count_launch();
}

void launch_add_f2d(cudaStream_t s, int n, const float* e, double* psi, const int* done) {
    add_f2d_k<<<grid_for(n), RED_NT, 0, s>>>(n, e, psi, done);
    count_launch();
}

void launch_cast_pred(cudaStream_t s, int n, const double* in, float* out, const int* done) {
    cast_pred_k<<<grid_for(n), RED_NT, 0, s>>>(n, in, out, done);
    count_launch();
}

template struct Kern<double>;
template struct Kern<float>;

}  // namespace cfx
