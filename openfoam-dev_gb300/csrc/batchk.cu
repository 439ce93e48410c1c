// batchk.cu - batched solves of independent systems in slot order, one
// thread group (a CTA or a thread-block cluster) per system.
//
// Reference loops restated (paths relative to the OpenFOAM-dev tree):
//   PCG::solve              src/OpenFOAM/matrices/lduMatrix/solvers/PCG/PCG.C:65-193
//   PBiCGStab::solve        src/OpenFOAM/matrices/lduMatrix/solvers/PBiCGStab/PBiCGStab.C:68-254
//   solver::normFactor      src/OpenFOAM/matrices/lduMatrix/lduMatrix/lduMatrixSolver.C:174-197
//   lduMatrix::Amul, sumA   src/OpenFOAM/matrices/lduMatrix/lduMatrix/lduMatrixATmul.C:34-92, 154-200
//   DIC / DILU              src/OpenFOAM/matrices/lduMatrix/preconditioners/DICPreconditioner/DICPreconditioner.C:57-126,
//                           src/OpenFOAM/matrices/lduMatrix/preconditioners/DILUPreconditioner/DILUPreconditioner.C:57-136
//   diagonal                src/OpenFOAM/matrices/lduMatrix/preconditioners/diagonalPreconditioner/diagonalPreconditioner.C:46-87
//
// Storage is in slot order (SlotSys): the forward sweep's levels are
// contiguous slot ranges, coefficients and neighbour slots are column-major
// ELL, so a thread's loads for a slot are independent of one another and
// coalesced across the warp.  Each thread takes SU slots at a time and issues
// all their loads before any store, which keeps SU x (ELL width) loads in
// flight per thread; the neighbour values gathered in a sweep level belong
// to earlier levels, so no load of a round reads a slot stored in it.  Every
// per-cell arithmetic sequence is the reference's (diag, then the faces
// where the cell is the neighbour in losort order, then the faces it owns in
// face order; the same for sumA and the DIC/DILU pivots), so a row of A x is
// bit-identical to the reference's.  Meshes with more than SW faces of
// either kind per cell take a one-slot-at-a-time path with the same
// arithmetic.

#include "device.cuh"
#include "groups.cuh"
#include "solvers.h"

namespace cfx {

namespace {

constexpr int SU = 2;  // slots per thread per round
constexpr int SW = 3;  // widest ELL of the unrolled path (hexahedra: 3 lower, 3 upper)

template <class T>
__device__ __forceinline__ bool fast(const SlotSys<T>& S) {
    return S.wLo <= SW && S.wUp <= SW;
}

// ---------------------------------------------------------------- sweeps
// Forward DIC/DILU sweep (w = rD r, then w[c] -= rD[c] lo w[l] over the
// faces where c is the neighbour) over slots [b, e) of one level.
template <class G, class T>
__device__ __forceinline__ void fwd_level(const G& g, const SlotSys<T>& S, int b, int e, const T* r, T* w) {
    const int n = S.n, wl = S.wLo;
    if (fast(S)) {
        for (int base = b + g.rank(); base < e; base += SU * g.size()) {
            T v[SU], rd[SU], cf[SU][SW], wv[SU][SW];
            int src[SU][SW], nl[SU];
#pragma unroll
            for (int u = 0; u < SU; ++u) {
                const int p = base + u * g.size();
                const int q = p < e ? p : b;
                nl[u] = p < e ? (S.cnt[q] & 0xffff) : 0;
                rd[u] = S.rD[q];
                v[u] = rd[u] * r[q];
#pragma unroll
                for (int j = 0; j < SW; ++j)
                    if (j < wl) {
                        cf[u][j] = S.lo[j * n + q];
                        src[u][j] = S.loSrc[j * n + q];
                    }
            }
#pragma unroll
            for (int u = 0; u < SU; ++u)
#pragma unroll
                for (int j = 0; j < SW; ++j)
                    if (j < wl) wv[u][j] = w[src[u][j]];
#pragma unroll
            for (int u = 0; u < SU; ++u) {
#pragma unroll
                for (int j = 0; j < SW; ++j)
                    if (j < nl[u]) v[u] -= (rd[u] * cf[u][j]) * wv[u][j];
                const int p = base + u * g.size();
                if (p < e) w[p] = v[u];
            }
        }
    } else {
        for (int p = b + g.rank(); p < e; p += g.size()) {
            const int nlp = S.cnt[p] & 0xffff;
            const T rdp = S.rD[p];
            T v = rdp * r[p];
            for (int j = 0; j < nlp; ++j) v -= (rdp * S.lo[j * n + p]) * w[S.loSrc[j * n + p]];
            w[p] = v;
        }
    }
}

// Backward sweep: w[c] -= rD[c] up w[u] over the faces c owns, last face
// first; d accumulates w.r when r is non-null (the PCG's wArA).
template <class G, class T>
__device__ __forceinline__ void bwd_level(const G& g, const SlotSys<T>& S, int L, T* w, const T* r, double& d) {
    const int n = S.n, wu = S.wUp;
    int b, e;
    if (S.bwdMirror) {
        b = S.fwdLevelStart[S.nFwd - 1 - L];
        e = S.fwdLevelStart[S.nFwd - L];
    } else {
        b = S.bwdLevelStart[L];
        e = S.bwdLevelStart[L + 1];
    }
    if (fast(S)) {
        for (int base = b + g.rank(); base < e; base += SU * g.size()) {
            T v[SU], rd[SU], cf[SU][SW], wv[SU][SW], rr[SU];
            int src[SU][SW], nu[SU], slot[SU];
#pragma unroll
            for (int u = 0; u < SU; ++u) {
                const int i = base + u * g.size();
                const int iq = i < e ? i : b;
                slot[u] = S.bwdMirror ? iq : S.bwdSlot[iq];
            }
#pragma unroll
            for (int u = 0; u < SU; ++u) {
                const int i = base + u * g.size();
                const int q = slot[u];
                nu[u] = i < e ? (S.cnt[q] >> 16) : 0;
                rd[u] = S.rD[q];
                v[u] = w[q];
                rr[u] = r ? r[q] : T(0);
#pragma unroll
                for (int j = 0; j < SW; ++j)
                    if (j < wu) {
                        cf[u][j] = S.up[j * n + q];
                        src[u][j] = S.upSrc[j * n + q];
                    }
            }
#pragma unroll
            for (int u = 0; u < SU; ++u)
#pragma unroll
                for (int j = 0; j < SW; ++j)
                    if (j < wu) wv[u][j] = w[src[u][j]];
#pragma unroll
            for (int u = 0; u < SU; ++u) {
#pragma unroll
                for (int j = SW - 1; j >= 0; --j)
                    if (j < nu[u]) v[u] -= (rd[u] * cf[u][j]) * wv[u][j];
                if (base + u * g.size() < e) {
                    w[slot[u]] = v[u];
                    d += double(v[u]) * double(rr[u]);
                }
            }
        }
    } else {
        for (int i = b + g.rank(); i < e; i += g.size()) {
            const int p = S.bwdMirror ? i : S.bwdSlot[i];
            const int nup = S.cnt[p] >> 16;
            const T rdp = S.rD[p];
            T v = w[p];
            for (int j = nup - 1; j >= 0; --j) v -= (rdp * S.up[j * n + p]) * w[S.upSrc[j * n + p]];
            w[p] = v;
            if (r) d += double(v) * double(r[p]);
        }
    }
}

// w = M^-1 r; returns the group sum of w.r when wantDot (else 0).
template <class G, class T>
__device__ __forceinline__ double s_precondition(G& g, const SlotSys<T>& S, const T* r, T* w, bool wantDot) {
    double d = 0.0;
    if (S.precond == CFX_PRE_DIC || S.precond == CFX_PRE_DILU) {
        for (int L = 0; L < S.nFwd; ++L) {
            fwd_level(g, S, S.fwdLevelStart[L], S.fwdLevelStart[L + 1], r, w);
            g.sync();
        }
        for (int L = 0; L < S.nBwd; ++L) {
            bwd_level(g, S, L, w, wantDot ? r : nullptr, d);
            g.sync();
        }
    } else {
        for (int p = g.rank(); p < S.n; p += g.size()) {
            const T v = S.precond == CFX_PRE_DIAGONAL ? S.rD[p] * r[p] : r[p];
            w[p] = v;
            if (wantDot) d += double(v) * double(r[p]);
        }
        g.sync();
    }
    return wantDot ? g.sum(d) : 0.0;
}

// ---------------------------------------------------------------- pointwise
// Element-wise loops: each thread loads PU elements (ld) before it stores
// any of them (st), so the loads of a round are in flight together.
constexpr int PU = 4;

template <class T>
struct V2 {
    T a, b;
};
template <class T>
struct V3 {
    T a, b, c;
};
template <class T>
struct V4 {
    T a, b, c, d;
};

template <class G, class Ld, class St>
__device__ __forceinline__ void pw(const G& g, int n, Ld&& ld, St&& st) {
    using V = decltype(ld(0));
    for (int base = g.rank(); base < n; base += PU * g.size()) {
        V v[PU];
#pragma unroll
        for (int u = 0; u < PU; ++u) {
            const int p = base + u * g.size();
            v[u] = ld(p < n ? p : 0);
        }
#pragma unroll
        for (int u = 0; u < PU; ++u) {
            const int p = base + u * g.size();
            if (p < n) st(p, v[u]);
        }
    }
}

// ---------------------------------------------------------------- A x
// y = A x over all slots; returns the group sum of y.x when wantDot.
template <class G, class T>
__device__ __forceinline__ double s_amul(G& g, const SlotSys<T>& S, const T* x, T* y, bool wantDot) {
    const int n = S.n, wl = S.wLo, wu = S.wUp;
    double d = 0.0;
    if (fast(S)) {
        for (int base = g.rank(); base < n; base += SU * g.size()) {
            T acc[SU], xp[SU], cf[SU][SW], xv[SU][SW];
            int src[SU][SW], cn[SU];
#pragma unroll
            for (int u = 0; u < SU; ++u) {
                const int p = base + u * g.size();
                const int q = p < n ? p : 0;
                cn[u] = S.cnt[q];
                xp[u] = x[q];
                acc[u] = S.diag[q];
#pragma unroll
                for (int j = 0; j < SW; ++j)
                    if (j < wl) {
                        cf[u][j] = S.lo[j * n + q];
                        src[u][j] = S.loSrc[j * n + q];
                    }
            }
#pragma unroll
            for (int u = 0; u < SU; ++u) {
                acc[u] = acc[u] * xp[u];
#pragma unroll
                for (int j = 0; j < SW; ++j)
                    if (j < wl) xv[u][j] = x[src[u][j]];
            }
            // lower part, then the upper coefficients into the same registers
#pragma unroll
            for (int u = 0; u < SU; ++u) {
                const int q = base + u * g.size() < n ? base + u * g.size() : 0;
#pragma unroll
                for (int j = 0; j < SW; ++j)
                    if (j < (cn[u] & 0xffff)) acc[u] += cf[u][j] * xv[u][j];
#pragma unroll
                for (int j = 0; j < SW; ++j)
                    if (j < wu) {
                        cf[u][j] = S.up[j * n + q];
                        src[u][j] = S.upSrc[j * n + q];
                    }
            }
#pragma unroll
            for (int u = 0; u < SU; ++u)
#pragma unroll
                for (int j = 0; j < SW; ++j)
                    if (j < wu) xv[u][j] = x[src[u][j]];
#pragma unroll
            for (int u = 0; u < SU; ++u) {
#pragma unroll
                for (int j = 0; j < SW; ++j)
                    if (j < (cn[u] >> 16)) acc[u] += cf[u][j] * xv[u][j];
                const int p = base + u * g.size();
                if (p < n) {
                    y[p] = acc[u];
                    d += double(acc[u]) * double(xp[u]);
                }
            }
        }
    } else {
        for (int p = g.rank(); p < n; p += g.size()) {
            const int c = S.cnt[p];
            T acc = S.diag[p] * x[p];
            for (int j = 0; j < (c & 0xffff); ++j) acc += S.lo[j * n + p] * x[S.loSrc[j * n + p]];
            for (int j = 0; j < (c >> 16); ++j) acc += S.up[j * n + p] * x[S.upSrc[j * n + p]];
            y[p] = acc;
            d += double(acc) * double(x[p]);
        }
    }
    if (wantDot) return g.sum(d);
    g.sync();
    return 0.0;
}

// sumA of slot p: diag, the lower coefficients, then the upper ones.
template <class T>
__device__ __forceinline__ T s_sumA(const SlotSys<T>& S, int p) {
    const int c = S.cnt[p];
    T a = S.diag[p];
    for (int j = 0; j < (c & 0xffff); ++j) a += S.lo[j * S.n + p];
    for (int j = 0; j < (c >> 16); ++j) a += S.up[j * S.n + p];
    return a;
}

// Preconditioner set-up: DIC/DILU pivots D[c] = diag[c] - sum up lo / D[l]
// in forward level order, then rD = 1/D; diagonal: rD = 1/diag.
template <class G, class T>
__device__ __forceinline__ void s_setup(G& g, const SlotSys<T>& S) {
    T* rD = S.rD;
    const int n = S.n;
    if (S.precond == CFX_PRE_DIC || S.precond == CFX_PRE_DILU) {
        const T* ul = S.upLo ? S.upLo : S.lo;
        for (int L = 0; L < S.nFwd; ++L) {
            for (int p = S.fwdLevelStart[L] + g.rank(); p < S.fwdLevelStart[L + 1]; p += g.size()) {
                const int nl = S.cnt[p] & 0xffff;
                T D = S.diag[p];
                for (int j = 0; j < nl; ++j) D -= (ul[j * n + p] * S.lo[j * n + p]) / rD[S.loSrc[j * n + p]];
                rD[p] = D;
            }
            g.sync();
        }
        for (int p = g.rank(); p < n; p += g.size()) rD[p] = T(1) / rD[p];
    } else if (S.precond == CFX_PRE_DIAGONAL) {
        for (int p = g.rank(); p < n; p += g.size()) rD[p] = T(1) / S.diag[p];
    }
    g.sync();
}

template <class T>
__device__ __forceinline__ bool s_check(const SlotSys<T>& S, double fin, double ini) {
    return fin < S.tolerance || (S.relTol > SP_SMALL && fin < S.relTol * ini);
}

// normFactor with psi (slot order) and b: sumA*gAverage(psi) = t,
// sum(|A psi - t| + |b - t|) + small; also r = b - A psi (and r0 = r).
// Returns normFactor; *mag = sum|r|.
template <class G, class T>
__device__ __forceinline__ double s_norm_init(G& g, SlotSys<T>& S, const T* psi, const T* b, double* mag) {
    const int n = S.n;
    double s0 = 0.0;
    for (int p = g.rank(); p < n; p += g.size()) s0 += double(psi[p]);
    const double avg = g.sum(s0) / n;
    s_amul(g, S, psi, S.q, false);
    double nf = 0.0, mg = 0.0;
    for (int p = g.rank(); p < n; p += g.size()) {
        const T t = s_sumA(S, p) * T(avg);
        const T qp = S.q[p], bp = b[p];
        nf += double(fabs(qp - t) + fabs(bp - t));
        const T rc = bp - qp;
        S.r[p] = rc;
        if (S.r0) S.r0[p] = rc;
        mg += fabs(double(rc));
    }
    const double normFactor = g.sum(nf) + SP_SMALL;
    *mag = g.sum(mg);
    return normFactor;
}

// ---------------------------------------------------------------- solves
// One PCG / PBiCGStab solve of S (slot order: S.psi, S.b) by group g, the
// reference's loop; S.rD must be set up.
template <class G, class T>
__device__ __noinline__ void s_solve(G& g, SlotSys<T>& S) {
    const int n = S.n;
    const int r0_ = g.rank(), st_ = g.size();
    T* psi = S.psi;
    double mg;
    const double normFactor = s_norm_init(g, S, psi, S.b, &mg);
    const double initial = mg / normFactor;
    double fin = initial;
    int nIter = 0, converged = s_check(S, fin, initial), singular = 0;
    if (S.minIter > 0 || !converged) {
        if (S.solver == CFX_SOLVER_PCG) {
            double wArA = SP_GREAT, wArAold;
            do {
                wArAold = wArA;
                wArA = s_precondition(g, S, S.r, S.w, true);
                const T beta = T(wArA / wArAold);
                const bool first = nIter == 0;
                pw(g, n, [&](int c) { return V2<T>{S.w[c], S.p[c]}; },
                   [&](int c, const V2<T>& v) { S.p[c] = first ? v.a : v.a + beta * v.b; });
                g.sync();
                const double wApA = s_amul(g, S, S.p, S.w, true);
                singular = fabs(wApA) / normFactor < VSMALL;
                if (singular) break;
                const T alpha = T(wArA / wApA);
                mg = 0.0;
                pw(g, n, [&](int c) { return V4<T>{psi[c], S.p[c], S.r[c], S.w[c]}; },
                   [&](int c, const V4<T>& v) {
                       psi[c] = v.a + alpha * v.b;
                       const T rc = v.c - alpha * v.d;
                       S.r[c] = rc;
                       mg += fabs(double(rc));
                   });
                fin = g.sum(mg) / normFactor;
                bool cont = false;
                if (++nIter < S.maxIter) {
                    converged = s_check(S, fin, initial);
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
                    pw(g, n, [&](int c) { return S.r[c]; }, [&](int c, T v) { S.p[c] = v; });
                } else {
                    singular = fabs(omega) < VSMALL;
                    if (singular) break;
                    const T beta = T((rA0rA / rA0rAold) * (alpha / omega));
                    pw(g, n, [&](int c) { return V3<T>{S.r[c], S.p[c], S.q[c]}; },
                       [&](int c, const V3<T>& v) { S.p[c] = v.a + beta * (v.b - T(omega) * v.c); });
                }
                g.sync();
                s_precondition(g, S, S.p, S.w, false);  // yA = w
                s_amul(g, S, S.w, S.q, false);          // AyA = q
                d = 0.0;
                for (int c = r0_; c < n; c += st_) d += double(S.r0[c]) * double(S.q[c]);
                alpha = rA0rA / g.sum(d);
                mg = 0.0;
                pw(g, n, [&](int c) { return V2<T>{S.r[c], S.q[c]}; },
                   [&](int c, const V2<T>& x) {
                       const T v = x.a - T(alpha) * x.b;
                       S.s[c] = v;
                       mg += fabs(double(v));
                   });
                fin = g.sum(mg) / normFactor;
                if (++nIter >= S.minIter && (converged = s_check(S, fin, initial))) {
                    pw(g, n, [&](int c) { return V2<T>{psi[c], S.w[c]}; },
                       [&](int c, const V2<T>& v) { psi[c] = v.a + T(alpha) * v.b; });
                    g.sync();
                    break;
                }
                s_precondition(g, S, S.s, S.t, false);  // zA = t
                s_amul(g, S, S.t, S.r, false);          // tA, kept in r
                double tt = 0.0, ts = 0.0;
                for (int c = r0_; c < n; c += st_) {
                    const T v = S.r[c];
                    tt += double(v) * double(v);
                    ts += double(v) * double(S.s[c]);
                }
                const double tAtA = g.sum(tt);
                omega = g.sum(ts) / tAtA;
                mg = 0.0;
                pw(g, n, [&](int c) { return V3<T>{psi[c], S.w[c], S.t[c]}; },
                   [&](int c, const V3<T>& v) { psi[c] = v.a + (T(alpha) * v.b + T(omega) * v.c); });
                pw(g, n, [&](int c) { return V2<T>{S.s[c], S.r[c]}; },
                   [&](int c, const V2<T>& x) {
                       const T v = x.a - T(omega) * x.b;
                       S.r[c] = v;
                       mg += fabs(double(v));
                   });
                fin = g.sum(mg) / normFactor;
                bool cont = false;
                if (nIter < S.maxIter) {
                    converged = s_check(S, fin, initial);
                    cont = !converged;
                }
                if (!(cont || nIter < S.minIter)) break;
            } while (true);
        }
    }
    if (threadIdx.x == 0) {  // every CTA's copy of the record
        S.initialResidual = initial;
        S.finalResidual = fin;
        S.nIterations = nIter;
        S.converged = converged;
        S.singular = singular;
    }
    g.sync();
}

// One system of a batch by group g: gather psi and b into slot order, solve
// (plain: the reference loop in the record's precision; mixed: FP64
// iterative refinement, normFactor, residuals, psi and the convergence test
// in FP64 with the reference's definitions, around FP32 solves of A e = r by
// the same solver and preconditioner reducing the residual by innerRelTol),
// scatter psi back.  nIterations counts the inner iterations, nOuter the
// refinement steps.
template <class G>
__device__ __noinline__ void batch_one(G& g, SlotSys<double>& S, SlotSys<float>* Ep, int mixed, double innerRelTol,
                          int maxOuter) {
    const int n = S.n;
    const int r0_ = g.rank(), st_ = g.size();
    for (int p = r0_; p < n; p += st_) {
        const int c = S.cellOf[p];
        S.psi[p] = S.psiCell[c];
        S.b[p] = S.bCell[c];
    }
    g.sync();
    if (!mixed) {
        s_setup(g, S);
        s_solve(g, S);
    } else {
        SlotSys<float>& E = *Ep;
        s_setup(g, E);
        double mg;
        const double normFactor = s_norm_init(g, S, S.psi, S.b, &mg);
        const double initial = mg / normFactor;
        double fin = initial;
        int outer = 0, inner = 0, singular = 0;
        while (!s_check(S, fin, initial) && outer < maxOuter) {
            pw(g, n, [&](int p) { return S.r[p]; }, [&](int p, double v) {
                E.b[p] = float(v);
                E.psi[p] = 0.0f;
            });
            if (threadIdx.x == 0) {
                E.tolerance = 0.0;
                E.relTol = innerRelTol;
            }
            g.sync();
            s_solve(g, E);
            inner += E.nIterations;
            if (E.singular || E.nIterations == 0) {
                singular = E.singular;
                break;
            }
            pw(g, n, [&](int p) { return V2<double>{S.psi[p], double(E.psi[p])}; },
               [&](int p, const V2<double>& v) { S.psi[p] = v.a + v.b; });
            g.sync();
            s_amul(g, S, S.psi, S.q, false);
            mg = 0.0;
            pw(g, n, [&](int p) { return V2<double>{S.b[p], S.q[p]}; },
               [&](int p, const V2<double>& v) {
                   const double rc = v.a - v.b;
                   S.r[p] = rc;
                   mg += fabs(rc);
               });
            fin = g.sum(mg) / normFactor;
            ++outer;
        }
        if (threadIdx.x == 0) {
            S.initialResidual = initial;
            S.finalResidual = fin;
            S.nIterations = inner;
            S.converged = s_check(S, fin, initial);
            S.singular = singular;
            S.nOuter = outer;
        }
    }
    for (int p = r0_; p < n; p += st_) S.psiCell[S.cellOf[p]] = S.psi[p];
    g.sync();
}

// The records are copied into shared memory for the solve (each CTA of a
// cluster holds its own copy, all kept identical), so their fields are read
// from shared memory instead of occupying registers; the results go back to
// the global record at the end.
__device__ __forceinline__ void load_records(const SlotSys<double>* s64, const SlotSys<float>* s32, int i,
                                             SlotSys<double>& a, SlotSys<float>& e) {
    if (threadIdx.x == 0) {
        a = s64[i];
        if (s32) e = s32[i];
    }
    __syncthreads();
}

__device__ __forceinline__ void store_results(SlotSys<double>* s64, int i, const SlotSys<double>& a,
                                              unsigned long long t0) {
    SlotSys<double>& o = s64[i];
    o.initialResidual = a.initialResidual;
    o.finalResidual = a.finalResidual;
    o.nIterations = a.nIterations;
    o.converged = a.converged;
    o.singular = a.singular;
    o.nOuter = a.nOuter;
    o.tStart = t0;
    o.tEnd = globaltimer_ns();
}

// The finished system's result to host-mapped memory, flag last (one
// thread, after every thread of the system's CTAs fenced its stores).
__device__ __forceinline__ void publish(BatchDone* done, int i, const SlotSys<double>& a) {
    BatchDone& d = done[i];
    d.initialResidual = a.initialResidual;
    d.finalResidual = a.finalResidual;
    d.nIterations = a.nIterations;
    d.converged = a.converged;
    d.singular = a.singular;
    d.nOuter = a.nOuter;
    __threadfence_system();
    *reinterpret_cast<volatile unsigned*>(&d.flag) = 1u;
}

// Persistent batch, one CTA per system: each CTA takes the next system from
// next[1] until all are done (the host orders them largest first).
__global__ void __launch_bounds__(BLK_NT, 2) batch_k(SlotSys<double>* s64, SlotSys<float>* s32, int nSys, int mixed,
                                                     double innerRelTol, int maxOuter, unsigned* next,
                                                     BatchDone* done) {
    __shared__ double sh[BLK_NT / 32 + 1];
    __shared__ int sIdx;
    __shared__ SlotSys<double> rec;
    __shared__ SlotSys<float> rec32;
    CtaGroup g{sh};
    for (;;) {
        if (threadIdx.x == 0) sIdx = int(atomicAdd(next + 1, 1u));
        __syncthreads();
        const int i = sIdx;
        __syncthreads();
        if (i >= nSys) return;
        const unsigned long long t0 = globaltimer_ns();
        load_records(s64, s32, i, rec, rec32);
        batch_one(g, rec, &rec32, mixed, innerRelTol, maxOuter);
        if (done) {
            __threadfence_system();
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            store_results(s64, i, rec, t0);
            if (done) publish(done, i, rec);
        }
        __syncthreads();
    }
}

// Persistent batch with thread-block clusters.  Phase 1: each cluster takes
// the next of the first nBig systems (the largest) from next[0] and solves it
// with all its CTAs.  Phase 2, once those are handed out: every CTA takes
// the remaining systems one at a time from next[1], as batch_k.  No CTA
// touches another's shared memory after phase 1's last cluster barrier.
__global__ void __launch_bounds__(BLK_NT, 2) batch_cluster_k(SlotSys<double>* s64, SlotSys<float>* s32, int nSys,
                                                             int nBig, int mixed, double innerRelTol, int maxOuter,
                                                             unsigned* next, BatchDone* done) {
    __shared__ double sh[BLK_NT / 32 + 1];
    __shared__ double slot[2];
    __shared__ int sIdx;
    __shared__ SlotSys<double> rec;
    __shared__ SlotSys<float> rec32;
    cg::cluster_group cl = cg::this_cluster();
    ClusterGroup cgp{sh, slot, 0, int(cl.block_rank()), int(cl.num_blocks())};
    for (;;) {
        if (cgp.crank == 0 && threadIdx.x == 0) sIdx = int(atomicAdd(next, 1u));
        cl.sync();
        const int i = *cl.map_shared_rank(&sIdx, 0);
        cl.sync();
        if (i >= nBig) break;
        const unsigned long long t0 = globaltimer_ns();
        load_records(s64, s32, i, rec, rec32);
        batch_one(cgp, rec, &rec32, mixed, innerRelTol, maxOuter);
        if (done) {
            __threadfence_system();
            cl.sync();
        }
        if (cgp.leader()) {
            store_results(s64, i, rec, t0);
            if (done) publish(done, i, rec);
        }
        __syncthreads();
    }
    CtaGroup g{sh};
    for (;;) {
        if (threadIdx.x == 0) sIdx = nBig + int(atomicAdd(next + 1, 1u));
        __syncthreads();
        const int i = sIdx;
        __syncthreads();
        if (i >= nSys) return;
        const unsigned long long t0 = globaltimer_ns();
        load_records(s64, s32, i, rec, rec32);
        batch_one(g, rec, &rec32, mixed, innerRelTol, maxOuter);
        if (done) {
            __threadfence_system();
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            store_results(s64, i, rec, t0);
            if (done) publish(done, i, rec);
        }
        __syncthreads();
    }
}
}  // namespace

void launch_batch(cudaStream_t s, SlotSys<double>* s64, SlotSys<float>* s32, int nSys, int nCta, int mixed,
                  double innerRelTol, int maxOuter, unsigned* next, BatchDone* done) {
    batch_k<<<nCta, BLK_NT, 0, s>>>(s64, s32, nSys, mixed, innerRelTol, maxOuter, next, done);
    count_launch();
}

cudaError_t launch_batch_cluster(cudaStream_t s, SlotSys<double>* s64, SlotSys<float>* s32, int nSys, int nBig,
                                 int clusterSize, int nClusters, int mixed, double innerRelTol, int maxOuter,
                                 unsigned* next, BatchDone* done) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(clusterSize * nClusters);
    cfg.blockDim = dim3(BLK_NT);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = clusterSize;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e =
        cudaLaunchKernelEx(&cfg, batch_cluster_k, s64, s32, nSys, nBig, mixed, innerRelTol, maxOuter, next, done);
    if (e == cudaSuccess) count_launch();
    return e;
}

int batch_ctas_per_sm() {
    int k = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, batch_k, BLK_NT, 0) != cudaSuccess) return 1;
    return k > 0 ? k : 1;
}

int batch_max_clusters(int clusterSize) {
    if (clusterSize > 8 &&
        cudaFuncSetAttribute(batch_cluster_k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(clusterSize);
    cfg.blockDim = dim3(BLK_NT);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = clusterSize;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, batch_cluster_k, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

}  // namespace cfx
