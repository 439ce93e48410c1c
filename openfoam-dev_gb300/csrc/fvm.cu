// fvm.cu - finite-volume assembly of a scalar transport equation on the
// device: fvm::ddt(psi) + fvm::div(phi, psi) +/- fvm::laplacian(gamma, psi)
// == su, written straight into a resident matrix so that PISO/PIMPLE
// correctors re-assemble without a host upload of coefficients.
//
// Every value is formed with the reference's arithmetic in the reference's
// order:
//   * each term as its scheme builds it: EulerDdtScheme.C:466-497,
//     gaussConvectionScheme.C:121-152 (upwind = pos0(phi), linear = mesh
//     weights), gaussLaplacianScheme.C:47-89 with gammaMagSf = gamma*magSf,
//     and the patch coefficients of fixedValue, zeroGradient, fixedGradient;
//   * each term's diagonal by its own negSumDiag (lduMatrixOperations.C:
//     55-74): one thread per cell subtracts, in face order, Upper of the faces
//     it neighbours, then Lower of the faces it owns;
//   * the terms combined as fvMatrix::operator+=/-= (fvMatrix.C:1094-1148)
//     and lduMatrix::operator+=/-= (lduMatrixOperations.C:159-318), including
//     the diagonal-matrix copy and the symmetric->asymmetric lower() copy;
//   * operator==(fvMatrix, field): source += V*su (fvMatrix.C:1705-1715);
//   * fvMatrix::solveSegregated's addBoundaryDiag / addBoundarySource
//     (fvMatrix.C:112-174): each cell adds its boundary faces' coefficients
//     in patch-then-face order, the cyclic faces' internalCoeffs to the
//     diagonal only; their boundaryCoeffs and internalCoeffs become the
//     solver's interfaceBouCoeffs / interfaceIntCoeffs (coupledFvPatchField
//     coefficients, coupledFvPatchField.C:157-205).
// Compiled with --fmad=false like the rest of the library: no contraction.

#include "internal.h"
#include "solvers.h"

namespace cfx {

namespace {

constexpr int FV_NT = 256;

struct FaceTerms {
    double lapU;           // laplacian upper (= lower)
    double divL, divU;     // div lower, upper
};

__device__ __forceinline__ double div_weight(const FvmArgs& a, const FvGeom& g, int f) {
    return a.divScheme == 0 ? (a.phi[f] >= 0.0 ? 1.0 : 0.0) : g.weights[f];
}

__device__ __forceinline__ FaceTerms face_terms(const FvmArgs& a, const FvGeom& g, int f) {
    FaceTerms t{0.0, 0.0, 0.0};
    if (a.hasDiv) {
        t.divL = -div_weight(a, g, f) * a.phi[f];
        t.divU = t.divL + a.phi[f];
    }
    if (a.lapSign) {
        const double gms = (a.gamma ? a.gamma[f] : a.gammaUniform) * g.magSf[f];
        t.lapU = g.deltaCoeffs[f] * gms;
    }
    return t;
}

// The combined upper/lower of one face: the first term's, then the others
// by lduMatrix::operator+=/-= (a ddt term has neither and starts a diagonal
// matrix, which the next term's coefficients are copied into).
__device__ __forceinline__ void face_combined(const FvmArgs& a, const FaceTerms& t, double& U, double& L,
                                              bool& hasU, bool& hasL) {
    hasU = hasL = false;
    U = L = 0.0;
    if (a.hasDiv) {
        if (!a.hasDdt) {
            L = t.divL;
            U = t.divU;
        } else {  // diagonal += asymmetric: copies
            U = t.divU;
            L = t.divL;
        }
        hasU = hasL = true;
    }
    if (a.lapSign) {
        if (!hasU && !hasL) {
            if (a.hasDdt)  // diagonal +/-= symmetric: upper = +/- A.upper
                U = a.lapSign > 0 ? t.lapU : -t.lapU;
            else  // the first term; "-laplacian" negates it
                U = a.lapSign > 0 ? t.lapU : -t.lapU;
            hasU = true;
        } else {  // asymmetric +/-= symmetric: lower, then upper
            if (a.lapSign > 0) {
                L += t.lapU;
                U += t.lapU;
            } else {
                L -= t.lapU;
                U -= t.lapU;
            }
        }
    }
}

constexpr int BC_CYCLIC = 3;

// One boundary face's combined internal and boundary coefficients.  A
// cyclic face takes the coupled patch coefficients: value (w, 1 - w) with the
// upwind weight pos0(phi), gradient (-deltaCoeffs, deltaCoeffs).
__device__ __forceinline__ void boundary_combined(const FvmArgs& a, const FvGeom& g, int b, double& ic, double& bc) {
    const int type = a.bcType[b];
    double divIc = 0.0, divBc = 0.0, lapIc = 0.0, lapBc = 0.0;
    if (a.hasDiv) {
        if (type == BC_CYCLIC) {
            const double w = a.phiB[b] >= 0.0 ? 1.0 : 0.0;
            divIc = a.phiB[b] * (1.0 * w);
            divBc = -a.phiB[b] * (1.0 * (1.0 - w));
        } else {
            const double vic = type == 1 ? 0.0 : 1.0;
            const double vbc = type == 1 ? a.bcValue[b] : type == 2 ? a.bcValue[b] / g.deltaCoeffsB[b] : 0.0;
            divIc = a.phiB[b] * vic;
            divBc = -a.phiB[b] * vbc;
        }
    }
    if (a.lapSign) {
        const double gms = (a.gammaB ? a.gammaB[b] : a.gammaUniform) * g.magSfB[b];
        const double gic = type == 1 || type == BC_CYCLIC ? -1.0 * g.deltaCoeffsB[b] : 0.0;
        const double gbc = type == BC_CYCLIC ? -gic
                           : type == 1 ? g.deltaCoeffsB[b] * a.bcValue[b] : type == 2 ? a.bcValue[b] : 0.0;
        lapIc = gms * gic;
        lapBc = -gms * gbc;
    }
    // combination in term order; a ddt term starts from zero fields
    bool started = false;
    ic = bc = 0.0;
    if (a.hasDdt) started = true;
    if (a.hasDiv) {
        if (started) {
            ic += divIc;
            bc += divBc;
        } else {
            ic = divIc;
            bc = divBc;
        }
        started = true;
    }
    if (a.lapSign) {
        if (started) {
            if (a.lapSign > 0) {
                ic += lapIc;
                bc += lapBc;
            } else {
                ic -= lapIc;
                bc -= lapBc;
            }
        } else {
            ic = a.lapSign > 0 ? lapIc : -lapIc;
            bc = a.lapSign > 0 ? lapBc : -lapBc;
        }
    }
}

// One thread per cell: the diagonal and source of the cell, and the
// combined upper/lower of the faces it owns (each face has one owner).
__global__ void __launch_bounds__(FV_NT) fvm_cells_k(int n, const int* __restrict__ ownerStart,
                                                     const int* __restrict__ losortStart,
                                                     const int* __restrict__ losort, FvGeom g, FvmArgs a,
                                                     double* __restrict__ diag, double* __restrict__ source,
                                                     double* __restrict__ upper, double* __restrict__ lower) {
    for (int c = blockIdx.x * FV_NT + threadIdx.x; c < n; c += gridDim.x * FV_NT) {
        // each term's negSumDiag: faces c neighbours (ascending, they precede
        // the faces c owns), subtracting Upper; then owned faces, Lower
        double dDiv = 0.0, dLap = 0.0;
        const int k1 = losortStart[c + 1];
        for (int k = losortStart[c]; k < k1; ++k) {
            const FaceTerms t = face_terms(a, g, losort[k]);
            dDiv -= t.divU;
            dLap -= t.lapU;
        }
        const int f1 = ownerStart[c + 1];
        for (int f = ownerStart[c]; f < f1; ++f) {
            const FaceTerms t = face_terms(a, g, f);
            dDiv -= t.divL;
            dLap -= t.lapU;
            double U, L;
            bool hasU, hasL;
            face_combined(a, t, U, L, hasU, hasL);
            upper[f] = U;
            if (lower) lower[f] = L;
        }
        double D = 0.0, S = 0.0;
        bool started = false;
        if (a.hasDdt) {
            D = a.rDeltaT * g.V[c];
            S = a.rDeltaT * a.psi0[c] * g.V[c];
            started = true;
        }
        if (a.hasDiv) {
            if (started) {
                D += dDiv;
                S += 0.0;
            } else {
                D = dDiv;
            }
            started = true;
        }
        if (a.lapSign) {
            if (started) {
                if (a.lapSign > 0) {
                    D += dLap;
                    S += 0.0;
                } else {
                    D -= dLap;
                    S -= 0.0;
                }
            } else if (a.lapSign > 0) {
                D = dLap;
            } else {
                D = -dLap;
                S = -S;
            }
        }
        if (a.su) S += g.V[c] * a.su[c];
        const int b1 = g.bStart[c + 1];
        for (int k = g.bStart[c]; k < b1; ++k) {
            double ic, bc;
            const int b = g.bFace[k];
            boundary_combined(a, g, b, ic, bc);
            D += ic;
            if (a.bcType[b] != BC_CYCLIC) S += bc;
        }
        diag[c] = D;
        source[c] = S;
    }
}

// The cyclic faces' coefficients as the solver's interface coefficients:
// one CTA walks the boundary faces in order, numbering the cyclic ones with
// a block-wide prefix count.
constexpr int FVI_NT = 1024;

__global__ void __launch_bounds__(FVI_NT) fvm_iface_k(FvGeom g, FvmArgs a, int nIf, const int* __restrict__ ifPos,
                                                      double* __restrict__ ifBou, double* __restrict__ ifInt,
                                                      int* status) {
    __shared__ int warpCount[FVI_NT / 32];
    __shared__ int base;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) base = 0;
    __syncthreads();
    for (int b0 = 0; b0 < g.nBoundary; b0 += FVI_NT) {
        const int b = b0 + threadIdx.x;
        const bool cyc = b < g.nBoundary && a.bcType[b] == BC_CYCLIC;
        const unsigned m = __ballot_sync(0xffffffffu, cyc);
        if (lane == 0) warpCount[w] = __popc(m);
        __syncthreads();
        int before = base;
        for (int i = 0; i < w; ++i) before += warpCount[i];
        const int k = before + __popc(m & ((1u << lane) - 1u));
        if (cyc) {
            if (a.hasDiv && a.divScheme != 0) {
                *status = CFX_ERR_ARG;  // linear weights of a cyclic patch are not given
            } else if (k < nIf) {
                double ic, bc;
                boundary_combined(a, g, b, ic, bc);
                ifBou[ifPos[k]] = bc;
                ifInt[ifPos[k]] = ic;
            }
        }
        __syncthreads();
        if (threadIdx.x == FVI_NT - 1) {
            int total = 0;
            for (int i = 0; i < FVI_NT / 32; ++i) total += warpCount[i];
            base += total;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0 && base != nIf) *status = CFX_ERR_ARG;
}

inline int fv_grid(int n) {
    int g = (n + FV_NT - 1) / FV_NT;
    return g < 1 ? 1 : (g > 152 * 16 ? 152 * 16 : g);
}

}  // namespace

void launch_fvm_interfaces(cudaStream_t s, const FvGeom& g, const FvmArgs& a, int nIf, const int* ifPos,
                           double* ifBou, double* ifInt, int* status) {
    fvm_iface_k<<<1, FVI_NT, 0, s>>>(g, a, nIf, ifPos, ifBou, ifInt, status);
    count_launch();
}

void launch_fvm_assemble(cudaStream_t s, const LevelMesh& m, const FvGeom& g, const FvmArgs& a, double* diag,
                         double* upper, double* lower, double* source) {
    fvm_cells_k<<<fv_grid(m.n), FV_NT, 0, s>>>(m.n, m.ownerStart, m.losortStart, m.losort, g, a, diag, source,
                                               upper, lower);
    count_launch();
}

}  // namespace cfx
