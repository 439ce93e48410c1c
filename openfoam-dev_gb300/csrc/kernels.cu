// kernels.cu - streaming LDU kernels: Amul/Tmul/residual/sumA as row gathers,
// coefficient permutation, GAMG coarse assembly, restriction/prolongation,
// deterministic reductions, precision casts.
//
// Row gather order.  The reference scatters face by face
// (lduMatrixATmul.C:66-79): y[u] += lower*x[l]; y[l] += upper*x[u].  Faces
// are owner-sorted and l < u, so the contributions that reach cell c arrive
// first from the faces where c is the neighbour (in face order = losort
// order), then from the faces c owns (ownerStart order).  The gathers below
// add them in exactly that order, without atomics, and the library is built
// with --fmad=false, so every result equals the reference's sequential loop
// bit for bit.

#include <cfloat>

#include "device.cuh"
#include "internal.h"
#include "solvers.h"

namespace cfx {

namespace {

// one element per thread (streaming kernels without block partials)
inline int grid_all(int64_t n, int nt = RED_NT) {
    int64_t b = (n + nt - 1) / nt;
    if (b < 1) b = 1;
    if (b > (int64_t(1) << 30)) b = int64_t(1) << 30;
    return int(b);
}

inline int grid_for(int64_t n, int nt = RED_NT) {
    int64_t b = (n + nt - 1) / nt;
    if (b < 1) b = 1;
    if (b > RED_MAXB) b = RED_MAXB;
    return int(b);
}

template <class T>
__global__ void __launch_bounds__(RED_NT) amul_k(int n, const int* __restrict__ ownerStart,
                                                 const int* __restrict__ losortStart,
                                                 const int* __restrict__ losortL, const int* __restrict__ u,
                                                 const T* __restrict__ diag, const T* __restrict__ lp,
                                                 const T* __restrict__ upper, Sell<T> S, const T* __restrict__ x,
                                                 T* __restrict__ y, Iface<T> itf) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x)
        y[c] = iface_sub(itf, c, x, row_ax<T>(c, ownerStart, losortStart, losortL, u, diag, lp, upper, S, x));
}

template <class T>
__global__ void __launch_bounds__(RED_NT) residual_k(int n, const int* __restrict__ ownerStart,
                                                     const int* __restrict__ losortStart,
                                                     const int* __restrict__ losortL, const int* __restrict__ u,
                                                     const T* __restrict__ diag, const T* __restrict__ lp,
                                                     const T* __restrict__ upper, Sell<T> S,
                                                     const T* __restrict__ x, const T* __restrict__ b,
                                                     T* __restrict__ r, Iface<T> itf) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x)
        r[c] = iface_sub_neg(itf, c, x, row_res<T>(c, ownerStart, losortStart, losortL, u, diag, lp, upper, S, x, b));
}

template <class T>
__global__ void __launch_bounds__(RED_NT) sumA_k(int n, const int* __restrict__ ownerStart,
                                                 const int* __restrict__ losortStart, const T* __restrict__ diag,
                                                 const T* __restrict__ lp, const T* __restrict__ upper,
                                                 T* __restrict__ s, Iface<T> itf) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        T acc = diag[c];
        const int k1 = losortStart[c + 1];
        for (int k = losortStart[c]; k < k1; ++k) acc += lp[k];
        const int f1 = ownerStart[c + 1];
        for (int f = ownerStart[c]; f < f1; ++f) acc += upper[f];
        // lduMatrix::sumA (lduMatrixATmul.C:185-198): minus the interface
        // boundary coefficients
        if (itf.start)
            for (int j = itf.start[c]; j < itf.start[c + 1]; ++j) acc -= itf.coef[j];
        s[c] = acc;
    }
}

template <class T>
__global__ void permute_k(int nf, const int* __restrict__ losort, const T* __restrict__ lower,
                          const T* __restrict__ upper, T* __restrict__ lowerPerm, T* __restrict__ upperPerm) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nf; k += gridDim.x * blockDim.x) {
        const int f = losort[k];
        lowerPerm[k] = lower[f];
        if (upperPerm) upperPerm[k] = upper[f];
    }
}

// The coefficients in the level's sliced ELL order: a lower term from the
// losort-permuted lower coefficients, an upper term from upper.
template <class T>
__global__ void sell_pack_k(int64_t nE, const int* __restrict__ src, const T* __restrict__ lowerPerm,
                            const T* __restrict__ upper, T* __restrict__ coef) {
    for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < nE; e += int64_t(gridDim.x) * blockDim.x) {
        const int sc = src[e];
        coef[e] = sc < 0 ? T(0) : (sc & SRC_UPPER) ? upper[sc & (SRC_UPPER - 1)] : lowerPerm[sc];
    }
}

// GAMGSolver::agglomerateMatrix (GAMGSolverAgglomerateMatrix.C:33-193): the
// coarse diagonal is the restricted fine diagonal (fine cells ascending), then
// the intra-cluster faces in fine-face order (2*upper when symmetric).
template <class T>
__global__ void coarse_diag_k(int nc, const int* __restrict__ ccStart, const int* __restrict__ ccFine,
                              const int* __restrict__ ifStart, const int* __restrict__ ifFine,
                              const T* __restrict__ fdiag, const T* __restrict__ fupper,
                              const T* __restrict__ flower, T* __restrict__ cdiag) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        T acc = T(0);
        for (int k = ccStart[c]; k < ccStart[c + 1]; ++k) acc += fdiag[ccFine[k]];
        for (int k = ifStart[c]; k < ifStart[c + 1]; ++k) {
            const int f = ifFine[k];
            acc += flower ? T(fupper[f] + flower[f]) : T(2 * fupper[f]);
        }
        cdiag[c] = acc;
    }
}

template <class T>
__global__ void coarse_faces_k(int ncf, const int* __restrict__ cfStart, const int* __restrict__ cfFine,
                               const int* __restrict__ flip, const T* __restrict__ fupper,
                               const T* __restrict__ flower, T* __restrict__ cupper, T* __restrict__ clower) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncf; c += gridDim.x * blockDim.x) {
        T up = T(0), lo = T(0);
        for (int k = cfStart[c]; k < cfStart[c + 1]; ++k) {
            const int f = cfFine[k];
            if (flower) {
                if (!flip[f]) {
                    up += fupper[f];
                    lo += flower[f];
                } else {
                    up += flower[f];
                    lo += fupper[f];
                }
            } else {
                up += fupper[f];
            }
        }
        cupper[c] = up;
        if (clower) clower[c] = lo;
    }
}

// GAMGAgglomeration::restrictField (GAMGAgglomerationTemplates.C:77-89) as a
// gather over the fine cells of each coarse cell, ascending.
template <class T>
__global__ void restrict_k(int nc, const int* __restrict__ ccStart, const int* __restrict__ ccFine,
                           const T* __restrict__ ff, T* __restrict__ cf) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        T acc = T(0);
        for (int k = ccStart[c]; k < ccStart[c + 1]; ++k) acc += ff[ccFine[k]];
        cf[c] = acc;
    }
}

// GAMGAgglomeration::prolongField (GAMGAgglomerationTemplates.C:171-219).
template <class T>
__global__ void prolong_k(int n, const int* __restrict__ ra, const T* __restrict__ cf, T* __restrict__ ff) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) ff[i] = cf[ra[i]];
}

// GAMGSolver::interpolate, first part (GAMGSolverInterpolate.C:30-79): the
// off-diagonal product (A - D) psi from zero, in the per-cell face order of
// the reference's face loop (neighbour faces in losort order, then owned).
template <class T>
__global__ void offdiag_amul_k(int n, const int* __restrict__ ownerStart, const int* __restrict__ losortStart,
                               const int* __restrict__ losortL, const int* __restrict__ u,
                               const T* __restrict__ lp, const T* __restrict__ upper, const T* __restrict__ x,
                               T* __restrict__ y, Iface<T> itf) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        T acc = T(0);
        const int k1 = losortStart[c + 1];
        for (int k = losortStart[c]; k < k1; ++k) acc += lp[k] * x[losortL[k]];
        const int f1 = ownerStart[c + 1];
        for (int f = ownerStart[c]; f < f1; ++f) acc += upper[f] * x[u[f]];
        // the interfaces' updateMatrixInterfaces (GAMGSolverInterpolate.C:60-67)
        y[c] = iface_sub(itf, c, x, acc);
    }
}

// GAMGInterface::agglomerateCoeffs (GAMGInterface.C:90-115) through
// restrictField: each coarse interface face sums its fine faces'
// coefficients from zero in the fine faces' order.
template <class T>
__global__ void iface_restrict_k(int nc, const int* __restrict__ start, const int* __restrict__ fineFaces,
                                 const T* __restrict__ fine, T* __restrict__ coarse) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nc; j += gridDim.x * blockDim.x) {
        T v = T(0);
        const int t1 = start[j + 1];
        for (int t = start[j]; t < t1; ++t) v += fine[fineFaces[t]];
        coarse[j] = v;
    }
}

// GAMGSolverInterpolate.C:69-127 for one coarse cell per thread, over its
// fine cells in ascending order (the order the reference's cell loop adds
// them in): psi = -Apsi/diag; corrC = psiC - sum(diag psi)/sum(diag);
// psi += corrC.
template <class T>
__global__ void interp_coarse_k(int nc, const int* __restrict__ ccStart, const int* __restrict__ ccFine,
                                const T* __restrict__ diag, const T* __restrict__ Apsi, const T* __restrict__ psiC,
                                T* __restrict__ psi) {
    for (int C = blockIdx.x * blockDim.x + threadIdx.x; C < nc; C += gridDim.x * blockDim.x) {
        const int k0 = ccStart[C], k1 = ccStart[C + 1];
        T corr = T(0), dg = T(0);
        for (int k = k0; k < k1; ++k) {
            const int c = ccFine[k];
            const T d = diag[c];
            const T p = -Apsi[c] / d;
            psi[c] = p;
            corr += d * p;
            dg += d;
        }
        const T cc = psiC[C] - corr / dg;
        for (int k = k0; k < k1; ++k) {
            const int c = ccFine[k];
            psi[c] = psi[c] + cc;
        }
    }
}

// LUscalarMatrix (LUscalarMatrix.C:205-266 convert, scalarMatrices.C:77-180
// LUDecompose) of one level in one block: the dense row-major matrix, the
// implicit row scaling, then Crout's column sweep with partial pivoting.
// Every sum runs in one thread in the reference's k order; the parallel
// parts (assembly, row scales, rows j..n-1 of a column, the row swap and
// the column scaling) touch disjoint entries.  An all-zero row sets
// *status = CFX_ERR_FATAL ("Singular matrix") and stops.
constexpr int LU_NT = 256;

template <class T>
__global__ void __launch_bounds__(LU_NT) lu_factor_k(int n, int nf, const int* __restrict__ l,
                                                     const int* __restrict__ u, const T* __restrict__ diag,
                                                     const T* __restrict__ upper, const T* __restrict__ lower,
                                                     int nIf, const int* __restrict__ ifRow,
                                                     const int* __restrict__ ifCol, const int* __restrict__ ifSrc,
                                                     const T* __restrict__ ifBou, T* __restrict__ A,
                                                     T* __restrict__ vv, int* __restrict__ piv, int* status) {
    __shared__ int singular, pivRow;
    const int t = threadIdx.x;
    const size_t nn = size_t(n) * n;
    for (size_t i = t; i < nn; i += LU_NT) A[i] = T(0);
    if (t == 0) singular = 0;
    __syncthreads();
    for (int c = t; c < n; c += LU_NT) A[size_t(c) * n + c] = diag[c];
    for (int f = t; f < nf; f += LU_NT) {
        A[size_t(u[f]) * n + l[f]] = lower[f];
        A[size_t(l[f]) * n + u[f]] = upper[f];
    }
    __syncthreads();
    // the cyclic interfaces, in the reference's patch then face order (one
    // thread: two faces may meet on one entry)
    if (t == 0)
        for (int k = 0; k < nIf; ++k) A[size_t(ifRow[k]) * n + ifCol[k]] -= ifBou[ifSrc[k]];
    __syncthreads();
    for (int i = t; i < n; i += LU_NT) {
        T big = T(0);
        for (int j = 0; j < n; ++j) {
            const T v = fabs(A[size_t(i) * n + j]);
            if (v > big) big = v;
        }
        if (big == T(0)) singular = 1;
        vv[i] = T(1) / big;
    }
    __syncthreads();
    if (singular) {
        if (t == 0) *status = CFX_ERR_FATAL;
        return;
    }
    const T small = sizeof(T) == 8 ? T(DBL_EPSILON) : T(FLT_EPSILON);
    for (int j = 0; j < n; ++j) {
        if (t == 0) {
            // rows above the diagonal: row i reads rows k < i of this column
            for (int i = 0; i < j; ++i) {
                T sum = A[size_t(i) * n + j];
                for (int k = 0; k < i; ++k) sum -= A[size_t(i) * n + k] * A[size_t(k) * n + j];
                A[size_t(i) * n + j] = sum;
            }
        }
        __syncthreads();
        for (int i = j + t; i < n; i += LU_NT) {
            T sum = A[size_t(i) * n + j];
            for (int k = 0; k < j; ++k) sum -= A[size_t(i) * n + k] * A[size_t(k) * n + j];
            A[size_t(i) * n + j] = sum;
        }
        __syncthreads();
        if (t == 0) {
            // the last row of largest scaled magnitude (>=, as the reference)
            int iMax = 0;
            T big = T(0);
            for (int i = j; i < n; ++i) {
                const T v = vv[i] * fabs(A[size_t(i) * n + j]);
                if (v >= big) {
                    big = v;
                    iMax = i;
                }
            }
            piv[j] = iMax;
            if (iMax != j) vv[iMax] = vv[j];
            pivRow = iMax;
        }
        __syncthreads();
        const int iMax = pivRow;
        if (iMax != j) {
            for (int k = t; k < n; k += LU_NT) {
                const T a = A[size_t(j) * n + k];
                A[size_t(j) * n + k] = A[size_t(iMax) * n + k];
                A[size_t(iMax) * n + k] = a;
            }
        }
        __syncthreads();
        T d = A[size_t(j) * n + j];
        if (d == T(0)) d = small;
        __syncthreads();
        if (t == 0) A[size_t(j) * n + j] = d;
        if (j != n - 1) {
            const T rDiag = T(1) / d;
            for (int i = j + 1 + t; i < n; i += LU_NT) A[size_t(i) * n + j] *= rDiag;
        }
        __syncthreads();
    }
}

// LUBacksubstitute (scalarMatricesTemplates.C:117-163) in one thread, the
// factors staged in shared memory when they fit (SH).
template <class T, bool SH>
__global__ void lu_solve_k(int n, const T* __restrict__ LUg, const int* __restrict__ piv, const T* __restrict__ b,
                           T* __restrict__ x) {
    extern __shared__ __align__(16) unsigned char lu_smem[];
    T* LUs = reinterpret_cast<T*>(lu_smem);
    T* xs = LUs + size_t(n) * n;
    if (SH) {
        for (size_t i = threadIdx.x; i < size_t(n) * n; i += blockDim.x) LUs[i] = LUg[i];
        for (int i = threadIdx.x; i < n; i += blockDim.x) xs[i] = b[i];
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    const T* LU = SH ? LUs : LUg;
    T* X = SH ? xs : x;
    if (!SH)
        for (int i = 0; i < n; ++i) X[i] = b[i];
    int ii = 0;
    for (int i = 0; i < n; ++i) {
        const int ip = piv[i];
        T sum = X[ip];
        X[ip] = X[i];
        if (ii != 0) {
            for (int j = ii - 1; j < i; ++j) sum -= LU[size_t(i) * n + j] * X[j];
        } else if (sum != T(0)) {
            ii = i + 1;
        }
        X[i] = sum;
    }
    for (int i = n - 1; i >= 0; --i) {
        T sum = X[i];
        for (int j = i + 1; j < n; ++j) sum -= LU[size_t(i) * n + j] * X[j];
        X[i] = sum / LU[size_t(i) * n + i];
    }
    if (SH)
        for (int i = 0; i < n; ++i) x[i] = X[i];
}

template <class T>
__global__ void iface_bprime_k(int n, Iface<T> itf, const T* __restrict__ b, const T* __restrict__ psi,
                               T* __restrict__ bp) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x)
        bp[c] = iface_sub_neg(itf, c, psi, b[c]);
}

template <class T>
__global__ void diag_solve_k(int n, const T* __restrict__ diag, const T* __restrict__ b, T* __restrict__ x) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] = b[i] / diag[i];
}

template <class T>
__global__ void reciprocal_k(int n, T* x) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] = T(1) / x[i];
}

__global__ void cast_d2f_k(int64_t n, const double* __restrict__ in, float* __restrict__ out) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        out[i] = float(in[i]);
}

__global__ void cast_f2d_k(int64_t n, const float* __restrict__ in, double* __restrict__ out) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        out[i] = double(in[i]);
}

// Deterministic reduction: fixed element->thread map for a given n, fixed
// block tree, fixed order over block partials in the last block.
template <class T, int WHICH>
__global__ void __launch_bounds__(RED_NT) reduce_k(int n, const T* __restrict__ a, const T* __restrict__ b,
                                                   double* __restrict__ partials, unsigned* counter,
                                                   double* out) {
    __shared__ double sh[RED_NT / 32];
    double acc = 0.0;
    for (int i = blockIdx.x * RED_NT + threadIdx.x; i < n; i += gridDim.x * RED_NT) {
        const double x = double(a[i]);
        if (WHICH == 0) acc += x;
        else if (WHICH == 1) acc += fabs(x);
        else if (WHICH == 2) acc += x * x;
        else acc += x * double(b[i]);
    }
    acc = block_sum<RED_NT>(acc, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
    if (last_block(counter)) {
        double s = 0.0;
        for (int i = threadIdx.x; i < gridDim.x; i += RED_NT) s += __ldcg(partials + i);
        s = block_sum<RED_NT>(s, sh);
        if (threadIdx.x == 0) *out = s;
    }
}

}  // namespace

template <class T>
void Ops<T>::amul(cudaStream_t s, const LevelMesh& m, const LevelCoeffs<T>& a, const T* x, T* y) {
    amul_k<T><<<grid_all(m.n), RED_NT, 0, s>>>(m.n, m.ownerStart, m.losortStart, m.losortL, m.u, a.diag,
                                               a.lowerPerm, a.upper, sell_of(m, a), x, y, if_bou(m, a));
    count_launch();
}

template <class T>
void Ops<T>::tmul(cudaStream_t s, const LevelMesh& m, const LevelCoeffs<T>& a, const T* x, T* y) {
    // Tmul (lduMatrixATmul.C:95-151): y[u] += upper*x[l]; y[l] += lower*x[u]
    amul_k<T><<<grid_all(m.n), RED_NT, 0, s>>>(m.n, m.ownerStart, m.losortStart, m.losortL, m.u, a.diag,
                                               a.sym ? a.lowerPerm : a.upperPerm, a.sym ? a.upper : a.lower,
                                               a.sym ? sell_of(m, a) : Sell<T>{}, x, y, if_int(m, a));
    count_launch();
}

template <class T>
void Ops<T>::residual(cudaStream_t s, const LevelMesh& m, const LevelCoeffs<T>& a, const T* x, const T* b,
                      T* r) {
    residual_k<T><<<grid_all(m.n), RED_NT, 0, s>>>(m.n, m.ownerStart, m.losortStart, m.losortL, m.u, a.diag,
                                                   a.lowerPerm, a.upper, sell_of(m, a), x, b, r, if_bou(m, a));
    count_launch();
}

template <class T>
void Ops<T>::sumA(cudaStream_t s, const LevelMesh& m, const LevelCoeffs<T>& a, T* out) {
    sumA_k<T><<<grid_for(m.n), RED_NT, 0, s>>>(m.n, m.ownerStart, m.losortStart, a.diag, a.lowerPerm, a.upper,
                                               out, if_bou(m, a));
    count_launch();
}

namespace {
int g_amul_sell = 2;
}
int amul_sell() { return g_amul_sell; }
void set_amul_sell(int on) { g_amul_sell = on; }

template <class T>
void Ops<T>::permute(cudaStream_t s, const LevelMesh& m, LevelCoeffs<T>& a) {
    if (m.nf == 0) return;
    permute_k<T><<<grid_for(m.nf), RED_NT, 0, s>>>(m.nf, m.losort, a.sym ? a.upper : a.lower, a.upper,
                                                   a.lowerPerm, a.sym ? nullptr : a.upperPerm);
    count_launch();
    if (m.sellCol && a.sellCoef) {
        sell_pack_k<T><<<grid_all(m.sellEntries), RED_NT, 0, s>>>(m.sellEntries, m.sellSrc, a.lowerPerm, a.upper,
                                                                  a.sellCoef);
        count_launch();
    }
}

template <class T>
void Ops<T>::coarsen(cudaStream_t s, const LevelMesh& f, const LevelCoeffs<T>& fa, const LevelMesh& c,
                     LevelCoeffs<T>& ca) {
    coarse_diag_k<T><<<grid_for(f.nCoarse), RED_NT, 0, s>>>(f.nCoarse, f.coarseCellStart, f.coarseCellFine,
                                                            f.intFaceStart, f.intFaceFine, fa.diag, fa.upper,
                                                            fa.sym ? nullptr : fa.lower, ca.diag);
    count_launch();
    if (f.nCoarseFaces > 0)
        coarse_faces_k<T><<<grid_for(f.nCoarseFaces), RED_NT, 0, s>>>(
            f.nCoarseFaces, f.coarseFaceStart, f.coarseFaceFine, f.faceFlip, fa.upper, fa.sym ? nullptr : fa.lower,
            ca.upper, ca.sym ? nullptr : ca.lower);
    count_launch();
    Ops<T>::permute(s, c, ca);
}

template <class T>
void Ops<T>::restrict_field(cudaStream_t s, const LevelMesh& f, const T* ff, T* cf) {
    restrict_k<T><<<grid_for(f.nCoarse), RED_NT, 0, s>>>(f.nCoarse, f.coarseCellStart, f.coarseCellFine, ff, cf);
    count_launch();
}

template <class T>
void Ops<T>::prolong_field(cudaStream_t s, const LevelMesh& f, const T* cf, T* ff) {
    prolong_k<T><<<grid_for(f.n), RED_NT, 0, s>>>(f.n, f.restrictAddr, cf, ff);
    count_launch();
}

template <class T>
void Ops<T>::interpolate(cudaStream_t s, const LevelMesh& f, const LevelCoeffs<T>& a, T* psi, T* Apsi,
                         const T* psiC) {
    offdiag_amul_k<T><<<grid_all(f.n), RED_NT, 0, s>>>(f.n, f.ownerStart, f.losortStart, f.losortL, f.u,
                                                       a.lowerPerm, a.upper, psi, Apsi, if_bou(f, a));
    interp_coarse_k<T><<<grid_for(f.nCoarse), RED_NT, 0, s>>>(f.nCoarse, f.coarseCellStart, f.coarseCellFine,
                                                             a.diag, Apsi, psiC, psi);
    count_launch(2);
}

template <class T>
void Ops<T>::lu_factor(cudaStream_t s, const LevelMesh& m, const LevelCoeffs<T>& a, T* A, T* vv, int* piv,
                       int* status) {
    const bool itf = m.nIf > 0 && m.luIfN > 0 && a.ifBou;
    lu_factor_k<T><<<1, LU_NT, 0, s>>>(m.n, m.nf, m.l, m.u, a.diag, a.upper, a.sym ? a.upper : a.lower,
                                       itf ? m.luIfN : 0, m.luIfRow, m.luIfCol, m.luIfSrc, a.ifBou, A, vv, piv,
                                       status);
    count_launch();
}

template <class T>
void Ops<T>::lu_solve(cudaStream_t s, int n, const T* A, const int* piv, const T* b, T* x) {
    const size_t sm = (size_t(n) * n + n) * sizeof(T);
    if (sm <= 48 * 1024)
        lu_solve_k<T, true><<<1, 128, sm, s>>>(n, A, piv, b, x);
    else
        lu_solve_k<T, false><<<1, 32, 0, s>>>(n, A, piv, b, x);
    count_launch();
}

template <class T>
void Ops<T>::iface_restrict(cudaStream_t s, const LevelMesh& m, const T* fine, T* coarse) {
    iface_restrict_k<T><<<grid_all(m.nIf), RED_NT, 0, s>>>(m.nIf, m.ifcStart, m.ifcFine, fine, coarse);
    count_launch();
}

template <class T>
void Ops<T>::iface_bprime(cudaStream_t s, int n, const Iface<T>& itf, const T* b, const T* psi, T* bp) {
    iface_bprime_k<T><<<grid_all(n), RED_NT, 0, s>>>(n, itf, b, psi, bp);
    count_launch();
}

template <class T>
void Ops<T>::diag_solve(cudaStream_t s, int n, const T* diag, const T* b, T* x) {
    diag_solve_k<T><<<grid_for(n), RED_NT, 0, s>>>(n, diag, b, x);
    count_launch();
}

template <class T>
void Ops<T>::reciprocal(cudaStream_t s, int n, T* x) {
    reciprocal_k<T><<<grid_for(n), RED_NT, 0, s>>>(n, x);
    count_launch();
}

void launch_cast_d2f(cudaStream_t s, int64_t n, const double* in, float* out) {
    cast_d2f_k<<<grid_for(n), RED_NT, 0, s>>>(n, in, out);
    count_launch();
}

void launch_cast_f2d(cudaStream_t s, int64_t n, const float* in, double* out) {
    cast_f2d_k<<<grid_for(n), RED_NT, 0, s>>>(n, in, out);
    count_launch();
}

template <class T>
void launch_reduce(cudaStream_t s, Scratch& sc, int which, int n, const T* a, const T* b, double* out) {
    const int g = grid_for(n);
    switch (which) {
        case 0: reduce_k<T, 0><<<g, RED_NT, 0, s>>>(n, a, b, sc.partials, sc.counters, out); break;
        case 1: reduce_k<T, 1><<<g, RED_NT, 0, s>>>(n, a, b, sc.partials, sc.counters, out); break;
        case 2: reduce_k<T, 2><<<g, RED_NT, 0, s>>>(n, a, b, sc.partials, sc.counters, out); break;
        default: reduce_k<T, 3><<<g, RED_NT, 0, s>>>(n, a, b, sc.partials, sc.counters, out); break;
    }
}

template struct Ops<double>;
template struct Ops<float>;
template void launch_reduce<double>(cudaStream_t, Scratch&, int, int, const double*, const double*, double*);
template void launch_reduce<float>(cudaStream_t, Scratch&, int, int, const float*, const float*, double*);

}  // namespace cfx
