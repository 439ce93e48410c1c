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
                                                 const T* __restrict__ upper, const T* __restrict__ x,
                                                 T* __restrict__ y) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        T acc = diag[c] * x[c];
        const int k1 = losortStart[c + 1];
        for (int k = losortStart[c]; k < k1; ++k) acc += lp[k] * x[losortL[k]];
        const int f1 = ownerStart[c + 1];
        for (int f = ownerStart[c]; f < f1; ++f) acc += upper[f] * x[u[f]];
        y[c] = acc;
    }
}

template <class T>
__global__ void __launch_bounds__(RED_NT) residual_k(int n, const int* __restrict__ ownerStart,
                                                     const int* __restrict__ losortStart,
                                                     const int* __restrict__ losortL, const int* __restrict__ u,
                                                     const T* __restrict__ diag, const T* __restrict__ lp,
                                                     const T* __restrict__ upper, const T* __restrict__ x,
                                                     const T* __restrict__ b, T* __restrict__ r) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        T acc = b[c] - diag[c] * x[c];
        const int k1 = losortStart[c + 1];
        for (int k = losortStart[c]; k < k1; ++k) acc -= lp[k] * x[losortL[k]];
        const int f1 = ownerStart[c + 1];
        for (int f = ownerStart[c]; f < f1; ++f) acc -= upper[f] * x[u[f]];
        r[c] = acc;
    }
}

template <class T>
__global__ void __launch_bounds__(RED_NT) sumA_k(int n, const int* __restrict__ ownerStart,
                                                 const int* __restrict__ losortStart, const T* __restrict__ diag,
                                                 const T* __restrict__ lp, const T* __restrict__ upper,
                                                 T* __restrict__ s) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        T acc = diag[c];
        const int k1 = losortStart[c + 1];
        for (int k = losortStart[c]; k < k1; ++k) acc += lp[k];
        const int f1 = ownerStart[c + 1];
        for (int f = ownerStart[c]; f < f1; ++f) acc += upper[f];
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
                                               a.lowerPerm, a.upper, x, y);
    count_launch();
}

template <class T>
void Ops<T>::tmul(cudaStream_t s, const LevelMesh& m, const LevelCoeffs<T>& a, const T* x, T* y) {
    // Tmul (lduMatrixATmul.C:95-151): y[u] += upper*x[l]; y[l] += lower*x[u]
    amul_k<T><<<grid_all(m.n), RED_NT, 0, s>>>(m.n, m.ownerStart, m.losortStart, m.losortL, m.u, a.diag,
                                               a.sym ? a.lowerPerm : a.upperPerm, a.sym ? a.upper : a.lower, x, y);
    count_launch();
}

template <class T>
void Ops<T>::residual(cudaStream_t s, const LevelMesh& m, const LevelCoeffs<T>& a, const T* x, const T* b,
                      T* r) {
    residual_k<T><<<grid_all(m.n), RED_NT, 0, s>>>(m.n, m.ownerStart, m.losortStart, m.losortL, m.u, a.diag,
                                                   a.lowerPerm, a.upper, x, b, r);
    count_launch();
}

template <class T>
void Ops<T>::sumA(cudaStream_t s, const LevelMesh& m, const LevelCoeffs<T>& a, T* out) {
    sumA_k<T><<<grid_for(m.n), RED_NT, 0, s>>>(m.n, m.ownerStart, m.losortStart, a.diag, a.lowerPerm, a.upper,
                                               out);
    count_launch();
}

template <class T>
void Ops<T>::permute(cudaStream_t s, const LevelMesh& m, LevelCoeffs<T>& a) {
    if (m.nf == 0) return;
    permute_k<T><<<grid_for(m.nf), RED_NT, 0, s>>>(m.nf, m.losort, a.sym ? a.upper : a.lower, a.upper,
                                                   a.lowerPerm, a.sym ? nullptr : a.upperPerm);
    count_launch();
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
