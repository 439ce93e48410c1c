// device.cuh - device helpers shared by the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cfloat>

#include "internal.h"

namespace cfx {

constexpr double VSMALL = DBL_MIN;  // doubleScalarVSmall
constexpr double SP_SMALL = 1e-20;  // SolverPerformance::small_
constexpr double SP_GREAT = 1e20;   // SolverPerformance::great_

// One row of A x in the reference's per-cell face order (Amul,
// lduMatrixATmul.C:34-92, seen from cell c): diag, then the lower
// coefficients of the faces where c is the neighbour (losort order), then
// the upper coefficients of the faces c owns.
template <class T>
__device__ __forceinline__ T row_amul(int c, const int* __restrict__ os, const int* __restrict__ ls,
                                      const int* __restrict__ lL, const int* __restrict__ u,
                                      const T* __restrict__ diag, const T* __restrict__ lp,
                                      const T* __restrict__ upper, const T* __restrict__ x) {
    T acc = diag[c] * x[c];
    const int k1 = ls[c + 1];
    for (int k = ls[c]; k < k1; ++k) acc += lp[k] * x[lL[k]];
    const int f1 = os[c + 1];
    for (int f = os[c]; f < f1; ++f) acc += upper[f] * x[u[f]];
    return acc;
}


// lduMatrix::updateMatrixInterfaces with cyclic fields
// (cyclicFvPatchField.C:150-174): acc -= coeffs*psi[nbr], face by face.
template <class T>
__device__ __forceinline__ T iface_sub(const Iface<T>& f, int c, const T* __restrict__ x, T acc) {
    if (f.start) {
        const int j1 = f.start[c + 1];
        for (int j = f.start[c]; j < j1; ++j) acc -= f.coef[j] * x[f.nbr[j]];
    }
    return acc;
}

// The same with the negated coefficients (lduMatrix::residual's and the
// Gauss-Seidel smoothers' mBouCoeffs).
template <class T>
__device__ __forceinline__ T iface_sub_neg(const Iface<T>& f, int c, const T* __restrict__ x, T acc) {
    if (f.start) {
        const int j1 = f.start[c + 1];
        for (int j = f.start[c]; j < j1; ++j) acc -= (-f.coef[j]) * x[f.nbr[j]];
    }
    return acc;
}

// Fixed-order warp tree (xor-free shuffle down): the same inputs always give
// the same sum, whatever the launch.
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Block tree sum; the result is valid in thread 0.  NT is the block size.
template <int NT>
__device__ __forceinline__ double block_sum(double v, double* sh /* NT/32 */) {
    v = warp_sum(v);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        r = lane < NT / 32 ? sh[lane] : 0.0;
        r = warp_sum(r);
    }
    __syncthreads();
    return r;
}

// True in every thread of the block that arrives last at `counter`; the
// counter is reset by that block.  Writes made before the call by any block
// are visible to the last block.
__device__ __forceinline__ bool last_block(unsigned* counter) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned t = atomicAdd(counter, 1u);
        last = (t == gridDim.x - 1);
        if (last) *counter = 0u;
    }
    __syncthreads();
    if (last) __threadfence();
    return last;
}

__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(int* p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ void red_release_add(int* p, int v) {
    asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// L2-coherent loads of values written by other CTAs during this launch.
template <class T>
__device__ __forceinline__ T ldcg(const T* p) {
    return __ldcg(p);
}

}  // namespace cfx
