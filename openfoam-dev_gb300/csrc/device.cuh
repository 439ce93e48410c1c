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


// The rows of A in sliced ELL form: slices of 32 rows (one warp), each
// row's entries in the order above (lower terms in losort order, then upper
// terms in face order), stored in pairs so that a lane reads two entries of
// its row with one 128-bit (FP64) coefficient load, and a warp reads 512
// contiguous bytes: entry k of row c (lane j of slice s) sits at
// start[s] + 64*(k/2) + 2*j + (k%2); a slice's width K is even.
//
// Two kinds of slice.  Explicit: cnt[c] entries, columns in col.  Pattern
// (pat[s] >= 0): the slice's rows draw their neighbours from one ascending
// list of at most 8 offsets, offs[8*pat[s] + k] (cell-index differences);
// cnt[c] is then a mask of the offsets row c has, entry k holds the
// coefficient of neighbour c + offs[k], and no column is read.  A row's
// terms come in ascending column order either way (lower neighbours before
// upper ones, each in face order), so both kinds keep the reference's order.
// col == nullptr: not built (rows with more than 255 entries); the kernels
// then gather through losort/ownerStart.
template <class T>
struct Sell {
    const int* start = nullptr;          // [slices + 1] first entry of each slice
    const unsigned char* cnt = nullptr;  // [n] entries of each row, or its offset mask
    const int* col = nullptr;
    const T* coef = nullptr;
    const int* pat = nullptr;   // [slices] offset list of each slice, -1 explicit (null: all explicit)
    const int* offs = nullptr;  // [8 x lists]
};

template <class T>
inline Sell<T> sell_of(const LevelMesh& m, const LevelCoeffs<T>& a) {
    Sell<T> S;
    const int form = amul_sell();
    if (m.sellCol && a.sellCoef && form) {
        S.start = m.sellStart;
        S.cnt = m.sellCnt;
        S.col = m.sellCol;
        S.coef = a.sellCoef;
        S.pat = m.sellPat;
        S.offs = m.sellOffs;
    }
    return S;
}

template <class T>
struct Pair2;
template <>
struct Pair2<double> {
    using type = double2;
};
template <>
struct Pair2<float> {
    using type = float2;
};

template <int OP, class T>
__device__ __forceinline__ T sell_acc(T acc, T a, T x) {
    return OP == 0 ? acc + a * x : acc - a * x;
}

// acc op= the row's terms in order: OP 0 adds coef*x[col], OP 1 subtracts.
// One 16-byte (FP64) or 8-byte (FP32) coefficient load per pair of entries;
// a pattern slice computes each column from the slice's offset list (an L1
// broadcast) instead of loading it.  In FP64 the row's products and sums
// (the reference's rounding, no contraction) keep the FP64 pipe busy rather
// than HBM; in FP32 the pattern slices move the fewest bytes.
template <class T, int OP>
__device__ __forceinline__ T sell_row(int c, const Sell<T>& S, const T* __restrict__ x, T acc) {
    using P2 = typename Pair2<T>::type;
    const int sl = c >> 5;
    const int s0 = __ldg(S.start + sl);
    const int e0 = s0 + 2 * (c & 31);
    const int k1 = __ldg(S.cnt + c);
    const int p = S.pat ? __ldg(S.pat + sl) : -1;
    if (p >= 0) {
        const int K = (__ldg(S.start + sl + 1) - s0) >> 5;
        const int* __restrict__ off = S.offs + 8 * p;
        for (int k = 0; k < K; k += 2) {
            const P2 cf = __ldg(reinterpret_cast<const P2*>(S.coef + e0 + 32 * k));
            if ((k1 >> k) & 1) acc = sell_acc<OP>(acc, cf.x, x[c + __ldg(off + k)]);
            if ((k1 >> (k + 1)) & 1) acc = sell_acc<OP>(acc, cf.y, x[c + __ldg(off + k + 1)]);
        }
        return acc;
    }
    for (int k = 0; k < k1; k += 2) {
        const int e = e0 + 32 * k;
        const P2 cf = __ldg(reinterpret_cast<const P2*>(S.coef + e));
        const int2 cl = __ldg(reinterpret_cast<const int2*>(S.col + e));
        acc = sell_acc<OP>(acc, cf.x, x[cl.x]);
        if (k + 1 < k1) acc = sell_acc<OP>(acc, cf.y, x[cl.y]);
    }
    return acc;
}

// One row of A x from whichever form the level has.
template <class T>
__device__ __forceinline__ T row_ax(int c, const int* __restrict__ os, const int* __restrict__ ls,
                                    const int* __restrict__ lL, const int* __restrict__ u,
                                    const T* __restrict__ diag, const T* __restrict__ lp,
                                    const T* __restrict__ upper, const Sell<T>& S, const T* __restrict__ x) {
    if (S.col) return sell_row<T, 0>(c, S, x, diag[c] * x[c]);
    return row_amul<T>(c, os, ls, lL, u, diag, lp, upper, x);
}

// lduMatrix::residual's order for one row (lduMatrixATmul.C:203-280):
// b - diag*x, then minus each neighbour product.
template <class T>
__device__ __forceinline__ T row_res(int c, const int* __restrict__ os, const int* __restrict__ ls,
                                     const int* __restrict__ lL, const int* __restrict__ u,
                                     const T* __restrict__ diag, const T* __restrict__ lp,
                                     const T* __restrict__ upper, const Sell<T>& S, const T* __restrict__ x,
                                     const T* __restrict__ b) {
    T acc = b[c] - diag[c] * x[c];
    if (S.col) return sell_row<T, 1>(c, S, x, acc);
    for (int k = ls[c]; k < ls[c + 1]; ++k) acc -= lp[k] * x[lL[k]];
    for (int f = os[c]; f < os[c + 1]; ++f) acc -= upper[f] * x[u[f]];
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
