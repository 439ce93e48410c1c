// device.cuh - device helpers shared by the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace cfx {

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
