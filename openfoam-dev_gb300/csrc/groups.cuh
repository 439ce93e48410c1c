// groups.cuh - thread groups that run one whole solve: a CTA, or all CTAs
// of a thread-block cluster.
//
//   CtaGroup      one CTA of BLK_NT threads; __syncthreads barriers.
//   ClusterGroup  all CTAs of a thread-block cluster; hardware cluster
//                 barriers (release/acquire at cluster scope, which makes the
//                 vectors written in global memory by one CTA visible to the
//                 others); sums add the CTAs' partials, read from each CTA's
//                 shared memory in rank order, so every CTA gets the same
//                 bits and takes the same branch.
// Both give rank() / size() for striding over cells, sync(), leader() and a
// fixed-order sum() whose result every thread receives.
#pragma once

#include <cooperative_groups.h>

#include "device.cuh"

namespace cfx {

namespace cg = cooperative_groups;

constexpr int BLK_NT = 256;

struct CtaGroup {
    double* sh;  // [BLK_NT/32 + 1] shared
    __device__ int rank() const { return threadIdx.x; }
    __device__ int size() const { return BLK_NT; }
    __device__ void sync() const { __syncthreads(); }
    __device__ bool leader() const { return threadIdx.x == 0; }
    __device__ double sum(double v) {
        v = block_sum<BLK_NT>(v, sh);
        if (threadIdx.x == 0) sh[BLK_NT / 32] = v;
        __syncthreads();
        v = sh[BLK_NT / 32];
        __syncthreads();
        return v;
    }
};

struct ClusterGroup {
    double* sh;    // [BLK_NT/32 + 1] shared
    double* slot;  // [2] shared, read by the other CTAs of the cluster
    int parity;    // alternates the slot: a slot is rewritten only after the
                   // next sum's barrier, when every CTA has read it
    int crank, nranks;
    __device__ int rank() const { return crank * BLK_NT + threadIdx.x; }
    __device__ int size() const { return nranks * BLK_NT; }
    __device__ void sync() const { cg::this_cluster().sync(); }
    __device__ bool leader() const { return crank == 0 && threadIdx.x == 0; }
    __device__ double sum(double v) {
        v = block_sum<BLK_NT>(v, sh);
        if (threadIdx.x == 0) slot[parity] = v;
        sync();
        if (threadIdx.x == 0) {
            cg::cluster_group cl = cg::this_cluster();
            double s = 0.0;
            for (int r = 0; r < nranks; ++r) s += *cl.map_shared_rank(slot + parity, r);
            sh[BLK_NT / 32] = s;
        }
        parity ^= 1;
        __syncthreads();
        v = sh[BLK_NT / 32];
        __syncthreads();
        return v;
    }
};

}  // namespace cfx
