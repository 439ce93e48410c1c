// sweeps.cu - level-scheduled triangular sweeps (DIC/DILU preconditioning,
// their reciprocal diagonals, Gauss-Seidel smoothing).
//
// The reference runs these as sequential face loops (DICPreconditioner.C:71-122,
// DILUPreconditioner.C:71-134, GaussSeidelSmoother.C:125-177).  Every cell's
// result depends only on its lower neighbours (forward) or upper neighbours
// (backward), so cells of one level of that dependency DAG are independent.
// Each cell gathers its contributions in the reference's per-cell face order:
//   forward:  losort slots of the cell (faces where it is the neighbour, in
//             face order), the order in which the face loop reaches it;
//   backward: owner faces in decreasing face index (the reverse face loop);
//   GS:       losort slots with new values, then owner faces with old values.
// With --fmad=false the results equal the sequential sweeps bit for bit.
//
// Two execution forms:
//   sweep_small_k  one CTA walks all levels with block barriers (small or
//                  coarse meshes: a block barrier costs ~0.1 us);
//   sweep_multi_k  persistent CTAs take chunks of <= SWEEP_CHUNK cells in
//                  level order from an atomic ticket; a chunk of level L waits
//                  (bounded spin) until every chunk of level L-1 has released
//                  its done-counter.  A CTA only waits on chunks with smaller
//                  tickets, which are held by running CTAs, so the kernel needs
//                  no co-residency guarantee.  A wait that exceeds its deadline
//                  sets the abort flag and an error status; every CTA then
//                  returns.

#include "device.cuh"
#include "internal.h"
#include "solvers.h"

namespace cfx {

namespace {

constexpr uint64_t SWEEP_TIMEOUT_NS = 2000000000ull;  // 2 s per wait
int g_small_threshold = 200000;
int g_num_sms = 152;

struct AddrPtrs {
    const int* __restrict__ ownerStart;
    const int* __restrict__ losortStart;
    const int* __restrict__ losortL;
    const int* __restrict__ u;
};

template <class T, int OP>
__device__ __forceinline__ T sweep_cell(int c, const AddrPtrs& m, const SweepArgs<T>& a) {
    if (OP == SW_DIC_FWD || OP == SW_T_FWD) {
        const T* cf = OP == SW_DIC_FWD ? a.lp : a.up;
        const T rDc = a.rD[c];
        T w = rDc * a.in[c];
        const int k1 = m.losortStart[c + 1];
        for (int k = m.losortStart[c]; k < k1; ++k) w -= (rDc * cf[k]) * ldcg(a.x + m.losortL[k]);
        return w;
    } else if (OP == SW_BWD) {
        const T rDc = a.rD[c];
        T w = ldcg(a.x + c);
        const int f0 = m.ownerStart[c];
        for (int f = m.ownerStart[c + 1] - 1; f >= f0; --f) w -= (rDc * a.upper[f]) * ldcg(a.x + m.u[f]);
        return w;
    } else if (OP == SW_GS) {
        T v = a.in[c];
        const int k1 = m.losortStart[c + 1];
        for (int k = m.losortStart[c]; k < k1; ++k) v -= a.lp[k] * ldcg(a.x + m.losortL[k]);
        const int f1 = m.ownerStart[c + 1];
        for (int f = m.ownerStart[c]; f < f1; ++f) v -= a.upper[f] * ldcg(a.x + m.u[f]);
        return v / a.diag[c];
    } else {  // SW_RD: pivots D (reciprocal taken afterwards)
        T D = a.diag[c];
        const int k1 = m.losortStart[c + 1];
        for (int k = m.losortStart[c]; k < k1; ++k) D -= (a.up[k] * a.lp[k]) / ldcg(a.x + m.losortL[k]);
        return D;
    }
}

template <class T, int OP>
__global__ void __launch_bounds__(SMALL_NT) sweep_small_k(AddrPtrs m, SweepArgs<T> a, const int* __restrict__ cells,
                                                          const int* __restrict__ levelStart, int nLevels) {
    __shared__ double sh[SMALL_NT / 32];
    if (a.done && *a.done) return;
    double dot = 0.0;
    for (int L = 0; L < nLevels; ++L) {
        const int e = levelStart[L + 1];
        for (int i = levelStart[L] + threadIdx.x; i < e; i += SMALL_NT) {
            const int c = cells[i];
            const T v = sweep_cell<T, OP>(c, m, a);
            a.x[c] = v;
            if (a.dotWith) dot += double(v) * double(a.dotWith[c]);
        }
        __syncthreads();
    }
    if (a.dotWith) {
        dot = block_sum<SMALL_NT>(dot, sh);
        if (threadIdx.x == 0) a.chunkPartials[0] = dot;
    }
}

template <class T, int OP>
__global__ void __launch_bounds__(SWEEP_NT) sweep_multi_k(AddrPtrs m, SweepArgs<T> a, Schedule s, int* status) {
    __shared__ int sh_chunk, sh_ok;
    __shared__ double sh[SWEEP_NT / 32];
    int* ticket = s.sync;
    int* abortf = s.sync + 1;
    int* done = s.sync + 2;
    if (a.done && *a.done) return;
    for (;;) {
        if (threadIdx.x == 0) sh_chunk = atomicAdd(ticket, 1);
        __syncthreads();
        const int chunk = sh_chunk;
        if (chunk >= s.nChunks) return;
        const int level = s.chunkLevel[chunk];
        const int i = s.chunkStart[chunk] + threadIdx.x;
        const int c = i < s.chunkStart[chunk + 1] ? s.cells[i] : -1;
        if (threadIdx.x == 0) {
            int ok = 1;
            if (level > 0) {
                const int target = s.levelChunks[level - 1];
                const int* d = done + level - 1;
                uint64_t t0 = 0;
                unsigned spins = 0;
                while (ld_acquire(d) < target) {
                    if (*(volatile int*)abortf) {
                        ok = 0;
                        break;
                    }
                    __nanosleep(32);
                    if ((++spins & 255u) == 0) {
                        const uint64_t t = globaltimer_ns();
                        if (t0 == 0) {
                            t0 = t;
                        } else if (t - t0 > SWEEP_TIMEOUT_NS) {
                            atomicExch(abortf, 1);
                            atomicExch(status, int(CFX_ERR_TIMEOUT));
                            ok = 0;
                            break;
                        }
                    }
                }
            } else if (*(volatile int*)abortf) {
                ok = 0;
            }
            sh_ok = ok;
        }
        __syncthreads();
        if (!sh_ok) return;
        T v = T(0);
        if (c >= 0) {
            v = sweep_cell<T, OP>(c, m, a);
            a.x[c] = v;
        }
        if (a.dotWith) {
            double p = c >= 0 ? double(v) * double(a.dotWith[c]) : 0.0;
            p = block_sum<SWEEP_NT>(p, sh);
            if (threadIdx.x == 0) a.chunkPartials[chunk] = p;
        }
        __syncthreads();
        if (threadIdx.x == 0) red_release_add(done + level, 1);
    }
}

template <class T, int OP>
cfx_status launch_op(cudaStream_t st, const LevelMesh& m, const Schedule& s, const SweepArgs<T>& a, int* status,
                     bool small) {
    AddrPtrs p{m.ownerStart, m.losortStart, m.losortL, m.u};
    if (s.nCells == 0) return CFX_OK;
    if (small) {
        sweep_small_k<T, OP><<<1, SMALL_NT, 0, st>>>(p, a, s.cells, s.levelStart, s.nLevels);
        count_launch();
    } else {
        // More CTAs than fit at once are harmless (tickets are taken only by
        // running CTAs); 8 x 256 threads fill an SM at <= 32 registers.
        const int grid = g_num_sms * 8;
        CFX_CUDA(cudaMemsetAsync(s.sync, 0, sizeof(int) * (2 + s.nLevels), st));
        const int g = s.nChunks < grid ? s.nChunks : grid;
        sweep_multi_k<T, OP><<<g, SWEEP_NT, 0, st>>>(p, a, s, status);
        count_launch();
    }
    return CFX_OK;
}

}  // namespace

int small_sweep_threshold() { return g_small_threshold; }
void set_num_sms(int n) { g_num_sms = n > 0 ? n : 152; }

int sweep_partials(const LevelMesh& m, const Schedule& s, bool forceSmall) {
    return (forceSmall || m.n <= g_small_threshold) ? 1 : s.nChunks;
}
void set_small_sweep_threshold(int n) { g_small_threshold = n; }

template <class T>
cfx_status run_sweep(cudaStream_t st, const LevelMesh& m, const Schedule& s, int op, const SweepArgs<T>& a,
                     int* status, bool forceSmall) {
    const bool small = forceSmall || m.n <= g_small_threshold;
    switch (op) {
        case SW_DIC_FWD: return launch_op<T, SW_DIC_FWD>(st, m, s, a, status, small);
        case SW_BWD: return launch_op<T, SW_BWD>(st, m, s, a, status, small);
        case SW_GS: return launch_op<T, SW_GS>(st, m, s, a, status, small);
        case SW_RD: return launch_op<T, SW_RD>(st, m, s, a, status, small);
        case SW_T_FWD: return launch_op<T, SW_T_FWD>(st, m, s, a, status, small);
        default: set_error("unknown sweep"); return CFX_ERR_ARG;
    }
}

template cfx_status run_sweep<double>(cudaStream_t, const LevelMesh&, const Schedule&, int, const SweepArgs<double>&,
                                      int*, bool);
template cfx_status run_sweep<float>(cudaStream_t, const LevelMesh&, const Schedule&, int, const SweepArgs<float>&,
                                     int*, bool);

}  // namespace cfx
