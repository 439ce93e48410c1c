// sweeps.cu - level-scheduled triangular sweeps on packed schedules: DIC/DILU
// forward and backward preconditioning, their reciprocal diagonals, and
// Gauss-Seidel smoothing (several sweeps fused into one pass).
//
// The reference runs these as sequential face loops (DICPreconditioner.C:71-122,
// DILUPreconditioner.C:71-134, GaussSeidelSmoother.C:125-177).  Every cell's
// result depends only on its lower neighbours (forward) or upper neighbours
// (backward), so all cells of one level of that dependency DAG are
// independent.  Each slot gathers its contributions in the reference's
// per-cell face order:
//   forward:  losort slots of the cell (faces where it is the neighbour, in
//             face order), coefficient rD_c*lower;
//   backward: owner faces in decreasing face index, coefficient rD_c*upper;
//   GS:       losort slots with this sweep's values, then owner faces with the
//             previous sweep's values, divided by the diagonal.
// Products such as rD_c*lower are rounded exactly as the reference rounds
// them, and the library is built with --fmad=false, so every result equals
// the sequential sweep bit for bit.
//
// Several Gauss-Seidel sweeps run as one pass over the combined DAG: cell c in
// sweep s waits for its lower neighbours in sweep s and its upper neighbours
// in sweep s-1, so S sweeps take D + 2(S-1) levels instead of S*D.
//
// Execution forms:
//   sweep_cta_k   one CTA of 1024 threads walks the levels with block
//                 barriers; the vector lives in shared memory when it fits.
//                 Used for coarse levels and small meshes.
//   sweep_cluster_k  a cluster of up to 16 CTAs (one GPC) holds the vector in
//                 distributed shared memory (cell c in CTA c / per) and
//                 separates levels with the hardware cluster barrier; each
//                 warp prefetches its next group's packed data into registers
//                 before the barrier.  Used up to ~16x the single-CTA size.
//   sweep_grid_k  persistent CTAs, chunk J (8 groups of 32 slots, level
//                 order) on CTA J mod grid; each CTA loads its next chunk's
//                 packed data, then waits (bounded spin, acquire) for every
//                 chunk of the previous level to release its done-counter.
//                 Launched cooperatively so all CTAs are resident.  A wait
//                 that exceeds its deadline sets the abort flag and an error
//                 status; every CTA then returns.
//   sweep_tile_k  persistent CTAs on a tiled schedule (build_sched_tiled):
//                 each tile (a band of levels x a range of cells) runs on
//                 one CTA level by level with block barriers, the values it
//                 produces held in shared memory; values of other tiles are
//                 read from global memory after waiting for the producing
//                 tile's published progress (cached per CTA, so a wait that
//                 is already satisfied costs nothing).  Most dependencies
//                 stay inside a CTA, and the cross-CTA ones are pipelined
//                 instead of paid at every level.  Launched cooperatively;
//                 waits bounded like the grid form's.

#include <cooperative_groups.h>

#include <algorithm>

#include "device.cuh"
#include "internal.h"
#include "solvers.h"

namespace cfx {

namespace {

constexpr uint64_t SWEEP_TIMEOUT_NS = 2000000000ull;  // 2 s per wait
constexpr int GRID_NT = 256;                            // 8 warps = one chunk
constexpr int CTA_NT = 256;
constexpr int CL_NT = 256;                              // threads per cluster CTA
constexpr int TILE_NT = 512;                            // threads per tile CTA
constexpr int PF_SMALL = 8, PF_LARGE = 16, PF_GRID_XL = 32;  // entries held in registers per slot
namespace cg = cooperative_groups;

int g_num_sms = 152;
int g_cluster = 0;          // CTAs per cluster of sweep_cluster_k (0: not used)
int g_cluster_pre = 0;      // the same for the DIC/DILU (forward/backward) schedules when g_cluster is 0
int g_cluster_avail = 0;    // largest cluster the GPU can hold (16 or 8; 0: none)
int g_small_threshold = 0;  // <= this many cells: single-CTA even without smem fit
int g_cluster_global = 0;   // <= this many cells: one cluster with the vector in global memory
int g_grid[2][8][3];        // resident CTAs of sweep_grid_k per (precision, op, PF 8/16/32)
int g_wave_grid[2][8][3];   // resident CTAs of sweep_wave_k, the same
int g_wave = 0;             // grid form: wavefront (1) or whole-level counters (0, default)
size_t g_smem_cap = 200 * 1024;
size_t g_smem_cap_max = 200 * 1024;
int g_tile = 0;             // build large schedules tiled (the tile form)
int g_tile_pub = 2;         // tile form: progress published every this many levels
int g_tile_ctas = 152;      // tile CTAs that can be resident at once

template <class T>
struct SweepCtx {
    const T* coef;
    const T* scalar;
    const T* in;     // right-hand side by cell (r or b)
    const T* inS;    // the same gathered into slot order
    T* x;
    const T* dotWith;
    double* partials;
    const int* done;
    unsigned long long timeoutNs;  // bound of every wait of the grid forms
};

template <int OP, class T>
__device__ __forceinline__ T sw_init(T sc, T in, T xc) {
    if (OP == OP_FWD) return sc * in;
    if (OP == OP_BWD) return xc;
    if (OP == OP_GS) return in;
    return sc;  // OP_RD: pivot starts at the diagonal
}

template <int OP, class T>
__device__ __forceinline__ T sw_step(T acc, T cf, T xn) {
    if (OP == OP_RD) return acc - cf / xn;
    return acc - cf * xn;
}

template <int OP, class T>
__device__ __forceinline__ T sw_fini(T acc, T sc) {
    if (OP == OP_GS) return acc / sc;
    return acc;
}

// Entries k >= k0 of one slot, loaded in batches of 8 independent loads so
// the latency is paid once per batch, then applied in order.
template <class T, int OP, class XF>
__device__ __forceinline__ T tail_entries(const DevSched& s, const T* coef, int e0, int k0, int n, T acc, XF xat) {
    for (int kb = k0; kb < n; kb += 8) {
        int nb[8];
        T cf[8];
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (kb + j < n) {
                nb[j] = s.nb[e0 + 32 * (kb + j)];
                cf[j] = coef[e0 + 32 * (kb + j)];
            }
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (kb + j < n) acc = sw_step<OP>(acc, cf[j], xat(nb[j]));
    }
    return acc;
}

template <class T, int OP, int PF>
__global__ void __launch_bounds__(GRID_NT) sweep_grid_k(DevSched s, SweepCtx<T> a, int* status) {
    __shared__ double sh[GRID_NT / 32];
    __shared__ int sh_ok;
    if (a.done && *a.done) return;
    int* abortf = s.sync;
    int* done = s.sync + 2;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int J = blockIdx.x; J < s.nChunks; J += gridDim.x) {
        const int L = s.chunkLevel[J];
        const int g = s.chunkGroup[J] + w;
        int c = -1, n = 0, e0 = 0;
        T sc = T(0), in = T(0);
        int nbr[PF];
        T cf[PF];
        if (g < s.chunkGroup[J + 1]) {
            const int slot = g * 32 + lane;
            c = s.cell[slot];
            if (c >= 0) {
                n = s.cnt[slot];
                e0 = s.groupEntry[g] + lane;
                sc = a.scalar[slot];
                if (OP == OP_FWD || OP == OP_GS) in = a.inS[slot];
#pragma unroll
                for (int k = 0; k < PF; ++k)
                    if (k < n) {
                        nbr[k] = s.nb[e0 + 32 * k];
                        cf[k] = a.coef[e0 + 32 * k];
                    }
            }
        }
        if (threadIdx.x == 0) {
            int ok = 1;
            if (L > 0) {
                const int target = s.levelChunks[L - 1];
                const int* d = done + L - 1;
                uint64_t t0 = 0;
                unsigned spins = 0;
                // relaxed poll, then a fence: the acquire pattern
                while (*(volatile const int*)d < target) {
                    if (*(volatile int*)abortf) {
                        ok = 0;
                        break;
                    }
                    if ((++spins & 63u) == 0) {
                        const uint64_t t = globaltimer_ns();
                        if (t0 == 0) {
                            t0 = t;
                        } else if (t - t0 > a.timeoutNs) {
                            atomicExch(abortf, 1);
                            atomicExch(status, int(CFX_ERR_TIMEOUT));
                            ok = 0;
                            break;
                        }
                    }
                }
                __threadfence();
            } else if (*(volatile int*)abortf) {
                ok = 0;
            }
            sh_ok = ok;
        }
        __syncthreads();
        if (!sh_ok) return;
        T v = T(0);
        if (c >= 0) {
            T acc = sw_init<OP>(sc, in, OP == OP_BWD ? ldcg(a.x + c) : T(0));
#pragma unroll
            for (int k = 0; k < PF; ++k)
                if (k < n) acc = sw_step<OP>(acc, cf[k], ldcg(a.x + nbr[k]));
            acc = tail_entries<T, OP>(s, a.coef, e0, PF, n, acc, [&](int cc) { return ldcg(a.x + cc); });
            v = sw_fini<OP>(acc, sc);
            a.x[c] = v;
        }
        if (a.dotWith) {
            double p = c >= 0 ? double(v) * double(a.dotWith[c]) : 0.0;
            p = block_sum<GRID_NT>(p, sh);
            if (threadIdx.x == 0) a.partials[J] = p;
        }
        __syncthreads();
        if (threadIdx.x == 0) red_release_add(done + L, 1);
    }
}

// Element c of the vector distributed over the cluster (c in CTA c / per).
template <class T>
__device__ __forceinline__ T* cl_ref(cg::cluster_group& cl, T* Xl, int per, int c) {
    const int o = c / per;
    return cl.map_shared_rank(Xl, o) + (c - o * per);
}

// Wavefront form (persistent, cooperative): warp-sized chunks.  Warp W of the
// grid takes groups W, W + NW, ... in order; before computing a group it
// waits only for the groups its slots read (the dependency lists built with
// the schedule: lower neighbours in the same sweep, and for Gauss-Seidel the
// upper neighbours and the cell itself in the previous sweep), each lane
// polling one of them with an acquire load, then publishes its own flag with
// a release store.  No block barrier, no whole-level counter: a group starts
// as soon as its own inputs exist.  Groups only depend on groups of earlier
// levels, which come earlier in every warp's order, and all warps are
// resident (cooperative launch), so the waits always end; every wait is
// bounded by SWEEP_TIMEOUT_NS on %globaltimer (abort flag + CFX_ERR_TIMEOUT,
// then every warp returns).  The dot partial (when requested) is summed per
// warp in its fixed group order, then per CTA: nPartials = gridDim.x.
template <class T, int OP, int PF>
__global__ void __launch_bounds__(GRID_NT) sweep_wave_k(DevSched s, SweepCtx<T> a, int* status) {
    __shared__ double sh[GRID_NT / 32];
    if (a.done && *a.done) return;
    int* abortf = s.sync;
    const int lane = threadIdx.x & 31;
    const int W = blockIdx.x * (GRID_NT / 32) + (threadIdx.x >> 5);
    const int NW = gridDim.x * (GRID_NT / 32);
    double dot = 0.0;
    bool ok = true;
    for (int g = W; g < s.nGroups && ok; g += NW) {
        const int slot = g * 32 + lane;
        const int c = s.cell[slot];
        const int n = s.cnt[slot];
        const int e0 = s.groupEntry[g] + lane;
        T sc = T(0), in = T(0);
        int nbr[PF];
        T cf[PF];
        if (c >= 0) {
            sc = a.scalar[slot];
            if (OP == OP_FWD || OP == OP_GS) in = a.inS[slot];
        }
#pragma unroll
        for (int k = 0; k < PF; ++k)
            if (k < n) {
                nbr[k] = s.nb[e0 + 32 * k];
                cf[k] = a.coef[e0 + 32 * k];
            }
        // wait for the groups this one reads, each lane polling one of them
        bool mine = true;
        const int d1 = s.depStart[g + 1];
        for (int k = s.depStart[g] + lane; k < d1 && mine; k += 32) {
            const int* f = s.gdone + s.dep[k];
            uint64_t t0 = 0;
            unsigned spins = 0;
            while (ld_acquire(f) == 0) {
                if ((++spins & 63u) == 0) {
                    if (*(volatile int*)abortf) {
                        mine = false;
                        break;
                    }
                    const uint64_t t = globaltimer_ns();
                    if (t0 == 0) {
                        t0 = t;
                    } else if (t - t0 > a.timeoutNs) {
                        atomicExch(abortf, 1);
                        atomicExch(status, int(CFX_ERR_TIMEOUT));
                        mine = false;
                        break;
                    }
                }
            }
        }
        ok = __all_sync(0xffffffffu, mine);
        if (!ok) break;
        T v = T(0);
        if (c >= 0) {
            T acc = sw_init<OP>(sc, in, OP == OP_BWD ? ldcg(a.x + c) : T(0));
#pragma unroll
            for (int k = 0; k < PF; ++k)
                if (k < n) acc = sw_step<OP>(acc, cf[k], ldcg(a.x + nbr[k]));
            acc = tail_entries<T, OP>(s, a.coef, e0, PF, n, acc, [&](int cc) { return ldcg(a.x + cc); });
            v = sw_fini<OP>(acc, sc);
            a.x[c] = v;
            if (a.dotWith) dot += double(v) * double(a.dotWith[c]);
        }
        __syncwarp();
        if (lane == 0) st_release(s.gdone + g, 1);
    }
    if (a.dotWith) {
        dot = block_sum<GRID_NT>(dot, sh);
        if (threadIdx.x == 0) a.partials[blockIdx.x] = dot;
    }
}

// Packed data of one group slot held in registers: the header (cell, entry
// count, entry offset, scalar, right-hand side) and the first PF entries.
template <class T, int PF>
struct SlotRegs {
    int c, n, e0;
    T sc, in;
    int nbr[PF];
    T cf[PF];
};

// Header of slot (g, lane): independent loads, and no branch on their
// values, so issuing them never waits for memory.
template <class T, int OP, int PF>
__device__ __forceinline__ void load_header(const DevSched& s, const SweepCtx<T>& a, int g, bool ok, int lane,
                                            SlotRegs<T, PF>& r) {
    r.c = -1;
    r.n = 0;
    if (ok) {
        const int slot = g * 32 + lane;
        r.c = s.cell[slot];
        r.n = s.cnt[slot];  // 0 for padding slots
        r.e0 = s.groupEntry[g] + lane;
        r.sc = a.scalar[slot];
        r.in = (OP == OP_FWD || OP == OP_GS) ? a.inS[slot] : T(0);
    }
}

// The first PF entries of a slot whose header was issued a level earlier.
template <class T, int PF>
__device__ __forceinline__ void load_entries(const DevSched& s, const T* coef, SlotRegs<T, PF>& r) {
#pragma unroll
    for (int k = 0; k < PF; ++k)
        if (k < r.n) {
            r.nbr[k] = s.nb[r.e0 + 32 * k];
            r.cf[k] = coef[r.e0 + 32 * k];
        }
}

// Level bounds (levelSlot) of the first LS_CACHE levels are copied to shared
// memory at kernel start, so level loops read no global memory for them.
constexpr int LS_CACHE = 4096;

// Pipeline of the single-CTA and cluster forms.  While level L is computed
// from register set X (header and entries in place), the entries of level
// L+1 are issued into set Y (its header arrived during level L-1) and the
// header of level L+2 into X: no load in the level loop waits for memory
// except the neighbour values of the level being computed.  A warp's further
// groups in a wide level are loaded directly.

// One CTA; X = shared-memory copy of the vector when XS, else global.
template <class T, int OP, bool XS, int PF>
__global__ void __launch_bounds__(CTA_NT) sweep_cta_k(DevSched s, SweepCtx<T> a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double sh[CTA_NT / 32];
    __shared__ int lsl[LS_CACHE + 1];
    if (a.done && *a.done) return;
    T* X = XS ? reinterpret_cast<T*>(smem_raw) : a.x;
    const int n = s.n;
    const int nL = s.nLevels;
    const int nc = nL + 1 < LS_CACHE + 1 ? nL + 1 : LS_CACHE + 1;
    for (int i = threadIdx.x; i < nc; i += CTA_NT) lsl[i] = s.levelSlot[i];
    if (XS && (OP == OP_BWD || OP == OP_GS)) {
        for (int i = threadIdx.x; i < n; i += CTA_NT) X[i] = a.x[i];
    }
    __syncthreads();
    constexpr int WARPS = CTA_NT / 32;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    auto lslot = [&](int L) -> int { return L < nc ? lsl[L] : s.levelSlot[L]; };
    auto xat = [&](int c) -> T { return XS ? X[c] : ldcg(a.x + c); };
    auto header = [&](int L, SlotRegs<T, PF>& r) {
        int g = 0;
        bool ok = false;
        if (L < nL) {
            g = (lslot(L) >> 5) + w;
            ok = g < (lslot(L + 1) >> 5);
        }
        load_header<T, OP, PF>(s, a, g, ok, lane, r);
    };
    double dot = 0.0;
    auto level = [&](int L, SlotRegs<T, PF>& cur, SlotRegs<T, PF>& nxt) {
        const int g0 = lslot(L) >> 5, g1 = lslot(L + 1) >> 5;
        if (cur.c >= 0) {
            T acc = sw_init<OP>(cur.sc, cur.in, OP == OP_BWD ? xat(cur.c) : T(0));
#pragma unroll
            for (int k = 0; k < PF; ++k)
                if (k < cur.n) acc = sw_step<OP>(acc, cur.cf[k], xat(cur.nbr[k]));
            acc = tail_entries<T, OP>(s, a.coef, cur.e0, PF, cur.n, acc, xat);
            const T v = sw_fini<OP>(acc, cur.sc);
            X[cur.c] = v;
            if (a.dotWith) dot += double(v) * double(a.dotWith[cur.c]);
        }
        for (int g = g0 + w + WARPS; g < g1; g += WARPS) {
            const int slot = g * 32 + lane;
            const int c = s.cell[slot];
            if (c < 0) continue;
            const int cnt = s.cnt[slot];
            const int e0 = s.groupEntry[g] + lane;
            const T sc = a.scalar[slot];
            const T in = (OP == OP_FWD || OP == OP_GS) ? a.inS[slot] : T(0);
            T acc = sw_init<OP>(sc, in, OP == OP_BWD ? xat(c) : T(0));
            acc = tail_entries<T, OP>(s, a.coef, e0, 0, cnt, acc, xat);
            const T v = sw_fini<OP>(acc, sc);
            X[c] = v;
            if (a.dotWith) dot += double(v) * double(a.dotWith[c]);
        }
        load_entries<T, PF>(s, a.coef, nxt);
        header(L + 2, cur);
        __syncthreads();
    };
    SlotRegs<T, PF> A, B;
    header(0, A);
    header(1, B);
    load_entries<T, PF>(s, a.coef, A);
    for (int L = 0; L < nL; L += 2) {
        level(L, A, B);
        if (L + 1 < nL) level(L + 1, B, A);
    }
    if (XS)
        for (int i = threadIdx.x; i < n; i += CTA_NT) a.x[i] = X[i];
    if (a.dotWith) {
        dot = block_sum<CTA_NT>(dot, sh);
        if (threadIdx.x == 0) a.partials[0] = dot;
    }
}

// DS: vector in distributed shared memory; otherwise in global memory (L2),
// read with L2-coherent loads, and only the barrier is the cluster's.  The
// groups of a level go round the CTAs: CTA r takes g0 + r + CS*j, its warp w
// the j = w, w + WARPS, ...  Between levels the barrier is split: arrive
// (release: this level's writes), issue the pipeline's loads, wait (acquire).
template <class T, int OP, bool DS, int PF>
__global__ void __launch_bounds__(CL_NT) sweep_cluster_k(DevSched s, SweepCtx<T> a, int per) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double sh[CL_NT / 32];
    __shared__ int lsl[LS_CACHE + 1];
    if (a.done && *a.done) return;
    cg::cluster_group cl = cg::this_cluster();
    const int CS = int(cl.num_blocks());
    const int rank = int(cl.block_rank());
    T* Xl = reinterpret_cast<T*>(smem_raw);
    const int n = s.n;
    const int nL = s.nLevels;
    const int nc = nL + 1 < LS_CACHE + 1 ? nL + 1 : LS_CACHE + 1;
    for (int i = threadIdx.x; i < nc; i += CL_NT) lsl[i] = s.levelSlot[i];
    const int base = rank * per;
    if (DS && (OP == OP_BWD || OP == OP_GS))
        for (int i = threadIdx.x; i < per && base + i < n; i += CL_NT) Xl[i] = a.x[base + i];
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    constexpr int WARPS = CL_NT / 32;
    auto lslot = [&](int L) -> int { return L < nc ? lsl[L] : s.levelSlot[L]; };
    auto xat = [&](int c) -> T { return DS ? *cl_ref(cl, Xl, per, c) : ldcg(a.x + c); };
    auto xset = [&](int c, T v) {
        if (DS)
            *cl_ref(cl, Xl, per, c) = v;
        else
            a.x[c] = v;
    };
    auto header = [&](int L, SlotRegs<T, PF>& r) {
        int g = 0;
        bool ok = false;
        if (L < nL) {
            g = (lslot(L) >> 5) + rank + CS * w;
            ok = g < (lslot(L + 1) >> 5);
        }
        load_header<T, OP, PF>(s, a, g, ok, lane, r);
    };
    double dot = 0.0;
    auto level = [&](int L, SlotRegs<T, PF>& cur, SlotRegs<T, PF>& nxt) {
        const int g0 = lslot(L) >> 5, g1 = lslot(L + 1) >> 5;
        if (cur.c >= 0) {
            T acc = sw_init<OP>(cur.sc, cur.in, OP == OP_BWD ? xat(cur.c) : T(0));
#pragma unroll
            for (int k = 0; k < PF; ++k)
                if (k < cur.n) acc = sw_step<OP>(acc, cur.cf[k], xat(cur.nbr[k]));
            acc = tail_entries<T, OP>(s, a.coef, cur.e0, PF, cur.n, acc, xat);
            const T v = sw_fini<OP>(acc, cur.sc);
            xset(cur.c, v);
            if (a.dotWith) dot += double(v) * double(a.dotWith[cur.c]);
        }
        for (int g = g0 + rank + CS * (w + WARPS); g < g1; g += CS * WARPS) {
            const int slot = g * 32 + lane;
            const int c = s.cell[slot];
            if (c < 0) continue;
            const int cnt = s.cnt[slot];
            const int e0 = s.groupEntry[g] + lane;
            const T sc = a.scalar[slot];
            const T in = (OP == OP_FWD || OP == OP_GS) ? a.inS[slot] : T(0);
            T acc = sw_init<OP>(sc, in, OP == OP_BWD ? xat(c) : T(0));
            acc = tail_entries<T, OP>(s, a.coef, e0, 0, cnt, acc, xat);
            const T v = sw_fini<OP>(acc, sc);
            xset(c, v);
            if (a.dotWith) dot += double(v) * double(a.dotWith[c]);
        }
        cl.barrier_arrive();
        load_entries<T, PF>(s, a.coef, nxt);
        header(L + 2, cur);
        cl.barrier_wait();
    };
    SlotRegs<T, PF> A, B;
    header(0, A);
    header(1, B);
    load_entries<T, PF>(s, a.coef, A);
    cl.sync();
    for (int L = 0; L < nL; L += 2) {
        level(L, A, B);
        if (L + 1 < nL) level(L + 1, B, A);
    }
    if (DS)
        for (int i = threadIdx.x; i < per && base + i < n; i += CL_NT) a.x[base + i] = Xl[i];
    if (a.dotWith) {
        dot = block_sum<CL_NT>(dot, sh);
        if (threadIdx.x == 0) a.partials[rank] = dot;
    }
}

// Tile form.  Shared memory: the tile's values at tile-local indices.  Each
// CTA keeps, in its own row of s.seen (global memory, touched by its warp 0
// only), the progress it has observed of every tile, its own tiles' final
// counts included.  Warp 0 does the waits for the next level before the
// level barrier, which also votes on the abort: every thread leaves at the
// same barrier.
template <class T>
__host__ __device__ __forceinline__ size_t tile_x_bytes(int maxTileCells) {
    return (sizeof(T) * size_t(maxTileCells > 0 ? maxTileCells : 1) + 15) & ~size_t(15);
}

template <class T, int OP, int PF>
__global__ void __launch_bounds__(TILE_NT, 1) sweep_tile_k(DevSched s, SweepCtx<T> a, int* status) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double sh[TILE_NT / 32];
    if (a.done && *a.done) return;
    T* X = reinterpret_cast<T*>(smem_raw);
    int* seen = s.seen + size_t(blockIdx.x) * s.nTiles;
    for (int i = threadIdx.x; i < s.nTiles; i += TILE_NT) seen[i] = 0;
    int* abortf = s.sync;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    constexpr int NW = TILE_NT / 32;
    double dot = 0.0;
    __syncthreads();
    // warp 0: wait until every tile segment q reads from has published
    auto wait_seg = [&](int q) -> bool {
        bool ok = true;
        for (int k = s.segWait[q] + lane; k < s.segWait[q + 1]; k += 32) {
            const int p = s.waitTile[k], need = s.waitNeed[k];
            if (seen[p] >= need) continue;
            uint64_t t0 = 0;
            unsigned spins = 0;
            int v;
            while ((v = ld_acquire(s.progress + p)) < need) {
                if ((++spins & 63u) == 0) {
                    if (*(volatile int*)abortf) {
                        ok = false;
                        break;
                    }
                    const uint64_t t = globaltimer_ns();
                    if (t0 == 0) {
                        t0 = t;
                    } else if (t - t0 > a.timeoutNs) {
                        atomicExch(abortf, 1);
                        atomicExch(status, int(CFX_ERR_TIMEOUT));
                        ok = false;
                        break;
                    }
                }
            }
            if (!ok) break;
            seen[p] = v;
        }
        return ok;
    };
    auto xat = [&](int e) -> T { return e >= 0 ? X[e] : ldcg(a.x + (-e - 1)); };
    for (int ti = s.ctaTile[blockIdx.x]; ti < s.ctaTile[blockIdx.x + 1]; ++ti) {
        const int t = s.ctaTiles[ti];
        const int q0 = s.tileSeg[t], q1 = s.tileSeg[t + 1];
        // header of this warp's first group in segment q (and the slot's
        // tile-local index), issued two levels ahead
        auto hdr = [&](int q, SlotRegs<T, PF>& r, int& loc) {
            int g = 0;
            bool okg = false;
            if (q < q1) {
                g = s.segGroup[q] + w;
                okg = g < s.segGroup[q + 1];
            }
            load_header<T, OP, PF>(s, a, g, okg, lane, r);
            loc = okg ? s.slotLocal[g * 32 + lane] : 0;
        };
        bool ok = true;
        if (w == 0) ok = wait_seg(q0);
        if (!__syncthreads_and(ok)) return;
        // one entry set (the level being computed, then refilled with the
        // next level's before the barrier) and two headers in flight
        SlotRegs<T, PF> E;
        SlotRegs<T, 1> H;  // header of level q + 1 (only its header fields are used)
        int locE = 0, locH = 0;
        {
            SlotRegs<T, PF> tmp;
            hdr(q0, E, locE);
            load_entries<T, PF>(s, a.coef, E);
            hdr(q0 + 1, tmp, locH);
            H.c = tmp.c;
            H.n = tmp.n;
            H.e0 = tmp.e0;
            H.sc = tmp.sc;
            H.in = tmp.in;
        }
        for (int q = q0; q < q1; ++q) {
            if (E.c >= 0) {
                T acc = sw_init<OP>(E.sc, E.in, OP == OP_BWD ? ldcg(a.x + E.c) : T(0));
#pragma unroll
                for (int k = 0; k < PF; ++k)
                    if (k < E.n) acc = sw_step<OP>(acc, E.cf[k], xat(E.nbr[k]));
                acc = tail_entries<T, OP>(s, a.coef, E.e0, PF, E.n, acc, xat);
                const T v = sw_fini<OP>(acc, E.sc);
                X[locE] = v;
                a.x[E.c] = v;
                if (a.dotWith) dot += double(v) * double(a.dotWith[E.c]);
            }
            // further groups of this warp in a wide level, loaded directly
            for (int g = s.segGroup[q] + w + NW; g < s.segGroup[q + 1]; g += NW) {
                const int slot = g * 32 + lane;
                const int c = s.cell[slot];
                if (c < 0) continue;
                const int cnt = s.cnt[slot];
                const int e0 = s.groupEntry[g] + lane;
                const T sc = a.scalar[slot];
                const T in = (OP == OP_FWD || OP == OP_GS) ? a.inS[slot] : T(0);
                T acc = sw_init<OP>(sc, in, OP == OP_BWD ? ldcg(a.x + c) : T(0));
                acc = tail_entries<T, OP>(s, a.coef, e0, 0, cnt, acc, xat);
                const T v = sw_fini<OP>(acc, sc);
                X[s.slotLocal[slot]] = v;
                a.x[c] = v;
                if (a.dotWith) dot += double(v) * double(a.dotWith[c]);
            }
            // level q + 1: its header (issued a level ago) becomes current and
            // its entries are issued now; the header of q + 2 is issued
            E.c = H.c;
            E.n = H.n;
            E.e0 = H.e0;
            E.sc = H.sc;
            E.in = H.in;
            locE = locH;
            load_entries<T, PF>(s, a.coef, E);
            {
                SlotRegs<T, 1> tmp;
                int g = 0;
                bool okg = false;
                if (q + 2 < q1) {
                    g = s.segGroup[q + 2] + w;
                    okg = g < s.segGroup[q + 3];
                }
                load_header<T, OP, 1>(s, a, g, okg, lane, tmp);
                locH = okg ? s.slotLocal[g * 32 + lane] : 0;
                H = tmp;
            }
            ok = true;
            if (w == 0 && q + 1 < q1) ok = wait_seg(q + 1);
            if (!__syncthreads_and(ok)) return;
            if (threadIdx.x == 0) {
                const int done = q - q0 + 1;
                if (done % s.pubEvery == 0 || q + 1 == q1) {
                    st_release(s.progress + t, done);
                    seen[t] = done;
                }
            }
        }
    }
    if (a.dotWith) {
        dot = block_sum<TILE_NT>(dot, sh);
        if (threadIdx.x == 0) a.partials[blockIdx.x] = dot;
    }
}

// Right-hand side gathered into slot order, so the sweeps load it without
// first loading the slot's cell index.
template <class T>
__global__ void gather_slots_k(int nSlots, const int* __restrict__ cell, const T* __restrict__ in,
                               T* __restrict__ inS, const int* done) {
    if (done && *done) return;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nSlots; t += gridDim.x * blockDim.x) {
        const int c = cell[t];
        inS[t] = c >= 0 ? in[c] : T(0);
    }
}

// Coefficients of a schedule for one operation (per matrix update).
template <class T>
__global__ void pack_k(DevSched s, int op, const T* __restrict__ lp, const T* __restrict__ up,
                       const T* __restrict__ upper, const T* __restrict__ diag, const T* __restrict__ rD,
                       T* __restrict__ coef, T* __restrict__ scalar) {
    const int nThreads = s.nGroups * 32;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nThreads; t += gridDim.x * blockDim.x) {
        const int g = t >> 5, lane = t & 31;
        const int c = s.cell[t];
        const int K = (s.groupEntry[g + 1] - s.groupEntry[g]) >> 5;
        const int e0 = s.groupEntry[g] + lane;
        const int n = c >= 0 ? s.cnt[t] : 0;
        scalar[t] = c < 0 ? T(0) : ((op == OP_FWD || op == OP_BWD) ? rD[c] : diag[c]);
        for (int k = 0; k < K; ++k) {
            const int e = e0 + 32 * k;
            T v = T(0);
            if (k < n) {
                const int src = s.src[e];
                const int i = src & (SRC_UPPER - 1);
                if (op == OP_FWD) v = rD[c] * lp[i];
                else if (op == OP_BWD) v = rD[c] * upper[i];
                else if (op == OP_GS) v = (src & SRC_UPPER) ? upper[i] : lp[i];
                else v = up[i] * lp[i];  // OP_RD: upper*upper (DIC) / upper*lower (DILU)
            }
            coef[e] = v;
        }
    }
}

template <class T>
inline int prec_index();
template <>
inline int prec_index<double>() { return 0; }
template <>
inline int prec_index<float>() { return 1; }

enum Mode { M_CTA = 0, M_CLUSTER_DS = 1, M_CTA_GLOBAL = 2, M_CLUSTER_GLOBAL = 3, M_GRID = 4, M_TILE = 5 };

// Execution form of a schedule: the vector in one CTA's shared memory, in a
// cluster's distributed shared memory, or in global memory with a single CTA,
// one cluster, or the whole grid separating the levels.
// CTAs per cluster for a schedule: the cluster knob, else for the DIC/DILU
// forward/backward schedules the preconditioner cluster size.  The vector
// of a PCG+DIC 64^3 system fits a 16-CTA cluster's shared memory, and its
// sweeps run 1.5x faster there than on the grid; the Gauss-Seidel sweeps of
// GAMG's levels were measured slower there, so they keep the grid.
inline int cluster_of(const DevSched& s) {
    if (g_cluster) return g_cluster;
    return (s.kind == SCHED_FWD || s.kind == SCHED_BWD) ? g_cluster_pre : 0;
}

template <class T>
int mode_of(const DevSched& s) {
    if (s.tiled) return M_TILE;
    const size_t xbytes = sizeof(T) * size_t(s.n);
    if (xbytes <= g_smem_cap) return M_CTA;
    const int cs = cluster_of(s);
    if (cs) {
        const int per = (s.n + cs - 1) / cs;
        if (sizeof(T) * size_t(per) <= g_smem_cap) return M_CLUSTER_DS;
    }
    if (s.n <= g_small_threshold) return M_CTA_GLOBAL;
    if (g_cluster && s.n <= g_cluster_global) return M_CLUSTER_GLOBAL;
    return M_GRID;
}

constexpr int pf_index(int pf) { return pf == PF_SMALL ? 0 : pf == PF_LARGE ? 1 : 2; }

template <class T, int OP, int PF>
cfx_status launch_grid(cudaStream_t st, const DevSched& s, const SweepCtx<T>& a, int* status);

template <class T>
size_t tile_smem_bytes(const DevSched& s) {
    return tile_x_bytes<T>(s.maxTileCells);
}

// The tile form: one cooperative launch of s.grid CTAs (all resident), the
// progress counters and the abort flag cleared first.
template <class T, int OP, int PF>
cfx_status launch_tile(cudaStream_t st, const DevSched& s, const SweepCtx<T>& a, int* status) {
    const size_t smem = tile_smem_bytes<T>(s);
    if (smem > g_smem_cap_max || s.grid > g_tile_ctas) {
        set_error("tiled sweep: schedule exceeds the shared memory or the resident CTAs");
        return CFX_ERR_STATE;
    }
    CFX_CUDA(cudaMemsetAsync(s.sync, 0, sizeof(int) * 2, st));
    CFX_CUDA(cudaMemsetAsync(s.progress, 0, sizeof(int) * size_t(s.nTiles), st));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(s.grid);
    cfg.blockDim = dim3(TILE_NT);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    CFX_CUDA(cudaLaunchKernelEx(&cfg, sweep_tile_k<T, OP, PF>, s, a, status));
    count_launch();
    return CFX_OK;
}

template <class T, int OP, int PF>
cfx_status launch_pf(cudaStream_t st, const DevSched& s, const SweepCtx<T>& a, int* status) {
    if (s.nSlots == 0) return CFX_OK;
    if (s.tiled) return launch_tile<T, OP, PF>(st, s, a, status);
    const size_t xbytes = sizeof(T) * size_t(s.n);
    const int cs = cluster_of(s);
    const int per = cs ? (s.n + cs - 1) / cs : 0;
    const int m = mode_of<T>(s);
    if (m == M_CTA) {
        sweep_cta_k<T, OP, true, PF><<<1, CTA_NT, xbytes, st>>>(s, a);
    } else if (m == M_CLUSTER_DS || m == M_CLUSTER_GLOBAL) {
        const bool ds = m == M_CLUSTER_DS;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(cs);
        cfg.blockDim = dim3(CL_NT);
        cfg.dynamicSmemBytes = ds ? sizeof(T) * size_t(per) : 0;
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = cs;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        if (ds)
            CFX_CUDA(cudaLaunchKernelEx(&cfg, sweep_cluster_k<T, OP, true, PF>, s, a, per));
        else
            CFX_CUDA(cudaLaunchKernelEx(&cfg, sweep_cluster_k<T, OP, false, PF>, s, a, per));
    } else if (m == M_CTA_GLOBAL) {
        sweep_cta_k<T, OP, false, PF><<<1, CTA_NT, 0, st>>>(s, a);
    } else if (sizeof(T) == 4 && PF == PF_LARGE && s.maxK > PF_LARGE) {
        // FP32: the grid form holds up to PF_GRID_XL entries (one register
        // set).  In FP64 the larger set costs more in occupancy than it saves.
        return launch_grid<T, OP, (sizeof(T) == 4 ? PF_GRID_XL : PF_LARGE)>(st, s, a, status);
    } else {
        return launch_grid<T, OP, PF>(st, s, a, status);
    }
    count_launch();
    return CFX_OK;
}

// CTAs of a wavefront launch: the smallest residency over the operations
// (so a schedule's dot-partial count does not depend on the operation), at
// most one warp per group.
int wave_ctas(int prec, int pf, int nGroups) {
    int r = 1 << 30;
    for (int op = 0; op < 4; ++op) r = std::min(r, g_wave_grid[prec][op][pf_index(pf)]);
    const int need = (nGroups + GRID_NT / 32 - 1) / (GRID_NT / 32);
    r = std::min(r, need);
    return r > 0 ? r : 1;
}

template <class T, int OP, int PF>
cfx_status launch_grid(cudaStream_t st, const DevSched& s, const SweepCtx<T>& a, int* status) {
    if (g_wave && s.waveOk) {
        CFX_CUDA(cudaMemsetAsync(s.sync, 0, sizeof(int) * 2, st));
        CFX_CUDA(cudaMemsetAsync(s.gdone, 0, sizeof(int) * size_t(s.nGroups), st));
        const int grid = wave_ctas(prec_index<T>(), PF, s.nGroups);
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(grid > 0 ? grid : 1);
        cfg.blockDim = dim3(GRID_NT);
        cfg.dynamicSmemBytes = 0;
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        CFX_CUDA(cudaLaunchKernelEx(&cfg, sweep_wave_k<T, OP, PF>, s, a, status));
        count_launch();
        return CFX_OK;
    }
    {
        CFX_CUDA(cudaMemsetAsync(s.sync, 0, sizeof(int) * (2 + s.nLevels), st));
        const int grid = std::min(s.nChunks, g_grid[prec_index<T>()][OP][pf_index(PF)]);
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(grid);
        cfg.blockDim = dim3(GRID_NT);
        cfg.dynamicSmemBytes = 0;
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        CFX_CUDA(cudaLaunchKernelEx(&cfg, sweep_grid_k<T, OP, PF>, s, a, status));
    }
    count_launch();
    return CFX_OK;
}

// Slots with at most PF_SMALL entries (hexahedral fine levels) take the
// lighter register set; agglomerated levels, whose cells have many more
// neighbours, hold PF_LARGE entries per slot in registers.
template <class T, int OP>
cfx_status launch(cudaStream_t st, const DevSched& s, const SweepCtx<T>& a, int* status) {
    if (s.maxK <= PF_SMALL) return launch_pf<T, OP, PF_SMALL>(st, s, a, status);
    return launch_pf<T, OP, PF_LARGE>(st, s, a, status);
}

template <class T, int OP, int PF>
void init_op_pf() {
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, sweep_grid_k<T, OP, PF>, GRID_NT, 0);
    g_grid[prec_index<T>()][OP][pf_index(PF)] = g_num_sms * (per > 0 ? per : 1);
    per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, sweep_wave_k<T, OP, PF>, GRID_NT, 0);
    g_wave_grid[prec_index<T>()][OP][pf_index(PF)] = g_num_sms * (per > 0 ? per : 1);
    cudaFuncSetAttribute(sweep_tile_k<T, OP, PF>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(g_smem_cap));
    cudaFuncSetAttribute(sweep_cta_k<T, OP, true, PF>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(g_smem_cap));
    cudaFuncSetAttribute(sweep_cluster_k<T, OP, true, PF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         int(g_smem_cap));
    cudaFuncSetAttribute(sweep_cluster_k<T, OP, true, PF>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaFuncSetAttribute(sweep_cluster_k<T, OP, false, PF>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
}

template <class T, int OP>
void init_op() {
    init_op_pf<T, OP, PF_SMALL>();
    init_op_pf<T, OP, PF_LARGE>();
    if (sizeof(T) == 4) {
        constexpr int XL = sizeof(T) == 4 ? PF_GRID_XL : PF_LARGE;
        int per = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, sweep_grid_k<T, OP, XL>, GRID_NT, 0);
        g_grid[prec_index<T>()][OP][pf_index(XL)] = g_num_sms * (per > 0 ? per : 1);
        per = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, sweep_wave_k<T, OP, XL>, GRID_NT, 0);
        g_wave_grid[prec_index<T>()][OP][pf_index(XL)] = g_num_sms * (per > 0 ? per : 1);
    }
}

// Largest cluster (16, else 8) that can be resident with a full-size
// shared-memory partition per CTA; 0 when none can.
int probe_cluster() {
    for (int cs : {16, 8}) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(cs);
        cfg.blockDim = dim3(CL_NT);
        cfg.dynamicSmemBytes = g_smem_cap;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = cs;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int num = 0;
        if (cudaOccupancyMaxActiveClusters(&num, sweep_cluster_k<double, OP_GS, true, PF_LARGE>, &cfg) == cudaSuccess && num > 0)
            return cs;
        cudaGetLastError();
    }
    return 0;
}

template <class T>
void init_attrs() {
    init_op<T, OP_FWD>();
    init_op<T, OP_BWD>();
    init_op<T, OP_GS>();
    init_op<T, OP_RD>();
}

}  // namespace

void sweeps_init(int numSms) {
    g_num_sms = numSms > 0 ? numSms : 152;
    int dev = 0;
    cudaGetDevice(&dev);
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    // leave room for the kernels' static shared memory (level bounds cache)
    constexpr int reserve = 4096 + 4 * (LS_CACHE + 1);
    if (optin > reserve) g_smem_cap = size_t(optin) - reserve;
    g_smem_cap_max = g_smem_cap;
    init_attrs<double>();
    init_attrs<float>();
    // resident tile CTAs with a full shared-memory partition each
    {
        int per = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, sweep_tile_k<double, OP_GS, PF_LARGE>, TILE_NT,
                                                      g_smem_cap);
        g_tile_ctas = g_num_sms * (per > 0 ? per : 1);
        cudaGetLastError();
    }
    // The cluster forms are kept behind CFX_TUNE_CLUSTER_SIZE: on GB300 the
    // persistent grid form sweeps the mid-size levels faster (a cluster
    // barrier per level costs more than the grid's per-level counters).
    g_cluster_avail = probe_cluster();
    g_cluster = 0;
    g_cluster_pre = g_cluster_avail >= 16 ? 16 : 0;
}

int sweep_cluster_size() { return g_cluster; }
int sweep_cluster_pre() { return g_cluster_pre; }
void set_sweep_cluster_pre(int cs) { g_cluster_pre = cs <= g_cluster_avail ? cs : g_cluster_avail; }
void set_sweep_cluster_size(int cs) { g_cluster = cs <= g_cluster_avail ? cs : g_cluster_avail; }

int small_sweep_threshold() { return g_small_threshold; }
void set_small_sweep_threshold(int n) { g_small_threshold = n; }
size_t sweep_smem_cap() { return g_smem_cap; }
size_t sweep_smem_cap_max() { return g_smem_cap_max; }
void set_sweep_smem_cap(size_t b) { g_smem_cap = b; }

// CTAs of the wavefront launch for s (its dot partial count)
template <class T>
int wave_grid(const DevSched& s) {
    const int pf = s.maxK <= PF_SMALL ? PF_SMALL : (sizeof(T) == 4 && s.maxK > PF_LARGE ? PF_GRID_XL : PF_LARGE);
    return wave_ctas(prec_index<T>(), pf, s.nGroups);
}

int sweep_wave() { return g_wave; }
void set_sweep_wave(int on) { g_wave = on ? 1 : 0; }
int sweep_tile() { return g_tile; }
void set_sweep_tile(int on) { g_tile = on ? 1 : 0; }
int sweep_tile_pub() { return g_tile_pub; }
void set_sweep_tile_pub(int k) { g_tile_pub = k < 1 ? 1 : k; }
int sweep_tile_ctas() { return g_tile_ctas; }

template <class T>
bool sweep_is_grid(const DevSched& s) {
    return mode_of<T>(s) == M_GRID;
}

template <class T>
int sweep_partials(const DevSched& s) {
    const int m = mode_of<T>(s);
    if (m == M_TILE) return s.grid;
    if (m == M_GRID) return g_wave && s.waveOk ? wave_grid<T>(s) : s.nChunks;
    return (m == M_CLUSTER_DS || m == M_CLUSTER_GLOBAL) ? cluster_of(s) : 1;
}

int cluster_global_cells() { return g_cluster_global; }
void set_cluster_global_cells(int n) { g_cluster_global = n; }

template <class T>
cfx_status run_sweep(cudaStream_t st, const DevSched& s, int op, const Packed<T>& p, const T* in, T* x,
                     const T* dotWith, double* partials, const int* done, int* status) {
    if ((op == OP_FWD || op == OP_GS) && s.nSlots > 0) {
        int blocks = (s.nSlots + 255) / 256;
        if (blocks > 4096) blocks = 4096;
        gather_slots_k<T><<<blocks, 256, 0, st>>>(s.nSlots, s.cell, in, p.inS, done);
        count_launch();
    }
    SweepCtx<T> a{p.coef, p.scalar, in, p.inS, x, dotWith, partials, done, SWEEP_TIMEOUT_NS};
    switch (op) {
        case OP_FWD: return launch<T, OP_FWD>(st, s, a, status);
        case OP_BWD: return launch<T, OP_BWD>(st, s, a, status);
        case OP_GS: return launch<T, OP_GS>(st, s, a, status);
        case OP_RD: return launch<T, OP_RD>(st, s, a, status);
        default: set_error("unknown sweep"); return CFX_ERR_ARG;
    }
}

// A Gauss-Seidel sweep in the level-counter grid form whose level-0
// completion counter starts one short, so every chunk of level 1 waits on a
// count that is never reached: each wait expires after timeoutNs, the kernel
// sets the abort flag and CFX_ERR_TIMEOUT in *status, and every CTA returns.
// Exercises the failure path of the bounded waits without any fault.
template <class T>
cfx_status run_sweep_stalled(cudaStream_t st, const DevSched& s, const Packed<T>& p, const T* in, T* x,
                             unsigned long long timeoutNs, int* status) {
    if (s.nLevels < 2 || s.nSlots == 0 || s.tiled) {
        set_error("stalled sweep: the schedule needs at least two levels (level-ordered, not tiled)");
        return CFX_ERR_ARG;
    }
    int blocks = (s.nSlots + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    gather_slots_k<T><<<blocks, 256, 0, st>>>(s.nSlots, s.cell, in, p.inS, nullptr);
    count_launch();
    SweepCtx<T> a{p.coef, p.scalar, in, p.inS, x, nullptr, nullptr, nullptr, timeoutNs};
    CFX_CUDA(cudaMemsetAsync(s.sync, 0, sizeof(int) * (2 + s.nLevels), st));
    CFX_CUDA(cudaMemsetAsync(s.sync + 2, 0xff, sizeof(int), st));  // done[0] = -1
    auto go = [&](auto kern, int pf) -> cfx_status {
        const int grid = std::min(s.nChunks, g_grid[prec_index<T>()][OP_GS][pf_index(pf)]);
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(grid > 0 ? grid : 1);
        cfg.blockDim = dim3(GRID_NT);
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        CFX_CUDA(cudaLaunchKernelEx(&cfg, kern, s, a, status));
        count_launch();
        return CFX_OK;
    };
    if (s.maxK <= PF_SMALL) return go(sweep_grid_k<T, OP_GS, PF_SMALL>, PF_SMALL);
    return go(sweep_grid_k<T, OP_GS, PF_LARGE>, PF_LARGE);
}

template <class T>
void pack_sweep(cudaStream_t st, const DevSched& s, int op, const LevelCoeffs<T>& c, Packed<T>& p) {
    if (s.nGroups == 0) {
        p.valid = true;
        return;
    }
    const T* up = c.sym ? c.lowerPerm : c.upperPerm;
    const int threads = 256;
    int blocks = (s.nGroups * 32 + threads - 1) / threads;
    if (blocks > 4096) blocks = 4096;
    pack_k<T><<<blocks, threads, 0, st>>>(s, op, c.lowerPerm, up, c.upper, c.diag, c.rD, p.coef, p.scalar);
    count_launch();
    p.valid = true;
}

template bool sweep_is_grid<double>(const DevSched&);
template bool sweep_is_grid<float>(const DevSched&);
template int sweep_partials<double>(const DevSched&);
template int sweep_partials<float>(const DevSched&);
template cfx_status run_sweep<double>(cudaStream_t, const DevSched&, int, const Packed<double>&, const double*,
                                      double*, const double*, double*, const int*, int*);
template cfx_status run_sweep<float>(cudaStream_t, const DevSched&, int, const Packed<float>&, const float*, float*,
                                     const float*, double*, const int*, int*);
template cfx_status run_sweep_stalled<double>(cudaStream_t, const DevSched&, const Packed<double>&,
                                               const double*, double*, unsigned long long, int*);
template void pack_sweep<double>(cudaStream_t, const DevSched&, int, const LevelCoeffs<double>&, Packed<double>&);
template void pack_sweep<float>(cudaStream_t, const DevSched&, int, const LevelCoeffs<float>&, Packed<float>&);

}  // namespace cfx
