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
//   sweep_cta_k   one CTA of 256 threads walks the levels with block
//                 barriers, each warp's next group prefetched into registers
//                 (up to 32 entries per slot); the vector lives in shared
//                 memory when it fits.  Used for coarse levels and small
//                 meshes.
//   sweep_cluster_k  a cluster of up to 16 CTAs (one GPC) holds the vector in
//                 distributed shared memory (cell c in CTA c / per) and
//                 separates levels with the hardware cluster barrier; each
//                 warp prefetches its next group's packed data into registers
//                 before the barrier.  Used up to ~16x the single-CTA size.
//   sweep_grid_k  persistent CTAs, chunk J (by default 2 groups of 32
//                 slots, level order) on CTA J mod grid; each CTA loads its next chunk's
//                 packed data, then waits (bounded spin, acquire) for every
//                 chunk of the previous level to release its done-counter.
//                 Launched cooperatively so all CTAs are resident.  A wait
//                 that exceeds its deadline sets the abort flag and an error
//                 status; every CTA then returns.
//   sweep_flow_k  dataflow: persistent warps take the level-ordered groups
//                 round-robin; every value a sweep produces goes to a buffer
//                 filled beforehand with a sentinel (all bits set, a NaN no
//                 arithmetic produces), and a slot spins, with a bounded and
//                 backed-off wait, on exactly the neighbour values it reads
//                 until they are no longer the sentinel.  The value is its own
//                 flag: no counters, release fences or block barriers, so a
//                 dependency costs one store-to-load trip through L2.
//   sweep_level_k one ordinary launch per DAG level (a warp per group, no
//                 waits: the launch order separates the levels), for
//                 schedules of few, wide levels (the multicolour ones: a few
//                 colours per sweep), where the persistent forms' per-chunk
//                 waits and counters cost more than a launch per level.

#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>

#include "device.cuh"
#include "internal.h"
#include "solvers.h"

namespace cfx {

namespace {

constexpr uint64_t SWEEP_TIMEOUT_NS = 2000000000ull;  // 2 s per wait
constexpr int GRID_NT = 256;                            // 8 warps = one chunk
constexpr int CTA_NT = 256;
constexpr int CL_NT = 256;                              // threads per cluster CTA
constexpr int PF_SMALL = 8, PF_LARGE = 16, PF_GRID_XL = 32;  // entries held in registers per slot
namespace cg = cooperative_groups;

int g_num_sms = 152;
int g_cluster = 0;          // CTAs per cluster of sweep_cluster_k (0: not used)
int g_cluster_pre = 0;      // the same for the DIC/DILU (forward/backward) schedules when g_cluster is 0
int g_cluster_avail = 0;    // largest cluster the GPU can hold (16 or 8; 0: none)
int g_small_threshold = 0;  // <= this many cells: single-CTA even without smem fit
int g_cluster_global = 0;   // <= this many cells: one cluster with the vector in global memory
int g_grid[2][8][3];        // resident CTAs of sweep_grid_k per (precision, op, PF 8/16/32)
int g_flow_grid[2][4];      // resident CTAs of sweep_flow_k per (precision, op)
int g_wave_grid[2][8][3];   // resident CTAs of sweep_wave_k, the same
int g_wave = 0;             // grid form: wavefront (1) or whole-level counters (0, default)
size_t g_smem_cap = 200 * 1024;
size_t g_smem_cap_max = 200 * 1024;
int g_flow = 2;             // the dataflow form: 0 off, 1 on, 2 for schedules of <= PF_SMALL entries
int g_flow_ahead = 4;       // dataflow form: levels of groups in flight (warps launched)
int g_cta_xl = 1;           // single-CTA form, FP32: PF_GRID_XL entries per slot in registers when slots have more than PF_LARGE
int g_level_launch = 96;    // schedules of at most this many levels run one launch per level (0: never)
int g_lvl_stride = 1;       // level-counter grid form: ints between consecutive level counters
int g_poll_ns = 0;          // and the back-off of its waiting polls (ns)

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
    const int stride = s.lvlStride;
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
                const int* d = done + size_t(L - 1) * stride;
                uint64_t t0 = 0;
                unsigned spins = 0;
                // acquire loads: the load that sees the count orders the
                // reads of the previous level's values after it
                while (ld_acquire(d) < target) {
                    if (s.pollNs) __nanosleep(s.pollNs);
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
        if (threadIdx.x == 0) red_release_add(done + size_t(L) * stride, 1);
    }
}

// Level-by-level form: groups g0..g1 of one DAG level, LVL_LAUNCH_GROUPS
// warps per CTA, a warp per group.  Every value a slot reads comes from an
// earlier level (an earlier launch), and the cells of one level are
// independent, so x is updated in place without waits.  The levels are
// launched as programmatic dependents of one another: a level's grid starts
// while the previous level runs, loads its slots' schedule data (cell,
// entry count, the first PF columns and coefficients, scalar, right-hand
// side by cell; all written by kernels that completed before the previous
// level passed its own wait, read through L2) and only then waits
// (griddepcontrol.wait) for the previous level's values; it lets its own
// dependents start once past that wait, so a level's prologue never reads
// anything a still-running kernel writes.  The dot partial (when requested)
// is one per CTA, at p0 + blockIdx.x.
struct LevelView {
    const int *cell, *cnt, *groupEntry, *nb;
};

template <class T, int OP, int PF>
__global__ void __launch_bounds__(32 * LVL_LAUNCH_GROUPS) sweep_level_k(LevelView s, SweepCtx<T> a, int g0, int g1,
                                                                       int p0) {
    constexpr int NT = 32 * LVL_LAUNCH_GROUPS;
    __shared__ double sh[LVL_LAUNCH_GROUPS];
    const int lane = threadIdx.x & 31;
    const int g = g0 + blockIdx.x * LVL_LAUNCH_GROUPS + (threadIdx.x >> 5);
    int c = -1, n = 0, e0 = 0;
    T sc = T(0), in = T(0);
    int nbr[PF];
    T cf[PF];
    if (g < g1) {
        const int slot = g * 32 + lane;
        c = ldcg(s.cell + slot);
        n = ldcg(s.cnt + slot);
        e0 = ldcg(s.groupEntry + g) + lane;
        sc = ldcg(a.scalar + slot);
#pragma unroll
        for (int k = 0; k < PF; ++k)
            if (k < n) {
                nbr[k] = ldcg(s.nb + e0 + 32 * k);
                cf[k] = ldcg(a.coef + e0 + 32 * k);
            }
        if ((OP == OP_FWD || OP == OP_GS) && c >= 0) in = ldcg(a.in + c);
    }
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    if (a.done && ldcg(a.done)) return;
    T v = T(0);
    if (c >= 0) {
        T acc = sw_init<OP>(sc, in, OP == OP_BWD ? ldcg(a.x + c) : T(0));
#pragma unroll
        for (int k = 0; k < PF; ++k)
            if (k < n) acc = sw_step<OP>(acc, cf[k], ldcg(a.x + nbr[k]));
        for (int kb = PF; kb < n; kb += 8) {
            int nb[8];
            T cb[8];
#pragma unroll
            for (int j = 0; j < 8; ++j)
                if (kb + j < n) {
                    nb[j] = ldcg(s.nb + e0 + 32 * (kb + j));
                    cb[j] = ldcg(a.coef + e0 + 32 * (kb + j));
                }
#pragma unroll
            for (int j = 0; j < 8; ++j)
                if (kb + j < n) acc = sw_step<OP>(acc, cb[j], ldcg(a.x + nb[j]));
        }
        v = sw_fini<OP>(acc, sc);
        a.x[c] = v;
    }
    if (a.dotWith) {
        double p = c >= 0 ? double(v) * double(ldcg(a.dotWith + c)) : 0.0;
        p = block_sum<NT>(p, sh);
        if (threadIdx.x == 0) a.partials[p0 + blockIdx.x] = p;
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

// Dataflow form.
constexpr int FLOW_NT = 256;
constexpr int FLOW_B = 8;  // entries per batch (all of a hexahedral cell's)

template <class T>
__device__ __forceinline__ T ld_flow(const T* p);
template <>
__device__ __forceinline__ double ld_flow<double>(const double* p) {
    double v;
    asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
    return v;
}
template <>
__device__ __forceinline__ float ld_flow<float>(const float* p) {
    float v;
    asm volatile("ld.relaxed.gpu.global.f32 %0, [%1];" : "=f"(v) : "l"(p) : "memory");
    return v;
}
template <class T>
__device__ __forceinline__ void st_flow(T* p, T v);
template <>
__device__ __forceinline__ void st_flow<double>(double* p, double v) {
    asm volatile("st.relaxed.gpu.global.f64 [%0], %1;" ::"l"(p), "d"(v) : "memory");
}
template <>
__device__ __forceinline__ void st_flow<float>(float* p, float v) {
    asm volatile("st.relaxed.gpu.global.f32 [%0], %1;" ::"l"(p), "f"(v) : "memory");
}
// the sentinel: all bits set
__device__ __forceinline__ bool flow_unset(double v) { return __double_as_longlong(v) == -1LL; }
__device__ __forceinline__ bool flow_unset(float v) { return __float_as_int(v) == -1; }
// a computed value that happens to have the sentinel's bits (a NaN) is
// stored as the canonical quiet NaN instead
__device__ __forceinline__ double flow_value(double v) {
    return flow_unset(v) ? __longlong_as_double(0x7ff8000000000000LL) : v;
}
__device__ __forceinline__ float flow_value(float v) { return flow_unset(v) ? __int_as_float(0x7fc00000) : v; }

// Wait for the value at p: relaxed loads (the value is the flag; nothing
// else is published with it), backing off with nanosleep, bounded by
// timeoutNs of %globaltimer; on expiry the abort flag and CFX_ERR_TIMEOUT
// are set and ok is cleared.
template <class T>
__device__ __forceinline__ T flow_wait(const T* p, int* abortf, int* status, unsigned long long timeoutNs, bool& ok) {
    T v = ld_flow(p);
    if (!flow_unset(v)) return v;
    uint64_t t0 = 0;
    unsigned spins = 0;
    while (flow_unset(v)) {
        // poll back to back at first (the value is usually a level away),
        // then back off
        if (spins > 32) __nanosleep(64);
        if ((++spins & 15u) == 0) {
            if (*(volatile int*)abortf) {
                ok = false;
                return T(0);
            }
            const uint64_t t = globaltimer_ns();
            if (t0 == 0) {
                t0 = t;
            } else if (t - t0 > timeoutNs) {
                atomicExch(abortf, 1);
                atomicExch(status, int(CFX_ERR_TIMEOUT));
                ok = false;
                return T(0);
            }
        }
        v = ld_flow(p);
    }
    return v;
}

// out: [nSweeps][n] values (sentinel-filled); for the forward and pivot
// sweeps out is x itself.  Reads: Gauss-Seidel, a slot of sweep sw takes
// its lower neighbours from out[sw] and its upper ones from out[sw - 1] (x,
// the values before the launch, for sw = 0); the backward Gauss-Seidel pass
// takes its lower neighbours from x and its upper ones from out; the
// forward, pivot and backward sweeps take every neighbour from out (the
// backward one its own previous value from x).  Warps take groups W, W + NW,
// ... in level order, and every group reads only groups of earlier levels:
// with all warps resident (cooperative launch) the lowest unfinished group
// can always proceed.  The dot partial (when requested) is summed per warp
// in its group order, then per CTA (nPartials = gridDim.x).
template <class T, int OP>
__global__ void __launch_bounds__(FLOW_NT) sweep_flow_k(DevSched s, SweepCtx<T> a, T* out, int* status) {
    __shared__ double sh[FLOW_NT / 32];
    if (a.done && *a.done) return;
    int* abortf = s.sync;
    const int n = s.n;
    const int lane = threadIdx.x & 31;
    const int W = blockIdx.x * (FLOW_NT / 32) + (threadIdx.x >> 5);
    const int NW = gridDim.x * (FLOW_NT / 32);
    const bool gs = s.kind == SCHED_GS, gsb = s.kind == SCHED_GSB;
    double dot = 0.0;
    bool ok = true;
    for (int g = W; g < s.nGroups; g += NW) {
        // the warp's lanes finish a group together, so no lane runs ahead
        // into a later group and competes with the ones still on this level
        __syncwarp();
        if (!__all_sync(0xffffffffu, ok)) break;
        const int slot = g * 32 + lane;
        const int c = s.cell[slot];
        if (c < 0) continue;
        const int cnt = s.cnt[slot];
        const int e0 = s.groupEntry[g] + lane;
        const T sc = a.scalar[slot];
        const T in = (OP == OP_FWD || OP == OP_GS) ? a.inS[slot] : T(0);
        const int sw = gs ? s.slotSweep[slot] : 0;
        const int nLow = (gs || gsb) ? s.slotLower[slot] : 0;
        const T* cur = out + size_t(sw) * n;
        const T* prev = sw > 0 ? out + size_t(sw - 1) * n : a.x;
        T acc = sw_init<OP>(sc, in, OP == OP_BWD ? ldcg(a.x + c) : T(0));
        // where entry k's value lives and whether it is produced in this launch
        auto src_of = [&](int k, int nbk, bool& live) -> const T* {
            if (gs) {
                live = k < nLow || sw > 0;
                return (k < nLow ? cur : prev) + nbk;
            }
            if (gsb) {
                live = k >= nLow;
                return (k < nLow ? a.x : cur) + nbk;
            }
            live = true;
            return cur + nbk;
        };
        // batches of FLOW_B entries: every value load of a batch is issued
        // before the first is waited on, so a slot pays one trip through L2
        // per batch plus the wait for the values still being produced
        for (int kb = 0; kb < cnt && ok; kb += FLOW_B) {
            int nb[FLOW_B];
            T cf[FLOW_B], v[FLOW_B];
#pragma unroll
            for (int j = 0; j < FLOW_B; ++j)
                if (kb + j < cnt) {
                    nb[j] = s.nb[e0 + 32 * (kb + j)];
                    cf[j] = a.coef[e0 + 32 * (kb + j)];
                }
#pragma unroll
            for (int j = 0; j < FLOW_B; ++j)
                if (kb + j < cnt) {
                    bool live;
                    const T* p = src_of(kb + j, nb[j], live);
                    v[j] = live ? ld_flow(p) : ldcg(p);
                }
#pragma unroll
            for (int j = 0; j < FLOW_B; ++j)
                if (kb + j < cnt && ok) {
                    bool live;
                    const T* p = src_of(kb + j, nb[j], live);
                    if (live && flow_unset(v[j])) v[j] = flow_wait(p, abortf, status, a.timeoutNs, ok);
                    acc = sw_step<OP>(acc, cf[j], v[j]);
                }
        }
        if (!ok) continue;
        const T v = flow_value(sw_fini<OP>(acc, sc));
        st_flow(out + size_t(sw) * n + c, v);
        if (a.dotWith) dot += double(v) * double(a.dotWith[c]);
    }
    __syncwarp();
    if (a.dotWith) {
        dot = block_sum<FLOW_NT>(dot, sh);
        if (threadIdx.x == 0) a.partials[blockIdx.x] = dot;
    }
}

// The dataflow form's buffers: filled with the sentinel before the sweep,
// and the last sweep's values copied back into x after it.
template <class T>
__global__ void flow_fill_k(int64_t nv, T* out, const int* done) {
    if (done && *done) return;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < nv; i += int64_t(gridDim.x) * blockDim.x)
        out[i] = sizeof(T) == 8 ? T(__longlong_as_double(-1LL)) : T(__int_as_float(-1));
}

template <class T>
__global__ void flow_copy_k(int n, const T* __restrict__ src, T* __restrict__ x, const int* done) {
    if (done && *done) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] = src[i];
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

// Coefficients of a schedule for one operation (per matrix update).  An
// entry's matrix coefficient A_cj is lower[losort slot] (lp) or, with
// SRC_UPPER, upper[face]: the reference's forward entries are all losort
// slots and its backward ones all owned faces; the multicolour schedules mix
// both.  The pivot products A_cj*A_jc are up*lp per losort slot (up: upper in
// losort order) and upper*lower per owned face (lo: lower by face).
template <class T>
__global__ void pack_k(DevSched s, int op, const T* __restrict__ lp, const T* __restrict__ up,
                       const T* __restrict__ upper, const T* __restrict__ lo, const T* __restrict__ diag,
                       const T* __restrict__ rD, T* __restrict__ coef, T* __restrict__ scalar) {
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
                const bool own = (src & SRC_UPPER) != 0;
                const T a = own ? upper[i] : lp[i];
                if (op == OP_FWD || op == OP_BWD) v = rD[c] * a;
                else if (op == OP_GS) v = a;
                else v = own ? upper[i] * lo[i] : up[i] * lp[i];  // OP_RD: upper*upper (DIC) / upper*lower (DILU)
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

enum Mode { M_CTA = 0, M_CLUSTER_DS = 1, M_CTA_GLOBAL = 2, M_CLUSTER_GLOBAL = 3, M_GRID = 4, M_FLOW = 5, M_LEVELS = 6 };

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
    const size_t xbytes = sizeof(T) * size_t(s.n);
    // few levels: a launch per level, unless the vector fits one CTA's
    // shared memory and the levels are narrow (fewer than 128 slots on
    // average: one CTA walks those faster than a launch per level)
    if (s.levelLaunch && s.nLevels <= g_level_launch &&
        (xbytes > g_smem_cap || int64_t(s.nSlots) >= 128 * int64_t(s.nLevels)))
        return M_LEVELS;
    if (xbytes <= g_smem_cap) return M_CTA;
    const int cs = cluster_of(s);
    if (cs) {
        const int per = (s.n + cs - 1) / cs;
        if (sizeof(T) * size_t(per) <= g_smem_cap) return M_CLUSTER_DS;
    }
    if (s.n <= g_small_threshold) return M_CTA_GLOBAL;
    if (g_cluster && s.n <= g_cluster_global) return M_CLUSTER_GLOBAL;
    // the dataflow form: forced (1), or by default (2) for schedules of at
    // most PF_SMALL entries per slot, where it measured faster than the
    // level counters (the finest hexahedral level; triangular sweeps)
    if (g_flow == 1 || (g_flow == 2 && s.maxK <= PF_SMALL)) return M_FLOW;
    return M_GRID;
}

constexpr int pf_index(int pf) { return pf == PF_SMALL ? 0 : pf == PF_LARGE ? 1 : 2; }

template <class T, int OP, int PF>
cfx_status launch_grid(cudaStream_t st, const DevSched& s, const SweepCtx<T>& a, int* status);

template <class T, int OP, int PF>
cfx_status launch_pf(cudaStream_t st, const DevSched& s, const SweepCtx<T>& a, int* status) {
    if (s.nSlots == 0) return CFX_OK;
    const size_t xbytes = sizeof(T) * size_t(s.n);
    const int cs = cluster_of(s);
    const int per = cs ? (s.n + cs - 1) / cs : 0;
    const int m = mode_of<T>(s);
    if (m == M_LEVELS) {
        const LevelView v{s.cell, s.cnt, s.groupEntry, s.nb};
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        for (int L = 0; L < s.nLevels; ++L) {
            const int g0 = s.hLvlSlot[L] / 32, g1 = s.hLvlSlot[L + 1] / 32;
            const int ctas = (g1 - g0 + LVL_LAUNCH_GROUPS - 1) / LVL_LAUNCH_GROUPS;
            if (ctas == 0) continue;
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(ctas);
            cfg.blockDim = dim3(32 * LVL_LAUNCH_GROUPS);
            cfg.stream = st;
            // the first level follows a kernel that does not signal its
            // dependents early (gather_slots_k): an ordinary launch
            cfg.attrs = L > 0 ? attr : nullptr;
            cfg.numAttrs = L > 0 ? 1 : 0;
            // PF_SMALL entries prefetched (more registers would cost
            // occupancy on the wide levels, which stream from HBM)
            CFX_CUDA(cudaLaunchKernelEx(&cfg, sweep_level_k<T, OP, PF_SMALL>, v, a, g0, g1, s.hLvlPart[L]));
            count_launch();
        }
        return CFX_OK;
    }
    if (m == M_CTA) {
        // FP32: the single CTA holds the larger register set (the next
        // level's entries prefetched, up to PF_GRID_XL per slot); in FP64 that
        // set spills and is slower
        bool xl = false;
        if constexpr (sizeof(T) == 4) {
            if (PF == PF_LARGE && s.maxK > PF_LARGE && g_cta_xl) {
                sweep_cta_k<T, OP, true, PF_GRID_XL><<<1, CTA_NT, xbytes, st>>>(s, a);
                xl = true;
            }
        }
        if (!xl) sweep_cta_k<T, OP, true, PF><<<1, CTA_NT, xbytes, st>>>(s, a);
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
        DevSched g = s;
        g.lvlStride = g_lvl_stride;
        g.pollNs = g_poll_ns;
        CFX_CUDA(cudaMemsetAsync(s.sync, 0, sizeof(int) * (2 + size_t(g.lvlStride) * s.nLevels), st));
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
        CFX_CUDA(cudaLaunchKernelEx(&cfg, sweep_grid_k<T, OP, PF>, g, a, status));
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
    if constexpr (sizeof(T) == 4)
        cudaFuncSetAttribute(sweep_cta_k<T, OP, true, PF_GRID_XL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(g_smem_cap));
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

template <class T, int OP>
void init_flow() {
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, sweep_flow_k<T, OP>, FLOW_NT, 0);
    g_flow_grid[prec_index<T>()][OP] = g_num_sms * (per > 0 ? per : 1);
}

template <class T>
void init_attrs() {
    init_op<T, OP_FWD>();
    init_op<T, OP_BWD>();
    init_op<T, OP_GS>();
    init_op<T, OP_RD>();
    init_flow<T, OP_FWD>();
    init_flow<T, OP_BWD>();
    init_flow<T, OP_GS>();
    init_flow<T, OP_RD>();
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
int sweep_flow() { return g_flow; }
void set_sweep_flow(int mode) { g_flow = mode < 0 ? 0 : (mode > 2 ? 2 : mode); }
int sweep_cta_xl() { return g_cta_xl; }
void set_sweep_cta_xl(int on) { g_cta_xl = on ? 1 : 0; }
int sweep_grid_stride() { return g_lvl_stride; }
void set_sweep_grid_stride(int k) { g_lvl_stride = k < 1 ? 1 : k > LVL_STRIDE_MAX ? LVL_STRIDE_MAX : k; }
int sweep_grid_poll_ns() { return g_poll_ns; }
void set_sweep_grid_poll_ns(int ns) { g_poll_ns = ns < 0 ? 0 : ns; }
int sweep_level_launch() { return g_level_launch; }
void set_sweep_level_launch(int v) { g_level_launch = v < 0 ? 0 : v > LVL_LAUNCH_MAX ? LVL_LAUNCH_MAX : v; }
int sweep_flow_ahead() { return g_flow_ahead; }
void set_sweep_flow_ahead(int k) { g_flow_ahead = k < 1 ? 1 : k; }

// Value buffers a pack of s needs in the dataflow form: the level-ordered
// schedules whose vector does not fit one CTA (FP64), for the sweeps that do
// not write their values straight into x.
size_t sweep_flow_values(const DevSched& s, int op) {
    if (s.n == 0 || sizeof(double) * size_t(s.n) <= g_smem_cap) return 0;
    if (op == OP_FWD || op == OP_RD) return 0;
    return size_t(s.nSweeps > 0 ? s.nSweeps : 1) * size_t(s.n);
}



template <class T>
bool sweep_is_grid(const DevSched& s) {
    return mode_of<T>(s) == M_GRID;
}

template <class T>
int sweep_mode(const DevSched& s) {
    return mode_of<T>(s);
}

template <class T>
int sweep_partials(const DevSched& s) {
    const int m = mode_of<T>(s);
    if (m == M_FLOW) return flow_ctas(prec_index<T>(), OP_BWD, s);
    if (m == M_LEVELS) return std::max(1, s.hLvlPart[s.nLevels]);
    if (m == M_GRID) return g_wave && s.waveOk ? wave_grid<T>(s) : s.nChunks;
    return (m == M_CLUSTER_DS || m == M_CLUSTER_GLOBAL) ? cluster_of(s) : 1;
}

int cluster_global_cells() { return g_cluster_global; }
void set_cluster_global_cells(int n) { g_cluster_global = n; }

// CTAs of a dataflow launch: enough warps for g_flow_ahead levels of the
// schedule's average width (warps further ahead would only spin), at most
// the resident maximum.
inline int flow_ctas(int prec, int op, const DevSched& s) {
    const double perLevel = double(s.nGroups) / double(s.nLevels > 0 ? s.nLevels : 1);
    const int want = int(std::ceil(perLevel * g_flow_ahead / double(FLOW_NT / 32)));
    return std::max(1, std::min(want, g_flow_grid[prec][op]));
}

// The dataflow form of one sweep: fill the value buffers with the sentinel,
// one cooperative launch of every resident CTA, copy the last sweep's
// values into x (Gauss-Seidel and the backward sweeps; the forward and
// pivot sweeps write x directly).
template <class T, int OP>
cfx_status launch_flow(cudaStream_t st, const DevSched& s, const Packed<T>& p, SweepCtx<T> a, int* status) {
    const bool own = OP == OP_FWD || OP == OP_RD;
    T* out = own ? a.x : p.flow;
    if (!out) {
        set_error("dataflow sweep: no value buffer");
        return CFX_ERR_STATE;
    }
    const int64_t nv = own ? int64_t(s.n) : int64_t(s.nSweeps) * s.n;
    const int fb = int(std::min<int64_t>((nv + 255) / 256, 4096));
    flow_fill_k<T><<<fb, 256, 0, st>>>(nv, out, a.done);
    count_launch();
    CFX_CUDA(cudaMemsetAsync(s.sync, 0, sizeof(int) * 2, st));
    const int grid = flow_ctas(prec_index<T>(), OP, s);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid > 0 ? grid : 1);
    cfg.blockDim = dim3(FLOW_NT);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    CFX_CUDA(cudaLaunchKernelEx(&cfg, sweep_flow_k<T, OP>, s, a, out, status));
    count_launch();
    if (!own) {
        const int cb = std::min((s.n + 255) / 256, 4096);
        flow_copy_k<T><<<cb, 256, 0, st>>>(s.n, out + size_t(s.nSweeps - 1) * s.n, a.x, a.done);
        count_launch();
    }
    return CFX_OK;
}

template <class T>
cfx_status run_sweep(cudaStream_t st, const DevSched& s, int op, const Packed<T>& p, const T* in, T* x,
                     const T* dotWith, double* partials, const int* done, int* status) {
    // the right-hand side in slot order (the level-by-level form reads it by
    // cell in its prologue instead)
    if ((op == OP_FWD || op == OP_GS) && s.nSlots > 0 && mode_of<T>(s) != M_LEVELS) {
        int blocks = (s.nSlots + 255) / 256;
        if (blocks > 4096) blocks = 4096;
        gather_slots_k<T><<<blocks, 256, 0, st>>>(s.nSlots, s.cell, in, p.inS, done);
        count_launch();
    }
    SweepCtx<T> a{p.coef, p.scalar, in, p.inS, x, dotWith, partials, done, SWEEP_TIMEOUT_NS};
    if (s.nSlots > 0 && mode_of<T>(s) == M_FLOW) {
        switch (op) {
            case OP_FWD: return launch_flow<T, OP_FWD>(st, s, p, a, status);
            case OP_BWD: return launch_flow<T, OP_BWD>(st, s, p, a, status);
            case OP_GS: return launch_flow<T, OP_GS>(st, s, p, a, status);
            case OP_RD: return launch_flow<T, OP_RD>(st, s, p, a, status);
            default: set_error("unknown sweep"); return CFX_ERR_ARG;
        }
    }
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
    if (s.nLevels < 2 || s.nSlots == 0) {
        set_error("stalled sweep: the schedule needs at least two levels");
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
    const T* lo = c.sym ? c.upper : c.lower;
    const int threads = 256;
    int blocks = (s.nGroups * 32 + threads - 1) / threads;
    if (blocks > 4096) blocks = 4096;
    pack_k<T><<<blocks, threads, 0, st>>>(s, op, c.lowerPerm, up, c.upper, lo, c.diag, c.rD, p.coef, p.scalar);
    count_launch();
    p.valid = true;
}

template bool sweep_is_grid<double>(const DevSched&);
template bool sweep_is_grid<float>(const DevSched&);
template int sweep_partials<double>(const DevSched&);
template int sweep_partials<float>(const DevSched&);
template int sweep_mode<double>(const DevSched&);
template int sweep_mode<float>(const DevSched&);
template cfx_status run_sweep<double>(cudaStream_t, const DevSched&, int, const Packed<double>&, const double*,
                                      double*, const double*, double*, const int*, int*);
template cfx_status run_sweep<float>(cudaStream_t, const DevSched&, int, const Packed<float>&, const float*, float*,
                                     const float*, double*, const int*, int*);
template cfx_status run_sweep_stalled<double>(cudaStream_t, const DevSched&, const Packed<double>&,
                                               const double*, double*, unsigned long long, int*);
template void pack_sweep<double>(cudaStream_t, const DevSched&, int, const LevelCoeffs<double>&, Packed<double>&);
template void pack_sweep<float>(cudaStream_t, const DevSched&, int, const LevelCoeffs<float>&, Packed<float>&);

}  // namespace cfx
