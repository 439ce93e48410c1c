// batch.cu - resident small systems and cfx_batch_*: many independent
// lduMatrix systems solved in one launch, one CTA per system.
//
// A persistent kernel (batch_k) runs nCta = SMs x CTAs-per-SM CTAs; each CTA
// takes the next system from a device counter and runs the reference's whole
// PCG / PBiCGStab loop on it (PCG.C:65-193, PBiCGStab.C:68-254) with block
// barriers between the level-scheduled DIC/DILU sweeps, or FP32 inner solves
// inside FP64 iterative refinement.  Systems are handed out largest first, so
// the long solves start early and the short ones fill the gaps (longest
// processing time first).  The counter reset and the kernel are captured in
// a CUDA graph and replayed while the batch and its controls are unchanged.

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <numeric>

#include "batch.h"

namespace cfx {

namespace {

constexpr size_t ALIGN = 256;

size_t up(size_t b) { return (b + ALIGN - 1) / ALIGN * ALIGN; }

// Bump allocator over one device allocation; also used to size it.
struct Carve {
    char* base;
    size_t off = 0;
    template <class T>
    T* take(size_t n) {
        T* p = reinterpret_cast<T*>(base ? base + off : nullptr);
        off += up(std::max<size_t>(n, 1) * sizeof(T));
        return p;
    }
};

size_t addr_bytes(int n, int wLo, int wUp, int nFwd, int nBwd) {
    Carve c{nullptr};
    c.take<int>(n);                 // cnt
    c.take<int>(size_t(wLo) * n);   // loSrc
    c.take<int>(size_t(wUp) * n);   // upSrc
    c.take<int>(n);                 // cellOf
    c.take<int>(nFwd + 1);
    c.take<int>(n);                 // bwdSlot
    c.take<int>(nBwd + 1);
    return c.off;
}

// The coefficient block: FP64 coefficients, FP32 coefficients (the part
// uploaded), then the work vectors.  Returns the bytes of the uploaded part
// in *coefPart when non-null.
template <bool SET>
size_t coef_layout(BSys& sys, char* base, size_t* coefPart) {
    const size_t n = size_t(sys.n), nl = size_t(sys.wLo) * n, nu = size_t(sys.wUp) * n;
    Carve c{base};
    SlotSys<double>& a = sys.h64;
    SlotSys<float>& e = sys.h32;
    double* diag = c.take<double>(n);
    double* lo = c.take<double>(nl);
    double* upc = c.take<double>(nu);
    double* upLo = sys.sym ? nullptr : c.take<double>(nl);
    float* diag32 = c.take<float>(n);
    float* lo32 = c.take<float>(nl);
    float* up32 = c.take<float>(nu);
    float* upLo32 = sys.sym ? nullptr : c.take<float>(nl);
    if (coefPart) *coefPart = c.off;
    double* rD = c.take<double>(n);
    double *b = c.take<double>(n), *psi = c.take<double>(n);
    double *r = c.take<double>(n), *q = c.take<double>(n), *w = c.take<double>(n), *p = c.take<double>(n);
    double *s = nullptr, *t = nullptr, *r0 = nullptr;
    if (!sys.sym) {
        s = c.take<double>(n);
        t = c.take<double>(n);
        r0 = c.take<double>(n);
    }
    float* rD32 = c.take<float>(n);
    float *b32 = c.take<float>(n), *psi32 = c.take<float>(n);
    float *r32 = c.take<float>(n), *q32 = c.take<float>(n), *w32 = c.take<float>(n), *p32 = c.take<float>(n);
    float *s32 = nullptr, *t32 = nullptr, *r032 = nullptr;
    if (!sys.sym) {
        s32 = c.take<float>(n);
        t32 = c.take<float>(n);
        r032 = c.take<float>(n);
    }
    if (SET) {
        a.diag = diag;
        a.lo = lo;
        a.up = upc;
        a.upLo = upLo;
        a.rD = rD;
        a.b = b;
        a.psi = psi;
        a.r = r;
        a.q = q;
        a.w = w;
        a.p = p;
        a.s = s;
        a.t = t;
        a.r0 = r0;
        e.diag = diag32;
        e.lo = lo32;
        e.up = up32;
        e.upLo = upLo32;
        e.rD = rD32;
        e.b = b32;
        e.psi = psi32;
        e.r = r32;
        e.q = q32;
        e.w = w32;
        e.p = p32;
        e.s = s32;
        e.t = t32;
        e.r0 = r032;
    }
    return c.off;
}

}  // namespace

namespace {

void* bsys_alloc(const BSys& sys, size_t bytes) {
    void* d = nullptr;
    if (sys.pool)
        CK(cudaMallocFromPoolAsync(&d, bytes, sys.pool, sys.poolStream));
    else
        CK(cudaMalloc(&d, bytes));
    return d;
}

void bsys_free(const BSys& sys, void* p) {
    if (!p) return;
    if (sys.pool)
        cudaFreeAsync(p, sys.poolStream);
    else
        cudaFree(p);
}

}  // namespace

BSys::~BSys() {
    bsys_free(*this, dAddr);
    bsys_free(*this, dCoef);
}

size_t bsys_bytes_estimate(int n, int nf, bool sym) {
    BSys tmp;
    tmp.n = n;
    tmp.nf = nf;
    tmp.sym = sym;
    tmp.wLo = tmp.wUp = 3;
    return addr_bytes(n, 3, 3, n, n) + coef_layout<false>(tmp, nullptr, nullptr);
}

cfx_status bsys_create(cudaStream_t s, int n, int nf, const int32_t* l, const int32_t* u, BSys& sys) {
    if (n < 1 || nf < 0) {
        set_error("batch system: need nCells >= 1 and nFaces >= 0");
        return CFX_ERR_ARG;
    }
    HostLevel h;
    CFX_TRY(build_host_level(n, nf, l, u, h, true));
    sys.n = n;
    sys.nf = nf;
    sys.nFwd = int(h.fwdLevelStart.size()) - 1;
    sys.nBwd = int(h.bwdLevelStart.size()) - 1;
    int wLo = 0, wUp = 0;
    for (int c = 0; c < n; ++c) {
        wLo = std::max(wLo, h.losortStart[c + 1] - h.losortStart[c]);
        wUp = std::max(wUp, h.ownerStart[c + 1] - h.ownerStart[c]);
    }
    if (wLo > 0xffff || wUp > 0x7fff) {
        set_error("batch system: a cell with more than 32767 faces");
        return CFX_ERR_ARG;
    }
    sys.wLo = wLo;
    sys.wUp = wUp;
    // slot order = forward level order
    const std::vector<int>& cellOf = h.fwdCells;
    std::vector<int> pos(n);
    for (int p = 0; p < n; ++p) pos[cellOf[p]] = p;
    std::vector<int> cnt(n), loSrc(size_t(wLo) * n), upSrc(size_t(wUp) * n), bwdSlot(n);
    sys.loFace.assign(size_t(wLo) * n, -1);
    sys.upFace.assign(size_t(wUp) * n, -1);
    for (int p = 0; p < n; ++p) {
        const int c = cellOf[p];
        const int nl = h.losortStart[c + 1] - h.losortStart[c];
        const int nu = h.ownerStart[c + 1] - h.ownerStart[c];
        cnt[p] = nl | (nu << 16);
        for (int j = 0; j < wLo; ++j) {
            const size_t k = size_t(j) * n + p;
            if (j < nl) {
                const int slotK = h.losortStart[c] + j;
                loSrc[k] = pos[h.losortL[slotK]];
                sys.loFace[k] = h.losort[slotK];
            } else {
                loSrc[k] = p;
            }
        }
        for (int j = 0; j < wUp; ++j) {
            const size_t k = size_t(j) * n + p;
            if (j < nu) {
                const int f = h.ownerStart[c] + j;
                upSrc[k] = pos[h.u[f]];
                sys.upFace[k] = f;
            } else {
                upSrc[k] = p;
            }
        }
    }
    for (int i = 0; i < n; ++i) bwdSlot[i] = pos[h.bwdCells[i]];
    // backward level L == forward level nFwd-1-L, cells in the same order?
    bool mirror = sys.nBwd == sys.nFwd;
    for (int L = 0; mirror && L < sys.nBwd; ++L) {
        const int fb = h.fwdLevelStart[sys.nFwd - 1 - L], fe = h.fwdLevelStart[sys.nFwd - L];
        const int bb = h.bwdLevelStart[L], be = h.bwdLevelStart[L + 1];
        if (fe - fb != be - bb) {
            mirror = false;
            break;
        }
        for (int i = bb; i < be; ++i)
            if (bwdSlot[i] != fb + (i - bb)) {
                mirror = false;
                break;
            }
    }
    sys.addrBytes = addr_bytes(n, wLo, wUp, sys.nFwd, sys.nBwd);
    std::vector<char> img(sys.addrBytes, 0);
    Carve hc{img.data()};
    Carve dc{nullptr};
    sys.dAddr = static_cast<char*>(bsys_alloc(sys, sys.addrBytes));
    dc.base = sys.dAddr;
    auto put = [&](const std::vector<int>& v, size_t count) -> const int* {
        int* hp = hc.take<int>(count);
        int* dp = dc.take<int>(count);
        if (!v.empty()) std::memcpy(hp, v.data(), std::min(v.size(), count) * sizeof(int));
        return dp;
    };
    SlotSys<double>& a = sys.h64;
    a.n = n;
    a.wLo = wLo;
    a.wUp = wUp;
    a.nFwd = sys.nFwd;
    a.nBwd = sys.nBwd;
    a.bwdMirror = mirror;
    a.cnt = put(cnt, n);
    a.loSrc = put(loSrc, size_t(wLo) * n);
    a.upSrc = put(upSrc, size_t(wUp) * n);
    a.cellOf = put(cellOf, n);
    a.fwdLevelStart = put(h.fwdLevelStart, sys.nFwd + 1);
    a.bwdSlot = put(bwdSlot, n);
    a.bwdLevelStart = put(h.bwdLevelStart, sys.nBwd + 1);
    SlotSys<float>& e = sys.h32;
    e.n = n;
    e.wLo = wLo;
    e.wUp = wUp;
    e.nFwd = a.nFwd;
    e.nBwd = a.nBwd;
    e.bwdMirror = a.bwdMirror;
    e.cnt = a.cnt;
    e.loSrc = a.loSrc;
    e.upSrc = a.upSrc;
    e.cellOf = a.cellOf;
    e.fwdLevelStart = a.fwdLevelStart;
    e.bwdSlot = a.bwdSlot;
    e.bwdLevelStart = a.bwdLevelStart;
    CK(cudaMemcpyAsync(sys.dAddr, img.data(), sys.addrBytes, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
    sys.cellOf = cellOf;
    return CFX_OK;
}

void bsys_set_coeffs(cudaStream_t s, BSys& sys, const double* diag, const double* upper, const double* lower) {
    if (!diag || (sys.nf > 0 && !upper)) throw std::invalid_argument("batch system: null coefficients");
    const bool sym = lower == nullptr;
    if (sys.dCoef && sys.sym != sym) {
        CK(cudaStreamSynchronize(s));
        bsys_free(sys, sys.dCoef);
        sys.dCoef = nullptr;
    }
    sys.sym = sym;
    size_t part = 0;
    if (!sys.dCoef) {
        sys.coefBytes = coef_layout<false>(sys, nullptr, nullptr);
        sys.dCoef = static_cast<char*>(bsys_alloc(sys, sys.coefBytes));
    }
    coef_layout<true>(sys, sys.dCoef, &part);
    // host image of the uploaded part, in the device layout
    const size_t n = size_t(sys.n), nl = size_t(sys.wLo) * n, nu = size_t(sys.wUp) * n;
    std::vector<char> img(part, 0);
    Carve c{img.data()};
    double* d64 = c.take<double>(n);
    double* l64 = c.take<double>(nl);
    double* u64 = c.take<double>(nu);
    double* ul64 = sym ? nullptr : c.take<double>(nl);
    float* d32 = c.take<float>(n);
    float* l32 = c.take<float>(nl);
    float* u32 = c.take<float>(nu);
    float* ul32 = sym ? nullptr : c.take<float>(nl);
    const double* lo = sym ? upper : lower;
    for (size_t p = 0; p < n; ++p) {
        d64[p] = diag[sys.cellOf[p]];
        d32[p] = float(d64[p]);
    }
    for (size_t k = 0; k < nl; ++k) {
        const int f = sys.loFace[k];
        l64[k] = f >= 0 ? lo[f] : 0.0;
        l32[k] = float(l64[k]);
        if (!sym) {
            ul64[k] = f >= 0 ? upper[f] : 0.0;
            ul32[k] = float(ul64[k]);
        }
    }
    for (size_t k = 0; k < nu; ++k) {
        const int f = sys.upFace[k];
        u64[k] = f >= 0 ? upper[f] : 0.0;
        u32[k] = float(u64[k]);
    }
    CK(cudaMemcpyAsync(sys.dCoef, img.data(), part, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
    sys.hasCoeffs = true;
}

const char* bsys_solver_name(const cfx_controls& c) {
    static const char* pcg[] = {"nonePCG", "diagonalPCG", "DICPCG", "DILUPCG"};
    static const char* bicg[] = {"nonePBiCGStab", "diagonalPBiCGStab", "DICPBiCGStab", "DILUPBiCGStab"};
    return c.solver == CFX_SOLVER_PCG ? pcg[c.preconditioner] : bicg[c.preconditioner];
}

cfx_status bsys_check_controls(const cfx_controls* c, bool sym) {
    if (!c) {
        set_error("null controls");
        return CFX_ERR_ARG;
    }
    if ((c->solver != CFX_SOLVER_PCG && c->solver != CFX_SOLVER_PBICGSTAB) || c->preconditioner < 0 ||
        c->preconditioner > 3 || (c->precision != CFX_FP64 && c->precision != CFX_MIXED)) {
        set_error("batched solves take cudaPCG or cudaPBiCGStab with a known preconditioner and precision");
        return CFX_ERR_CONFIG;
    }
    // registrations as lduMatrix::solver::New / preconditioner::New
    // (PCG.C:30-36, DICPreconditioner.C:33-36, DILUPreconditioner.C:33-36)
    if (c->solver == CFX_SOLVER_PCG && !sym) {
        set_error("Unknown asymmetric matrix solver cudaPCG");
        return CFX_ERR_CONFIG;
    }
    if (c->preconditioner == CFX_PRE_DIC && !sym) {
        set_error("Unknown asymmetric matrix preconditioner DIC");
        return CFX_ERR_CONFIG;
    }
    if (c->preconditioner == CFX_PRE_DILU && sym) {
        set_error("Unknown symmetric matrix preconditioner DILU");
        return CFX_ERR_CONFIG;
    }
    return CFX_OK;
}

void bsys_records(const BSys& sys, const cfx_controls& c, double* psi, const double* b, SlotSys<double>& r64,
                  SlotSys<float>& r32) {
    r64 = sys.h64;
    r32 = sys.h32;
    r64.bCell = b;
    r64.psiCell = psi;
    r64.tolerance = c.tolerance;
    r64.relTol = c.relTol;
    r64.maxIter = c.maxIter;
    r64.minIter = c.minIter;
    r64.precond = c.preconditioner;
    r64.solver = c.solver;
    if (c.solver == CFX_SOLVER_PCG) {
        r64.s = r64.t = r64.r0 = nullptr;
        r32.s = r32.t = r32.r0 = nullptr;
    }
    r32.maxIter = c.maxIter;
    r32.minIter = 0;
    r32.precond = c.preconditioner;
    r32.solver = c.solver;
    r32.tolerance = 0.0;
    r32.relTol = 0.0;  // set by the kernel
}

}  // namespace cfx

// ------------------------------------------------------------------ batches
namespace cfx {
namespace {
int g_inner_digits = 3;  // FP32 inner solves reduce the residual by 10^-digits
}
void batch_set_inner_digits(int d) { g_inner_digits = d; }
int batch_inner_digits() { return g_inner_digits; }
}  // namespace cfx

struct cfx_batch {
    cfx_ctx* ctx = nullptr;
    std::vector<std::unique_ptr<BSys>> sys;   // creation order
    std::vector<int64_t> offset;              // cell offsets, creation order [nSys+1]
    std::vector<int> order;                   // launch slot -> system (largest first)
    Arena arena;
    double *d_psi = nullptr, *d_src = nullptr, *d_save = nullptr;
    SlotSys<double>* d64 = nullptr;
    SlotSys<float>* d32 = nullptr;
    SlotSys<double>* h64 = nullptr;          // pinned
    SlotSys<float>* h32 = nullptr;           // pinned
    unsigned* d_next = nullptr;
    GraphCache graph;
    uint64_t recKey = 0;
    bool dirty = true;
    int sms = 0, ctasPerSm = 0;
    int clusterSize = 0, nBig = 0;            // cluster form: the nBig largest systems per cluster
    std::map<int, int> maxClusters;           // co-resident clusters per cluster size
    ~cfx_batch() {
        if (h64) cudaFreeHost(h64);
        if (h32) cudaFreeHost(h32);
    }
};

namespace {

uint64_t mix(uint64_t h, uint64_t x) { return (h ^ x) * 1099511628211ull; }

uint64_t dbits(double d) {
    uint64_t b;
    std::memcpy(&b, &d, sizeof(b));
    return b;
}

int batch_ctas(cfx_batch* bt) {
    const int occ = batch_ctas_per_sm();
    const int k = bt->ctasPerSm > 0 ? std::min(bt->ctasPerSm, occ) : occ;
    return std::max(1, std::min<int>(bt->sms * k, int(bt->sys.size())));
}

cfx_status batch_check(cfx_batch* bt, const cfx_controls* ctl) {
    for (size_t i = 0; i < bt->sys.size(); ++i) {
        if (!bt->sys[i]->hasCoeffs) {
            set_error("cfx_batch: system " + std::to_string(i) + " has no coefficients");
            return CFX_ERR_STATE;
        }
        CFX_TRY(bsys_check_controls(ctl, bt->sys[i]->sym));
    }
    return CFX_OK;
}

// Enqueues one batch solve on the context stream (records uploaded when the
// controls or the systems changed); the caller reads the results.
void batch_enqueue(cfx_batch* bt, const cfx_controls& c) {
    cudaStream_t s = bt->ctx->stream;
    const int nSys = int(bt->sys.size());
    const int mixed = c.precision == CFX_MIXED;
    const double innerRelTol = std::pow(10.0, -double(batch_inner_digits()));
    uint64_t key = 1469598103934665603ull;
    for (uint64_t x : {uint64_t(c.solver), uint64_t(c.preconditioner), dbits(c.tolerance), dbits(c.relTol),
                       uint64_t(c.maxIter), uint64_t(c.minIter), uint64_t(mixed)})
        key = mix(key, x);
    if (bt->dirty || key != bt->recKey) {
        for (int j = 0; j < nSys; ++j) {
            const int i = bt->order[j];
            bsys_records(*bt->sys[i], c, bt->d_psi + bt->offset[i], bt->d_src + bt->offset[i], bt->h64[j],
                         bt->h32[j]);
        }
        CK(cudaMemcpyAsync(bt->d64, bt->h64, sizeof(SlotSys<double>) * nSys, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(bt->d32, bt->h32, sizeof(SlotSys<float>) * nSys, cudaMemcpyHostToDevice, s));
        CK(cudaStreamSynchronize(s));
        bt->recKey = key;
        bt->dirty = false;
    }
    const int nCta = batch_ctas(bt);
    int cs = 0, nClusters = 0;
    const int nBig = std::min(bt->nBig, nSys);
    if (bt->clusterSize > 1 && nBig > 0) {
        auto it = bt->maxClusters.find(bt->clusterSize);
        if (it == bt->maxClusters.end())
            it = bt->maxClusters.emplace(bt->clusterSize, batch_max_clusters(bt->clusterSize)).first;
        if (it->second > 0) {
            cs = bt->clusterSize;
            nClusters = it->second;
        }
    }
    const uint64_t gkey = mix(mix(mix(mix(mix(key, uint64_t(nCta)), dbits(innerRelTol)), uint64_t(nSys)), uint64_t(cs)),
                              uint64_t(cs ? nBig : 0));
    graph_launch(bt->graph, gkey, s, [&]() {
        CK(cudaMemsetAsync(bt->d_next, 0, 2 * sizeof(unsigned), s));
        if (cs)
            CK(launch_batch_cluster(s, bt->d64, mixed ? bt->d32 : nullptr, nSys, nBig, cs, nClusters, mixed,
                                    innerRelTol, 50, bt->d_next));
        else
            launch_batch(s, bt->d64, mixed ? bt->d32 : nullptr, nSys, nCta, mixed, innerRelTol, 50, bt->d_next);
    });
}

void batch_results(cfx_batch* bt, const cfx_controls& c, cfx_perf* perf) {
    cudaStream_t s = bt->ctx->stream;
    const int nSys = int(bt->sys.size());
    CK(cudaMemcpyAsync(bt->h64, bt->d64, sizeof(SlotSys<double>) * nSys, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (!perf) return;
    for (int j = 0; j < nSys; ++j) {
        const SlotSys<double>& r = bt->h64[j];
        cfx_perf& p = perf[bt->order[j]];
        std::memset(&p, 0, sizeof(p));
        std::snprintf(p.solverName, sizeof(p.solverName), "%s", bsys_solver_name(c));
        p.initialResidual = r.initialResidual;
        p.finalResidual = r.finalResidual;
        p.nIterations = r.nIterations;
        p.converged = r.converged;
        p.singular = r.singular;
        p.status = CFX_OK;
        p.nOuter = c.precision == CFX_MIXED ? r.nOuter : 0;
    }
}

}  // namespace

// ===================================================================== C ABI
extern "C" {

cfx_status cfx_batch_create(cfx_ctx* ctx, int nSystems, const int32_t* nCells, const int32_t* nFaces,
                            const int32_t* const* l, const int32_t* const* u, cfx_batch** out) {
    if (!ctx || !out || nSystems < 1 || !nCells || !nFaces || !l || !u) {
        set_error("cfx_batch_create: bad argument");
        return CFX_ERR_ARG;
    }
    return guard([&]() -> cfx_status {
        auto bt = std::make_unique<cfx_batch>();
        bt->ctx = ctx;
        CK(cudaDeviceGetAttribute(&bt->sms, cudaDevAttrMultiProcessorCount, ctx->device));
        bt->offset.assign(1, 0);
        for (int i = 0; i < nSystems; ++i) {
            auto sy = std::make_unique<BSys>();
            const cfx_status st = bsys_create(ctx->stream, nCells[i], nFaces[i], l[i], u[i], *sy);
            if (st != CFX_OK) {
                set_error("cfx_batch_create: system " + std::to_string(i) + ": " + last_error());
                return st;
            }
            bt->offset.push_back(bt->offset.back() + nCells[i]);
            bt->sys.push_back(std::move(sy));
        }
        bt->order.resize(nSystems);
        std::iota(bt->order.begin(), bt->order.end(), 0);
        // largest first (work per solve grows faster than the cell count)
        std::stable_sort(bt->order.begin(), bt->order.end(), [&](int a, int b) {
            const BSys &x = *bt->sys[a], &y = *bt->sys[b];
            return int64_t(x.n) + x.nf > int64_t(y.n) + y.nf;
        });
        const int64_t N = bt->offset.back();
        bt->d_psi = bt->arena.get<double>(N);
        bt->d_src = bt->arena.get<double>(N);
        CK(cudaMemsetAsync(bt->d_psi, 0, sizeof(double) * N, ctx->stream));
        CK(cudaMemsetAsync(bt->d_src, 0, sizeof(double) * N, ctx->stream));
        bt->d64 = bt->arena.get<SlotSys<double>>(nSystems);
        bt->d32 = bt->arena.get<SlotSys<float>>(nSystems);
        bt->d_next = bt->arena.get<unsigned>(2);
        CK(cudaMallocHost(&bt->h64, sizeof(SlotSys<double>) * nSystems));
        CK(cudaMallocHost(&bt->h32, sizeof(SlotSys<float>) * nSystems));
        CK(cudaStreamSynchronize(ctx->stream));
        ctx_retain(ctx);
        *out = bt.release();
        return CFX_OK;
    });
}

cfx_status cfx_batch_destroy(cfx_batch* bt) {
    if (!bt) return CFX_ERR_ARG;
    cfx_ctx* ctx = bt->ctx;  // alive: the batch holds a reference
    cudaStreamSynchronize(ctx->stream);
    delete bt;
    ctx_release(ctx);
    return CFX_OK;
}

cfx_status cfx_batch_set_matrix(cfx_batch* bt, int i, const double* diag, const double* upper, const double* lower) {
    if (!bt || i < 0 || i >= int(bt->sys.size()) || !diag || !upper) {
        set_error("cfx_batch_set_matrix: bad argument");
        return CFX_ERR_ARG;
    }
    return guard([&]() -> cfx_status {
        bsys_set_coeffs(bt->ctx->stream, *bt->sys[i], diag, upper, lower);
        bt->dirty = true;
        return CFX_OK;
    });
}

cfx_status cfx_batch_vectors(cfx_batch* bt, double** d_psi, double** d_source, int64_t* offsets) {
    if (!bt) return CFX_ERR_ARG;
    if (d_psi) *d_psi = bt->d_psi;
    if (d_source) *d_source = bt->d_src;
    if (offsets) std::copy(bt->offset.begin(), bt->offset.end(), offsets);
    return CFX_OK;
}

cfx_status cfx_batch_solve_device(cfx_batch* bt, const cfx_controls* ctl, cfx_perf* perf) {
    if (!bt) return CFX_ERR_ARG;
    CFX_TRY(batch_check(bt, ctl));
    return guard([&]() -> cfx_status {
        after_caller(bt->ctx);  // the caller may have filled the vectors on its stream
        batch_enqueue(bt, *ctl);
        batch_results(bt, *ctl, perf);
        return CFX_OK;
    });
}

cfx_status cfx_batch_solve(cfx_batch* bt, const cfx_controls* ctl, double* psi, const double* source,
                           cfx_perf* perf) {
    if (!bt || !psi || !source) {
        set_error("cfx_batch_solve: bad argument");
        return CFX_ERR_ARG;
    }
    CFX_TRY(batch_check(bt, ctl));
    return guard([&]() -> cfx_status {
        cudaStream_t s = bt->ctx->stream;
        const size_t bytes = sizeof(double) * size_t(bt->offset.back());
        CK(cudaMemcpyAsync(bt->d_psi, psi, bytes, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(bt->d_src, source, bytes, cudaMemcpyHostToDevice, s));
        batch_enqueue(bt, *ctl);
        CK(cudaMemcpyAsync(psi, bt->d_psi, bytes, cudaMemcpyDeviceToHost, s));
        batch_results(bt, *ctl, perf);
        return CFX_OK;
    });
}

cfx_status cfx_batch_timings(cfx_batch* bt, double* startMs, double* endMs) {
    if (!bt || !startMs || !endMs) return CFX_ERR_ARG;
    const int nSys = int(bt->sys.size());
    unsigned long long t0 = ~0ull;
    for (int j = 0; j < nSys; ++j) t0 = std::min(t0, bt->h64[j].tStart);
    for (int j = 0; j < nSys; ++j) {
        const int i = bt->order[j];
        startMs[i] = double(bt->h64[j].tStart - t0) * 1e-6;
        endMs[i] = double(bt->h64[j].tEnd - t0) * 1e-6;
    }
    return CFX_OK;
}

cfx_status cfx_batch_set_ctas_per_sm(cfx_batch* bt, int k) {
    if (!bt || k < 0) return CFX_ERR_ARG;
    bt->ctasPerSm = k;
    return CFX_OK;
}

cfx_status cfx_batch_set_groups(cfx_batch* bt, int clusterSize, int bigCells) {
    if (!bt || clusterSize < 0 || clusterSize > 16 || bigCells < 0) return CFX_ERR_ARG;
    bt->clusterSize = clusterSize;
    int nBig = 0;
    for (int j = 0; j < int(bt->order.size()); ++j)
        if (clusterSize > 1 && bt->sys[bt->order[j]]->n >= bigCells) nBig = j + 1;
    bt->nBig = nBig;
    return CFX_OK;
}

cfx_status cfx_batch_tune(cfx_batch* bt, const cfx_controls* ctl, int* best, float* bestMs) {
    if (!bt) return CFX_ERR_ARG;
    CFX_TRY(batch_check(bt, ctl));
    return guard([&]() -> cfx_status {
        cudaStream_t s = bt->ctx->stream;
        const int nSys = int(bt->sys.size());
        const size_t N = size_t(bt->offset.back());
        if (!bt->d_save) bt->d_save = bt->arena.get<double>(N);
        CK(cudaMemcpyAsync(bt->d_save, bt->d_psi, sizeof(double) * N, cudaMemcpyDeviceToDevice, s));
        cudaEvent_t e0, e1;
        CK(cudaEventCreate(&e0));
        CK(cudaEventCreate(&e1));
        auto trial = [&]() {
            CK(cudaMemcpyAsync(bt->d_psi, bt->d_save, sizeof(double) * N, cudaMemcpyDeviceToDevice, s));
            CK(cudaEventRecord(e0, s));
            batch_enqueue(bt, *ctl);
            CK(cudaEventRecord(e1, s));
            CK(cudaEventSynchronize(e1));
            float ms = 0.0f;
            CK(cudaEventElapsedTime(&ms, e0, e1));
            return ms;
        };
        // 1. one CTA per system, as many CTAs as fit
        const int occ = batch_ctas_per_sm();
        bt->ctasPerSm = occ;
        bt->clusterSize = 0;
        bt->nBig = 0;
        float bms = trial();
        int bcs = 0, bnb = 0;
        // 2. the systems whose single-CTA solve outlasts the balanced share
        //    of the whole batch (sum of solve times / CTAs) go to clusters
        CK(cudaMemcpyAsync(bt->h64, bt->d64, sizeof(SlotSys<double>) * nSys, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        double total = 0.0;
        for (int j = 0; j < nSys; ++j) total += double(bt->h64[j].tEnd - bt->h64[j].tStart);
        const double share = total / double(batch_ctas(bt));
        int nBig = 0;
        for (int j = 0; j < nSys; ++j)
            if (double(bt->h64[j].tEnd - bt->h64[j].tStart) > 0.5 * share) nBig = j + 1;
        if (nBig > 0) {
            for (int cs : {4, 8, 16}) {
                bt->clusterSize = cs;
                bt->nBig = nBig;
                if (batch_max_clusters(cs) <= 0) continue;
                const float ms = trial();
                if (ms < bms) {
                    bms = ms;
                    bcs = cs;
                    bnb = nBig;
                }
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        bt->clusterSize = bcs;
        bt->nBig = bnb;
        CK(cudaMemcpyAsync(bt->d_psi, bt->d_save, sizeof(double) * N, cudaMemcpyDeviceToDevice, s));
        CK(cudaStreamSynchronize(s));
        if (best) *best = bcs;
        if (bestMs) *bestMs = bms;
        return CFX_OK;
    });
}

cfx_status cfx_batch_get_groups(cfx_batch* bt, int* clusterSize, int* nBig, int* ctasPerSm) {
    if (!bt) return CFX_ERR_ARG;
    if (clusterSize) *clusterSize = bt->clusterSize;
    if (nBig) *nBig = bt->nBig;
    if (ctasPerSm) *ctasPerSm = bt->ctasPerSm;
    return CFX_OK;
}

}  // extern "C"
