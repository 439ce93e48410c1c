// server.cu - the solve server (cfx_server_*): an in-process component that
// keeps matrices resident in HBM and serves solve requests from any number of
// client threads with continuous batching.
//
//   * Matrices are registered once (cfx_server_add_matrix) and stay resident
//     until removed: small ones as slot-ordered batch systems, large ones
//     (more than largeCells cells) as a cfx_mesh + cfx_matrix with their GAMG
//     hierarchy.  A request names a matrix and brings a new right-hand side
//     (and initial psi), so re-solving a resident matrix (a PISO corrector)
//     uploads two vectors only.
//   * Admission: every resident matrix and every request's device vectors
//     count against an HBM budget.  A matrix or request that alone exceeds
//     the budget is refused (CFX_ERR_ADMISSION); one that does not fit now
//     waits (the submitting thread blocks) until completions free space.
//   * Batch lanes and a large worker share the GPU.  A lane (a thread with
//     its own stream and launch buffers) takes the queued small requests of
//     the oldest one's precision and size class (cluster-sized systems or
//     one-CTA systems), at most one per matrix, up to maxBatch, and solves
//     them in one persistent launch, one CTA or one thread-block cluster per
//     system.  Lanes run concurrently: the batch kernels never wait on each
//     other (each CTA or cluster finishes its systems alone), so a request
//     that arrives while a long launch runs starts at once on an idle lane
//     on the SMs that launch leaves free, and one-CTA systems never wait for
//     a cluster-sized one launched with them.  The large worker runs large
//     requests one at a time through the whole-GPU drivers on its own
//     context.  Those launch cooperative grids that must have the device to
//     themselves, so large kernels and batch kernels never run at the same
//     time: a large solve starts once the lanes are idle (lanes start
//     nothing new once a large request has waited 100 ms), and yields
//     between its V-cycles (or
//     batches of Krylov iterations) whenever small requests are waiting:
//     the idle lanes start launches in that gap, the gap closes when the
//     first of them finishes, and the large solve resumes when all have.  A
//     small request waits at most one cycle of a large solve, not all of it.
//   * Completion is signalled per request; a request can be cancelled while
//     it is queued (or its result dropped later), and requests whose client
//     never collects them are freed at release or shutdown.
// Latency (submit to completion) and throughput counters are kept for
// cfx_server_stats.

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>

#include "batch.h"

using namespace cfx;

namespace {

using Clock = std::chrono::steady_clock;

enum ReqState { Q_WAITING = 0, Q_RUNNING = 1, Q_DONE = 2, Q_CANCELLED = 3, Q_FAILED = 4 };

struct SrvMatrix {
    int64_t id = 0;
    int n = 0, nf = 0;
    bool large = false, sym = true;
    std::unique_ptr<BSys> bs;
    cfx_mesh* mesh = nullptr;
    cfx_matrix* mat = nullptr;
    size_t bytes = 0;
    bool busy = false;      // a request on it is running
    bool removing = false;  // remove requested; freed when idle
    int pending = 0;        // queued or running requests
};

struct SrvRequest {
    int64_t id = 0, matrixId = 0;
    cfx_controls ctl{};
    double *d_psi = nullptr, *d_b = nullptr;
    size_t bytes = 0;
    int n = 0;
    ReqState state = Q_WAITING;
    bool detached = false;  // released by its client: freed when it completes
    cfx_status status = CFX_OK;
    std::string error;
    cfx_perf perf{};
    Clock::time_point tSubmit, tStart, tDone;
};

}  // namespace

// A batch lane: one launch at a time on its own stream.
struct SrvLane {
    cudaStream_t stream = nullptr;
    SlotSys<double>* d64 = nullptr;
    SlotSys<float>* d32 = nullptr;
    SlotSys<double>* h64 = nullptr;
    SlotSys<float>* h32 = nullptr;
    BatchDone* hDone = nullptr;  // host-mapped per-system results ...
    BatchDone* dDone = nullptr;  // ... and the kernels' view of them
    unsigned* d_next = nullptr;
    int cap = 0;
    std::thread th;
};

struct cfx_server {
    cfx_ctx* ctx = nullptr;           // the device; batch lanes have their own streams
    cfx_ctx* ctxLarge = nullptr;      // large matrices: their uploads and solves
    cudaStream_t copyStream = nullptr;  // request vectors and small-matrix uploads
    cudaMemPool_t pool = nullptr;       // their device memory, stream-ordered on copyStream
    cfx_server_config cfg{};
    int sms = 0;
    int clusterMax = 0;  // clusters of cfg.groupSize CTAs resident at once (0: no cluster form)
    std::mutex mu;
    std::condition_variable cvWork;   // worker: something to do
    std::condition_variable cvDone;   // clients: a request finished / space freed
    std::map<int64_t, std::unique_ptr<SrvMatrix>> mats;
    std::map<int64_t, std::unique_ptr<SrvRequest>> reqs;
    std::deque<int64_t> queue;        // waiting requests, arrival order
    int64_t nextMat = 1, nextReq = 1;
    size_t used = 0;                  // bytes admitted (matrices + request vectors)
    bool stop = false;
    std::vector<std::unique_ptr<SrvLane>> lanes;  // batches of small requests
    std::thread largeWorker;                       // large requests
    // (mu held) activeLanes: lanes running a launch; largeActive: a large
    // solve is in progress (possibly yielding); yieldOpen: it has yielded
    // and lanes may start; batchGen counts finished launches
    int activeLanes = 0;
    bool largeActive = false, yieldOpen = false;
    int64_t batchGen = 0, yields = 0;
    // statistics
    Clock::time_point t0;
    int64_t submitted = 0, completed = 0, cancelled = 0, failed = 0, refused = 0;
    int64_t batches = 0, batchedSolves = 0, largeSolves = 0, running = 0;
    std::vector<double> latMs, queueMs, runMs;  // submit-to-done, submit-to-start, start-to-done
};

namespace {

size_t large_estimate(int n, int nf) {
    // fine level + GAMG hierarchy (< the fine level again), FP64 and FP32
    // coefficients, the sliced ELL rows (about 2.3 entries a face of column,
    // source and both coefficient copies), schedules and work vectors
    return size_t(n) * 420 + size_t(nf) * 150 + (size_t(64) << 20);
}

void finish(cfx_server* sv, SrvRequest& r, ReqState st) {
    const bool ran = r.state == Q_RUNNING;
    r.state = st;
    r.tDone = Clock::now();
    if (st == Q_DONE) {
        ++sv->completed;
        sv->latMs.push_back(std::chrono::duration<double, std::milli>(r.tDone - r.tSubmit).count());
        sv->queueMs.push_back(std::chrono::duration<double, std::milli>(r.tStart - r.tSubmit).count());
        sv->runMs.push_back(std::chrono::duration<double, std::milli>(r.tDone - r.tStart).count());
    } else if (st == Q_FAILED) {
        ++sv->failed;
    }
    auto m = sv->mats.find(r.matrixId);
    if (m != sv->mats.end()) {
        // only the running request holds its matrix: cancelling a queued one
        // must not free the matrix for a second launch while one runs on it
        if (ran) m->second->busy = false;
        m->second->pending--;
    }
}

void free_request_buffers(cfx_server* sv, SrvRequest& r) {
    if (r.d_psi) cudaFreeAsync(r.d_psi, sv->copyStream);
    if (r.d_b) cudaFreeAsync(r.d_b, sv->copyStream);
    r.d_psi = r.d_b = nullptr;
    sv->used -= r.bytes;
    r.bytes = 0;
}

// Drops finished requests that no client will collect.
void drop_detached(cfx_server* sv) {
    for (auto it = sv->reqs.begin(); it != sv->reqs.end();) {
        SrvRequest& r = *it->second;
        if (r.detached && r.state != Q_WAITING && r.state != Q_RUNNING) {
            free_request_buffers(sv, r);
            it = sv->reqs.erase(it);
        } else {
            ++it;
        }
    }
}

void free_matrix(cfx_server* sv, SrvMatrix& m) {
    if (m.mat) cfx_matrix_destroy(m.mat);
    if (m.mesh) cfx_mesh_destroy(m.mesh);
    m.mat = nullptr;
    m.mesh = nullptr;
    m.bs.reset();
    sv->used -= m.bytes;
}

// Matrices whose removal was requested go once no request uses them.
void reap(cfx_server* sv) {
    for (auto it = sv->mats.begin(); it != sv->mats.end();) {
        if (it->second->removing && it->second->pending == 0) {
            free_matrix(sv, *it->second);
            it = sv->mats.erase(it);
        } else {
            ++it;
        }
    }
}

void ensure_cap(SrvLane& ln, int k) {
    if (k <= ln.cap) return;
    const int c = std::max(k, 2 * ln.cap);
    if (ln.d64) cudaFree(ln.d64);
    if (ln.d32) cudaFree(ln.d32);
    if (ln.h64) cudaFreeHost(ln.h64);
    if (ln.h32) cudaFreeHost(ln.h32);
    if (ln.hDone) cudaFreeHost(ln.hDone);
    ln.d64 = nullptr;
    ln.d32 = nullptr;
    ln.h64 = nullptr;
    ln.h32 = nullptr;
    ln.hDone = ln.dDone = nullptr;
    ln.cap = 0;
    CK(cudaMalloc(&ln.d64, sizeof(SlotSys<double>) * c));
    CK(cudaMalloc(&ln.d32, sizeof(SlotSys<float>) * c));
    CK(cudaMallocHost(&ln.h64, sizeof(SlotSys<double>) * c));
    CK(cudaMallocHost(&ln.h32, sizeof(SlotSys<float>) * c));
    CK(cudaHostAlloc(reinterpret_cast<void**>(&ln.hDone), sizeof(BatchDone) * c, cudaHostAllocMapped));
    CK(cudaHostGetDevicePointer(reinterpret_cast<void**>(&ln.dDone), ln.hDone, 0));
    ln.cap = c;
}

// A small matrix's size class: solved by a cluster of groupSize CTAs (1) or
// by one CTA (0), by its size alone, so that a request's result does not
// depend on what else is in the launch.
int size_class(const cfx_server* sv, const SrvMatrix& m) {
    return sv->cfg.groupSize > 1 && sv->clusterMax > 0 && m.n >= sv->cfg.groupCells;
}

// Runs one batch of small requests of one size class on a lane (lane
// thread, lock not held), largest first.  Each system's result is published
// by the kernel the moment it finishes (BatchDone in host-mapped memory):
// the lane polls the flags while the launch runs and hands every finished
// request to complete() at once, so a small system does not wait for the
// largest of its launch.  done[i] marks the requests handed over.
template <class Complete>
void run_batch(cfx_server* sv, SrvLane& ln, std::vector<SrvRequest*>& rs, std::vector<SrvMatrix*>& ms,
               std::vector<char>& done, Complete&& complete) {
    const int k = int(rs.size());
    std::vector<int> order(k);
    for (int i = 0; i < k; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return ms[a]->n > ms[b]->n; });
    ensure_cap(ln, k);
    int mixed = 0;
    for (int j = 0; j < k; ++j) {
        const int i = order[j];
        bsys_records(*ms[i]->bs, rs[i]->ctl, rs[i]->d_psi, rs[i]->d_b, ln.h64[j], ln.h32[j]);
        mixed |= rs[i]->ctl.precision == CFX_MIXED;
    }
    std::memset(ln.hDone, 0, sizeof(BatchDone) * k);
    cudaStream_t s = ln.stream;
    CK(cudaMemcpyAsync(ln.d64, ln.h64, sizeof(SlotSys<double>) * k, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(ln.d32, ln.h32, sizeof(SlotSys<float>) * k, cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(ln.d_next, 0, 2 * sizeof(unsigned), s));
    const bool clusters = size_class(sv, *ms[0]);
    const double innerRelTol = std::pow(10.0, -double(batch_inner_digits()));
    // a mixed launch solves every system of it in mixed precision; a lane
    // only batches requests of one precision together
    if (clusters)
        CK(launch_batch_cluster(s, ln.d64, mixed ? ln.d32 : nullptr, k, k, sv->cfg.groupSize, sv->clusterMax, mixed,
                                innerRelTol, 50, ln.d_next, ln.dDone));
    else
        launch_batch(s, ln.d64, mixed ? ln.d32 : nullptr, k, std::min(k, sv->sms * batch_ctas_per_sm()), mixed,
                     innerRelTol, 50, ln.d_next, ln.dDone);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(ln.h64, ln.d64, sizeof(SlotSys<double>) * k, cudaMemcpyDeviceToHost, s));
    auto set_perf = [&](int j, double ini, double fin, int it, int conv, int sing, int outer) {
        SrvRequest& q = *rs[order[j]];
        std::memset(&q.perf, 0, sizeof(q.perf));
        std::snprintf(q.perf.solverName, sizeof(q.perf.solverName), "%s", bsys_solver_name(q.ctl));
        q.perf.initialResidual = ini;
        q.perf.finalResidual = fin;
        q.perf.nIterations = it;
        q.perf.converged = conv;
        q.perf.singular = sing;
        q.perf.nOuter = mixed ? outer : 0;
    };
    std::vector<SrvRequest*> now;
    int left = k;
    for (;;) {
        now.clear();
        for (int j = 0; j < k; ++j) {
            if (done[order[j]] || !__atomic_load_n(&ln.hDone[j].flag, __ATOMIC_ACQUIRE)) continue;
            const BatchDone& d = ln.hDone[j];
            set_perf(j, d.initialResidual, d.finalResidual, d.nIterations, d.converged, d.singular, d.nOuter);
            done[order[j]] = 1;
            now.push_back(rs[order[j]]);
        }
        left -= int(now.size());
        if (!now.empty()) complete(now);
        if (left == 0) break;
        const cudaError_t q = cudaStreamQuery(s);
        if (q == cudaSuccess) break;  // the launch is over: the rest from its records
        if (q != cudaErrorNotReady) CK(q);
        std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
    CK(cudaStreamSynchronize(s));
    now.clear();
    for (int j = 0; j < k; ++j) {
        if (done[order[j]]) continue;
        const SlotSys<double>& r = ln.h64[j];
        set_perf(j, r.initialResidual, r.finalResidual, r.nIterations, r.converged, r.singular, r.nOuter);
        done[order[j]] = 1;
        now.push_back(rs[order[j]]);
    }
    if (!now.empty()) complete(now);
}

}  // namespace

namespace {

// A queued request of the kind the worker serves whose matrix is idle
// (mu held).
SrvRequest* next_ready(cfx_server* sv, bool large) {
    for (int64_t id : sv->queue) {
        SrvRequest* r = sv->reqs[id].get();
        SrvMatrix* m = sv->mats[r->matrixId].get();
        if (m->large == large && !m->busy) return r;
    }
    return nullptr;
}

void finish_all(cfx_server* sv, std::vector<SrvRequest*>& rs, cfx_status st, const std::string& err) {
    for (SrvRequest* r : rs) {
        r->status = st;
        r->error = err;
        r->perf.status = st;
        finish(sv, *r, st == CFX_OK ? Q_DONE : Q_FAILED);
    }
    drop_detached(sv);
    reap(sv);
    sv->cvDone.notify_all();
    sv->cvWork.notify_all();
}

// A large request waits this long for the lanes to go idle on their own
// before the lanes stop starting launches for it.
constexpr auto LARGE_HOLD = std::chrono::milliseconds(100);

// Whether a lane may start a launch now (mu held): small requests are
// ready, and either no large solve is in progress and no large request has
// waited LARGE_HOLD for the lanes, or the running one has yielded.
bool lane_may_start(cfx_server* sv) {
    if (!next_ready(sv, false)) return false;
    if (sv->largeActive) return sv->yieldOpen;
    const SrvRequest* big = next_ready(sv, true);
    return !big || Clock::now() - big->tSubmit < LARGE_HOLD;
}

// A batch lane: every queued small request of the oldest ready one's
// precision and size class, at most one per matrix, in one launch.
void lane_worker(cfx_server* sv, SrvLane* ln) {
    cudaSetDevice(sv->ctx->device);
    std::unique_lock<std::mutex> lk(sv->mu);
    for (;;) {
        // timed: a waiting large request's hold runs out without a notify
        while (!sv->stop && !lane_may_start(sv)) sv->cvWork.wait_for(lk, std::chrono::milliseconds(10));
        if (sv->stop) return;
        SrvRequest* first = next_ready(sv, false);
        const int prec = first->ctl.precision;
        const int cls = size_class(sv, *sv->mats[first->matrixId]);
        std::vector<SrvRequest*> rs;
        std::vector<SrvMatrix*> ms;
        std::deque<int64_t> keep;
        while (!sv->queue.empty()) {
            const int64_t id = sv->queue.front();
            sv->queue.pop_front();
            SrvRequest* r = sv->reqs[id].get();
            SrvMatrix* m = sv->mats[r->matrixId].get();
            if (!m->large && !m->busy && r->ctl.precision == prec && size_class(sv, *m) == cls &&
                int(rs.size()) < sv->cfg.maxBatch) {
                m->busy = true;
                rs.push_back(r);
                ms.push_back(m);
            } else {
                keep.push_back(id);
            }
        }
        sv->queue.swap(keep);
        const Clock::time_point now = Clock::now();
        for (SrvRequest* r : rs) {
            r->state = Q_RUNNING;
            r->tStart = now;
        }
        sv->running += int64_t(rs.size());
        ++sv->activeLanes;
        lk.unlock();
        std::vector<char> done(rs.size(), 0);
        auto complete = [&](std::vector<SrvRequest*>& fin) {
            std::lock_guard<std::mutex> g(sv->mu);
            sv->running -= int64_t(fin.size());
            finish_all(sv, fin, CFX_OK, std::string());
        };
        cfx_status st = CFX_OK;
        std::string err;
        try {
            run_batch(sv, *ln, rs, ms, done, complete);
        } catch (const std::exception& e) {
            st = CFX_ERR_CUDA;
            err = e.what();
        }
        lk.lock();
        std::vector<SrvRequest*> rest;
        for (size_t i = 0; i < rs.size(); ++i)
            if (!done[i]) rest.push_back(rs[i]);
        sv->running -= int64_t(rest.size());
        ++sv->batches;
        sv->batchedSolves += int64_t(rs.size());
        --sv->activeLanes;
        ++sv->batchGen;
        sv->yieldOpen = false;  // a yield's gap closes at its first finished launch
        finish_all(sv, rest, st, err);
    }
}

// Called by the large worker's solve between iterations (lock not held, the
// device idle): when small requests wait, open a gap for the lanes and take
// the GPU back once the launches started in it have finished.
void large_yield(void* arg) {
    cfx_server* sv = static_cast<cfx_server*>(arg);
    std::unique_lock<std::mutex> lk(sv->mu);
    if (sv->stop || !next_ready(sv, false)) return;
    const int64_t gen = sv->batchGen;
    sv->yieldOpen = true;
    ++sv->yields;
    sv->cvWork.notify_all();
    sv->cvWork.wait(lk, [&] {
        return sv->stop || (sv->activeLanes == 0 && (sv->batchGen != gen || !next_ready(sv, false)));
    });
    sv->yieldOpen = false;
}

// The large worker: one large request at a time through the whole-GPU
// drivers on the large context, yielding to batches between iterations.
void large_worker(cfx_server* sv) {
    cudaSetDevice(sv->ctxLarge->device);
    std::unique_lock<std::mutex> lk(sv->mu);
    for (;;) {
        sv->cvWork.wait(lk, [&] {
            return sv->stop || (sv->activeLanes == 0 && !sv->largeActive && next_ready(sv, true));
        });
        if (sv->stop) return;
        SrvRequest* r = next_ready(sv, true);
        SrvMatrix* m = sv->mats[r->matrixId].get();
        sv->queue.erase(std::find(sv->queue.begin(), sv->queue.end(), r->id));
        m->busy = true;
        r->state = Q_RUNNING;
        r->tStart = Clock::now();
        sv->largeActive = true;
        sv->running += 1;
        lk.unlock();
        cfx_status st = CFX_OK;
        std::string err;
        try {
            cfx_perf perf;
            std::memset(&perf, 0, sizeof(perf));
            st = cfx_solve_device(m->mat, &r->ctl, r->d_psi, r->d_b, &perf);
            if (st != CFX_OK) err = cfx_last_error();
            r->perf = perf;
        } catch (const std::exception& e) {
            st = CFX_ERR_CUDA;
            err = e.what();
        }
        lk.lock();
        sv->running -= 1;
        ++sv->largeSolves;
        sv->largeActive = false;
        std::vector<SrvRequest*> rs{r};
        finish_all(sv, rs, st, err);
    }
}

}  // namespace

// ===================================================================== C ABI
extern "C" {

void cfx_server_default_config(cfx_server_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->hbmBudget = int64_t(150) * 1000 * 1000 * 1000;
    c->largeCells = 1000000;
    c->maxBatch = 1024;
    c->nCellsInCoarsestLevel = 10;
    c->groupCells = 100000;
    c->groupSize = 4;
    c->lanes = 8;
}

cfx_status cfx_server_create(cfx_ctx* ctx, const cfx_server_config* cfg, cfx_server** out) {
    if (!ctx || !out) {
        set_error("cfx_server_create: bad argument");
        return CFX_ERR_ARG;
    }
    return guard([&]() -> cfx_status {
        auto sv = std::make_unique<cfx_server>();
        sv->ctx = ctx;
        if (cfg) {
            sv->cfg = *cfg;
        } else {
            cfx_server_default_config(&sv->cfg);
        }
        if (sv->cfg.hbmBudget <= 0 || sv->cfg.largeCells < 1 || sv->cfg.maxBatch < 1 || sv->cfg.groupSize < 0 ||
            sv->cfg.groupSize > 16 || sv->cfg.lanes < 1 || sv->cfg.lanes > 16) {
            set_error("cfx_server_create: bad configuration");
            return CFX_ERR_ARG;
        }
        CK(cudaSetDevice(ctx->device));
        CK(cudaDeviceGetAttribute(&sv->sms, cudaDevAttrMultiProcessorCount, ctx->device));
        CK(cudaStreamCreateWithFlags(&sv->copyStream, cudaStreamNonBlocking));
        // a pool of its own that keeps freed memory for reuse: registering,
        // removing and serving small matrices never waits for the device
        cudaMemPoolProps pp = {};
        pp.allocType = cudaMemAllocationTypePinned;
        pp.location.type = cudaMemLocationTypeDevice;
        pp.location.id = ctx->device;
        CK(cudaMemPoolCreate(&sv->pool, &pp));
        uint64_t keep = UINT64_MAX;
        CK(cudaMemPoolSetAttribute(sv->pool, cudaMemPoolAttrReleaseThreshold, &keep));
        CFX_TRY(cfx_ctx_create(ctx->device, &sv->ctxLarge));
        if (sv->cfg.groupSize > 1) sv->clusterMax = batch_max_clusters(sv->cfg.groupSize);
        for (int i = 0; i < sv->cfg.lanes; ++i) {
            auto ln = std::make_unique<SrvLane>();
            CK(cudaStreamCreateWithFlags(&ln->stream, cudaStreamNonBlocking));
            CK(cudaMalloc(&ln->d_next, 2 * sizeof(unsigned)));
            sv->lanes.push_back(std::move(ln));
        }
        sv->t0 = Clock::now();
        sv->ctxLarge->yield = large_yield;
        sv->ctxLarge->yieldArg = sv.get();
        for (auto& ln : sv->lanes) ln->th = std::thread(lane_worker, sv.get(), ln.get());
        sv->largeWorker = std::thread(large_worker, sv.get());
        ctx_retain(ctx);
        *out = sv.release();
        return CFX_OK;
    });
}

cfx_status cfx_server_destroy(cfx_server* sv) {
    if (!sv) return CFX_ERR_ARG;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop = true;
    }
    sv->cvWork.notify_all();
    for (auto& ln : sv->lanes)
        if (ln->th.joinable()) ln->th.join();
    if (sv->largeWorker.joinable()) sv->largeWorker.join();
    for (auto& ln : sv->lanes) cudaStreamSynchronize(ln->stream);
    for (auto& kv : sv->reqs) free_request_buffers(sv, *kv.second);
    sv->reqs.clear();
    for (auto& kv : sv->mats) free_matrix(sv, *kv.second);
    sv->mats.clear();
    cudaStreamSynchronize(sv->copyStream);
    for (auto& ln : sv->lanes) {
        if (ln->d64) cudaFree(ln->d64);
        if (ln->d32) cudaFree(ln->d32);
        if (ln->h64) cudaFreeHost(ln->h64);
        if (ln->h32) cudaFreeHost(ln->h32);
        if (ln->hDone) cudaFreeHost(ln->hDone);
        if (ln->d_next) cudaFree(ln->d_next);
        if (ln->stream) cudaStreamDestroy(ln->stream);
    }
    sv->lanes.clear();
    cudaStreamDestroy(sv->copyStream);
    if (sv->pool) cudaMemPoolDestroy(sv->pool);
    if (sv->ctxLarge) cfx_ctx_destroy(sv->ctxLarge);
    sv->cvDone.notify_all();
    cfx_ctx* ctx = sv->ctx;  // alive: the server holds a reference
    delete sv;
    ctx_release(ctx);
    return CFX_OK;
}

cfx_status cfx_server_add_matrix(cfx_server* sv, int nCells, int nFaces, const int32_t* l, const int32_t* u,
                                 const double* diag, const double* upper, const double* lower,
                                 const double* faceWeights, int64_t* matrixId) {
    if (!sv || !matrixId || nCells < 1 || nFaces < 0 || !diag || (nFaces > 0 && (!l || !u || !upper))) {
        set_error("cfx_server_add_matrix: bad argument");
        return CFX_ERR_ARG;
    }
    const bool large = nCells > sv->cfg.largeCells;
    const bool sym = lower == nullptr;
    const size_t est = large ? large_estimate(nCells, nFaces) : bsys_bytes_estimate(nCells, nFaces, sym);
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        if (int64_t(est) > sv->cfg.hbmBudget || int64_t(sv->used + est) > sv->cfg.hbmBudget) {
            ++sv->refused;
            set_error("cfx_server_add_matrix: " + std::to_string(est) + " bytes do not fit the HBM budget (" +
                      std::to_string(sv->used) + " of " + std::to_string(sv->cfg.hbmBudget) + " in use)");
            return CFX_ERR_ADMISSION;
        }
        sv->used += est;  // reserved while the matrix is built
    }
    auto m = std::make_unique<SrvMatrix>();
    m->n = nCells;
    m->nf = nFaces;
    m->large = large;
    m->sym = sym;
    cfx_status st = guard([&]() -> cfx_status {
        if (large) {
            CFX_TRY(cfx_mesh_create(sv->ctxLarge, nCells, nFaces, l, u, &m->mesh));
            if (faceWeights)
                CFX_TRY(cfx_gamg_agglomerate(m->mesh, faceWeights, sv->cfg.nCellsInCoarsestLevel, 1));
            CFX_TRY(cfx_matrix_create(m->mesh, diag, upper, lower, &m->mat));
            m->bytes = est;
        } else {
            m->bs = std::make_unique<BSys>();
            m->bs->pool = sv->pool;
            m->bs->poolStream = sv->copyStream;
            CFX_TRY(bsys_create(sv->copyStream, nCells, nFaces, l, u, *m->bs));
            bsys_set_coeffs(sv->copyStream, *m->bs, diag, upper, lower);
            m->bytes = m->bs->addrBytes + m->bs->coefBytes;
        }
        return CFX_OK;
    });
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->used -= est;
    if (st != CFX_OK) {
        if (m->mat) cfx_matrix_destroy(m->mat);
        if (m->mesh) cfx_mesh_destroy(m->mesh);
        return st;
    }
    sv->used += m->bytes;
    m->id = sv->nextMat++;
    *matrixId = m->id;
    sv->mats[m->id] = std::move(m);
    return CFX_OK;
}

cfx_status cfx_server_remove_matrix(cfx_server* sv, int64_t matrixId) {
    if (!sv) return CFX_ERR_ARG;
    std::lock_guard<std::mutex> lk(sv->mu);
    auto it = sv->mats.find(matrixId);
    if (it == sv->mats.end() || it->second->removing) {
        set_error("cfx_server_remove_matrix: unknown matrix " + std::to_string(matrixId));
        return CFX_ERR_ARG;
    }
    it->second->removing = true;
    reap(sv);
    sv->cvDone.notify_all();
    return CFX_OK;
}

}  // extern "C"

extern "C" {

cfx_status cfx_server_submit(cfx_server* sv, int64_t matrixId, const cfx_controls* ctl, const double* psi0,
                             const double* source, int64_t* requestId) {
    if (!sv || !ctl || !source || !requestId) {
        set_error("cfx_server_submit: bad argument");
        return CFX_ERR_ARG;
    }
    auto r = std::make_unique<SrvRequest>();
    r->tSubmit = Clock::now();
    r->ctl = *ctl;
    r->matrixId = matrixId;
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->mats.find(matrixId);
    if (it == sv->mats.end() || it->second->removing) {
        set_error("cfx_server_submit: unknown matrix " + std::to_string(matrixId));
        return CFX_ERR_ARG;
    }
    SrvMatrix* m = it->second.get();
    if (!m->large) {
        const cfx_status st = bsys_check_controls(ctl, m->sym);
        if (st != CFX_OK) return st;
    } else if (ctl->solver == CFX_SOLVER_GAMG) {
        int nl = 0;
        if (cfx_gamg_n_levels(m->mesh, &nl) != CFX_OK || nl < 1) {
            set_error("cfx_server_submit: cudaGAMG on a matrix registered without face weights");
            return CFX_ERR_STATE;
        }
    }
    r->n = m->n;
    r->bytes = 2 * sizeof(double) * size_t(m->n);
    if (int64_t(r->bytes) > sv->cfg.hbmBudget) {
        ++sv->refused;
        set_error("cfx_server_submit: request vectors exceed the HBM budget");
        return CFX_ERR_ADMISSION;
    }
    // admission: wait for space (completions free request vectors)
    sv->cvDone.wait(lk, [&] { return sv->stop || int64_t(sv->used + r->bytes) <= sv->cfg.hbmBudget; });
    if (sv->stop) {
        set_error("cfx_server_submit: server stopping");
        return CFX_ERR_STATE;
    }
    sv->used += r->bytes;
    m->pending++;
    r->id = sv->nextReq++;
    SrvRequest* rp = r.get();
    sv->reqs[r->id] = std::move(r);
    ++sv->submitted;
    lk.unlock();
    // device vectors and uploads outside the lock (the request is not queued yet)
    const cfx_status st = guard([&]() -> cfx_status {
        const size_t b = sizeof(double) * size_t(rp->n);
        CK(cudaMallocFromPoolAsync(reinterpret_cast<void**>(&rp->d_psi), b, sv->pool, sv->copyStream));
        CK(cudaMallocFromPoolAsync(reinterpret_cast<void**>(&rp->d_b), b, sv->pool, sv->copyStream));
        if (psi0)
            CK(cudaMemcpyAsync(rp->d_psi, psi0, b, cudaMemcpyHostToDevice, sv->copyStream));
        else
            CK(cudaMemsetAsync(rp->d_psi, 0, b, sv->copyStream));
        CK(cudaMemcpyAsync(rp->d_b, source, b, cudaMemcpyHostToDevice, sv->copyStream));
        CK(cudaStreamSynchronize(sv->copyStream));
        return CFX_OK;
    });
    lk.lock();
    if (st != CFX_OK) {
        rp->status = st;
        rp->error = cfx_last_error();
        finish(sv, *rp, Q_FAILED);
        free_request_buffers(sv, *rp);
        sv->reqs.erase(rp->id);
        return st;
    }
    *requestId = rp->id;
    sv->queue.push_back(rp->id);
    sv->cvWork.notify_all();
    return CFX_OK;
}

cfx_status cfx_server_wait(cfx_server* sv, int64_t requestId, int timeoutMs, double* psi, cfx_perf* perf) {
    if (!sv) return CFX_ERR_ARG;
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->reqs.find(requestId);
    if (it == sv->reqs.end() || it->second->detached) {
        set_error("cfx_server_wait: unknown request " + std::to_string(requestId));
        return CFX_ERR_ARG;
    }
    SrvRequest* r = it->second.get();
    auto ready = [&] { return r->state != Q_WAITING && r->state != Q_RUNNING; };
    if (timeoutMs < 0) {
        sv->cvDone.wait(lk, ready);
    } else if (!sv->cvDone.wait_for(lk, std::chrono::milliseconds(timeoutMs), ready)) {
        set_error("cfx_server_wait: request " + std::to_string(requestId) + " not finished after " +
                  std::to_string(timeoutMs) + " ms");
        return CFX_ERR_TIMEOUT;
    }
    cfx_status st = r->status;
    if (r->state == Q_CANCELLED) {
        set_error("cfx_server_wait: request " + std::to_string(requestId) + " was cancelled");
        st = CFX_ERR_STATE;
    } else if (r->state == Q_FAILED) {
        set_error(r->error);
    } else {
        if (perf) *perf = r->perf;
        if (psi) {
            st = guard([&]() -> cfx_status {
                CK(cudaMemcpyAsync(psi, r->d_psi, sizeof(double) * size_t(r->n), cudaMemcpyDeviceToHost,
                                   sv->copyStream));
                CK(cudaStreamSynchronize(sv->copyStream));
                return CFX_OK;
            });
        }
    }
    free_request_buffers(sv, *r);
    sv->reqs.erase(it);
    sv->cvDone.notify_all();
    return st;
}

cfx_status cfx_server_cancel(cfx_server* sv, int64_t requestId) {
    if (!sv) return CFX_ERR_ARG;
    std::lock_guard<std::mutex> lk(sv->mu);
    auto it = sv->reqs.find(requestId);
    if (it == sv->reqs.end()) {
        set_error("cfx_server_cancel: unknown request " + std::to_string(requestId));
        return CFX_ERR_ARG;
    }
    SrvRequest& r = *it->second;
    if (r.state == Q_WAITING) {
        sv->queue.erase(std::remove(sv->queue.begin(), sv->queue.end(), requestId), sv->queue.end());
        ++sv->cancelled;
        finish(sv, r, Q_CANCELLED);
        free_request_buffers(sv, r);
        if (r.detached) sv->reqs.erase(it);
        reap(sv);
        sv->cvDone.notify_all();
        return CFX_OK;
    }
    // running: it completes; finished: nothing to stop
    set_error("cfx_server_cancel: request " + std::to_string(requestId) + " is already running or finished");
    return CFX_ERR_STATE;
}

cfx_status cfx_server_release(cfx_server* sv, int64_t requestId) {
    if (!sv) return CFX_ERR_ARG;
    std::lock_guard<std::mutex> lk(sv->mu);
    auto it = sv->reqs.find(requestId);
    if (it == sv->reqs.end()) {
        set_error("cfx_server_release: unknown request " + std::to_string(requestId));
        return CFX_ERR_ARG;
    }
    SrvRequest& r = *it->second;
    r.detached = true;
    if (r.state == Q_WAITING) {
        sv->queue.erase(std::remove(sv->queue.begin(), sv->queue.end(), requestId), sv->queue.end());
        ++sv->cancelled;
        finish(sv, r, Q_CANCELLED);
    }
    drop_detached(sv);
    reap(sv);
    sv->cvDone.notify_all();
    return CFX_OK;
}

cfx_status cfx_server_stats(cfx_server* sv, cfx_server_stats_t* o) {
    if (!sv || !o) return CFX_ERR_ARG;
    std::lock_guard<std::mutex> lk(sv->mu);
    std::memset(o, 0, sizeof(*o));
    o->submitted = sv->submitted;
    o->completed = sv->completed;
    o->cancelled = sv->cancelled;
    o->failed = sv->failed;
    o->refused = sv->refused;
    o->batches = sv->batches;
    o->batchedSolves = sv->batchedSolves;
    o->largeSolves = sv->largeSolves;
    o->queueDepth = int64_t(sv->queue.size());
    o->running = sv->running;
    o->residentMatrices = int64_t(sv->mats.size());
    o->hbmInUse = int64_t(sv->used);
    o->hbmBudget = sv->cfg.hbmBudget;
    o->elapsedS = std::chrono::duration<double>(Clock::now() - sv->t0).count();
    o->solvesPerS = o->elapsedS > 0 ? double(sv->completed) / o->elapsedS : 0.0;
    auto pct = [](std::vector<double> v, double q) {
        if (v.empty()) return 0.0;
        std::sort(v.begin(), v.end());
        const size_t i = std::min(v.size() - 1, size_t(std::ceil(q * double(v.size()))) - (q > 0 ? 1 : 0));
        return v[i];
    };
    if (!sv->latMs.empty()) {
        o->p50Ms = pct(sv->latMs, 0.50);
        o->p99Ms = pct(sv->latMs, 0.99);
        o->maxMs = *std::max_element(sv->latMs.begin(), sv->latMs.end());
        double sum = 0.0;
        for (double x : sv->latMs) sum += x;
        o->meanMs = sum / double(sv->latMs.size());
    }
    o->largeYields = sv->yields;
    o->queueP50Ms = pct(sv->queueMs, 0.50);
    o->queueP99Ms = pct(sv->queueMs, 0.99);
    o->runP50Ms = pct(sv->runMs, 0.50);
    o->runP99Ms = pct(sv->runMs, 0.99);
    return CFX_OK;
}

cfx_status cfx_server_reset_stats(cfx_server* sv) {
    if (!sv) return CFX_ERR_ARG;
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->t0 = Clock::now();
    sv->submitted = sv->completed = sv->cancelled = sv->failed = sv->refused = 0;
    sv->batches = sv->batchedSolves = sv->largeSolves = sv->yields = 0;
    sv->latMs.clear();
    sv->queueMs.clear();
    sv->runMs.clear();
    return CFX_OK;
}

}  // extern "C"
