// objects.h - host-side objects shared by the C ABI's translation units:
// device allocation arenas, the context (device, stream, scratch), cached
// CUDA graphs and the exception-to-status guard.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "internal.h"
#include "solvers.h"

namespace cfx {

struct CudaError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// An error the reference reports as FatalError (or another fixed status),
// raised from deep inside a solve's set-up.
struct StatusError : std::runtime_error {
    cfx_status status;
    StatusError(cfx_status st, const std::string& what) : std::runtime_error(what), status(st) {}
};

inline void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        if (e == cudaErrorMemoryAllocation) throw std::bad_alloc();
        throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
    }
}
#define CK(x) ck((x), #x)

// Owner of a set of device allocations.
struct Arena {
    std::vector<void*> ptrs;
    size_t bytes = 0;
    template <class T>
    T* get(size_t n) {
        void* p = nullptr;
        const size_t b = std::max<size_t>(n, 1) * sizeof(T);
        CK(cudaMalloc(&p, b));
        ptrs.push_back(p);
        bytes += b;
        return static_cast<T*>(p);
    }
    template <class T>
    T* upload(const std::vector<T>& v, cudaStream_t s) {
        T* p = get<T>(v.size());
        if (!v.empty()) CK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
        return p;
    }
    void release() {
        for (void* p : ptrs) cudaFree(p);
        ptrs.clear();
        bytes = 0;
    }
    ~Arena() { release(); }
};

}  // namespace cfx

using namespace cfx;

struct cfx_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    Arena arena;
    Scratch sc;
    SolveState* d_state = nullptr;  // [4]: outer, inner, spare
    SolveState* h_state = nullptr;  // pinned mirror
    int* d_status = nullptr;
    double* d_red = nullptr;        // [8] reduction outputs
    double* h_red = nullptr;        // pinned
    // The creator's handle plus one reference per mesh, batch and server
    // built on this context: cfx_ctx_destroy drops the creator's, and the
    // context is freed when the last user goes, in whatever order the
    // caller (or a garbage collector) destroys them.
    std::atomic<int> refs{1};
    // Stream order with the caller: entry points that take the caller's
    // device pointers first make this context's (non-blocking) stream wait
    // for the work already enqueued on the legacy default stream, where
    // CUDA runtime callers and PyTorch produce their arrays by default, and
    // the asynchronous ones make that stream wait for their results.
    cudaEvent_t evIn = nullptr, evOut = nullptr;
    // Called by the solve drivers between iterations (V-cycles, batches of
    // Krylov iterations), when the device is idle: lets an owner such as the
    // solve server run other work there.  Not part of the C ABI.
    void (*yield)(void*) = nullptr;
    void* yieldArg = nullptr;
};

namespace cfx {
void ctx_retain(cfx_ctx* ctx);
void ctx_release(cfx_ctx* ctx);

// The caller's inputs are ready before this context's stream reads them.
inline void after_caller(cfx_ctx* ctx) {
    CK(cudaEventRecord(ctx->evIn, cudaStreamLegacy));
    CK(cudaStreamWaitEvent(ctx->stream, ctx->evIn, 0));
}

// The caller's later work on the default stream sees this stream's results
// (and may reuse the input arrays it passed).
inline void to_caller(cfx_ctx* ctx) {
    CK(cudaEventRecord(ctx->evOut, ctx->stream));
    CK(cudaStreamWaitEvent(cudaStreamLegacy, ctx->evOut, 0));
}
}  // namespace cfx

struct GraphCache {
    cudaGraphExec_t exec = nullptr;
    uint64_t key = 0;
    int64_t kernels = 0;  // kernel nodes per replay (launch accounting)
    void reset() {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        key = 0;
        kernels = 0;
    }
    ~GraphCache() { reset(); }
};

namespace cfx {

template <class F>
inline cfx_status guard(F&& f) {
    try {
        return f();
    } catch (const std::bad_alloc&) {
        set_error("device or host allocation failed");
        return CFX_ERR_NOMEM;
    } catch (const CudaError& e) {
        set_error(e.what());
        return CFX_ERR_CUDA;
    } catch (const StatusError& e) {
        set_error(e.what());
        return e.status;
    } catch (const std::exception& e) {
        set_error(e.what());
        return CFX_ERR_ARG;
    }
}

// Capture `body` into the cache's executable graph once (keyed), then launch.
template <class F>
inline void graph_launch(GraphCache& g, uint64_t key, cudaStream_t s, F&& body) {
    if (!g.exec || g.key != key) {
        g.reset();
        cudaGraph_t graph;
        // kernels are counted when a replay runs them, not when captured
        const int64_t before = launch_count();
        CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        body();
        CK(cudaStreamEndCapture(s, &graph));
        g.kernels = launch_count() - before;
        count_launch(-int(g.kernels));
        CK(cudaGraphInstantiate(&g.exec, graph, 0));
        cudaGraphDestroy(graph);
        g.key = key;
    }
    CK(cudaGraphLaunch(g.exec, s));
    count_launch(int(g.kernels));
}

}  // namespace cfx
