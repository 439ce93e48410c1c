// noalloc.cu - a reduction entry point that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a host application whose own memory
// pool has reserved the whole GPU up front (a cudaMalloc from a library then
// fails, or takes memory the pool accounts for), or one that runs under a
// fixed device-memory budget with no room for a library's allocations.
// cfx_reduce_noalloc serves them: its only scratch is the file-scope array
// below, which the CUDA runtime places when the library's device code is
// loaded and which every GPU that loads the library holds until the process
// exits.  The first call on a device looks up the array's device address
// (once, with that device current); make that first call before any stream
// capture.
//
// Scratch: NA_MAX_BLOCKS fixed-order block partials plus a completion
// counter.  Each block reduces exactly NA_NT*NA_ITEMS consecutive elements,
// so n may be at most NA_MAX_BLOCKS*NA_NT*NA_ITEMS = 33,554,432.  All calls on
// a device share the array and it keeps the last call's contents; calls whose
// kernels overlap on the GPU (different streams, no ordering) race on it.

#include <mutex>
#include <string>

#include "device.cuh"
#include "internal.h"
#include "solvers.h"

namespace cfx {

namespace {

constexpr int NA_NT = 256;
constexpr int NA_ITEMS = 32;
constexpr int NA_MAX_BLOCKS = 4096;
constexpr long long NA_MAX_N = (long long)NA_MAX_BLOCKS * NA_NT * NA_ITEMS;
constexpr int NA_MAX_DEVICES = 64;

struct NaScratch {
    double partials[NA_MAX_BLOCKS];
    unsigned counter;
};

static __device__ __align__(256) NaScratch g_na_scratch;

std::mutex g_na_mutex;
NaScratch* g_na_ptr[NA_MAX_DEVICES] = {};

template <int WHICH>
__global__ void __launch_bounds__(NA_NT) na_reduce_k(int n, const double* __restrict__ a,
                                                    const double* __restrict__ b, NaScratch* sc, double* out) {
    __shared__ double sh[NA_NT / 32];
    const long long base = (long long)blockIdx.x * NA_NT * NA_ITEMS;
    double acc = 0.0;
#pragma unroll 4
    for (int k = 0; k < NA_ITEMS; ++k) {
        const long long i = base + (long long)k * NA_NT + threadIdx.x;
        if (i < n) {
            const double x = a[i];
            if (WHICH == 0) acc += x;
            else if (WHICH == 1) acc += fabs(x);
            else if (WHICH == 2) acc += x * x;
            else acc += x * b[i];
        }
    }
    acc = block_sum<NA_NT>(acc, sh);
    if (threadIdx.x == 0) sc->partials[blockIdx.x] = acc;
    if (last_block(&sc->counter)) {
        double s = 0.0;
        for (int i = threadIdx.x; i < gridDim.x; i += NA_NT) s += __ldcg(sc->partials + i);
        s = block_sum<NA_NT>(s, sh);
        if (threadIdx.x == 0) *out = s;
    }
}

}  // namespace

}  // namespace cfx

using namespace cfx;

extern "C" cfx_status cfx_reduce_noalloc(int which, int n, const double* d_a, const double* d_b, double* d_out,
                                         void* stream) {
    if (which < 0 || which > 3 || n < 0 || !d_a || !d_out || (which == 3 && !d_b)) {
        set_error("cfx_reduce_noalloc: bad argument");
        return CFX_ERR_ARG;
    }
    if ((long long)n > NA_MAX_N) {
        set_error("cfx_reduce_noalloc: n = " + std::to_string(n) + " exceeds the maximum " +
                  std::to_string(NA_MAX_N) + " that its static scratch (" + std::to_string(NA_MAX_BLOCKS) +
                  " block partials) covers");
        return CFX_ERR_ARG;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES) {
        set_error(std::string("cfx_reduce_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
        return CFX_ERR_CUDA;
    }
    NaScratch* sc = nullptr;
    {
        // Set-up, once per device with that device current: the host-side
        // name g_na_scratch is not a device address; ask the runtime for it.
        std::lock_guard<std::mutex> lock(g_na_mutex);
        if (!g_na_ptr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_na_scratch);
            if (e != cudaSuccess || !p) {
                set_error(std::string("cfx_reduce_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e) +
                          " (a device's first call looks up the scratch address and must be made outside "
                          "stream capture)");
                return CFX_ERR_CUDA;
            }
            g_na_ptr[dev] = static_cast<NaScratch*>(p);
        }
        sc = g_na_ptr[dev];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the completion counter must start at zero (a previous call leaves it
    // zero, but an interrupted one might not)
    e = cudaMemsetAsync(&sc->counter, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) {
        set_error(std::string("cfx_reduce_noalloc: cudaMemsetAsync: ") + cudaGetErrorString(e));
        return CFX_ERR_CUDA;
    }
    const int blocks = n == 0 ? 1 : int((n + (long long)NA_NT * NA_ITEMS - 1) / ((long long)NA_NT * NA_ITEMS));
    switch (which) {
        case 0: na_reduce_k<0><<<blocks, NA_NT, 0, s>>>(n, d_a, d_b, sc, d_out); break;
        case 1: na_reduce_k<1><<<blocks, NA_NT, 0, s>>>(n, d_a, d_b, sc, d_out); break;
        case 2: na_reduce_k<2><<<blocks, NA_NT, 0, s>>>(n, d_a, d_b, sc, d_out); break;
        default: na_reduce_k<3><<<blocks, NA_NT, 0, s>>>(n, d_a, d_b, sc, d_out); break;
    }
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(std::string("cfx_reduce_noalloc: launch: ") + cudaGetErrorString(e));
        return CFX_ERR_CUDA;
    }
    return CFX_OK;
}
