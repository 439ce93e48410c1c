// internal.h - shared types of libcudaLduSolvers (host + device).
//
// Layout in HBM (one LevelMesh per GAMG level, level 0 = the fvMesh):
//   l, u                 int32[nf]   lowerAddr / upperAddr (upper-triangular)
//   ownerStart           int32[n+1]  faces of each owner (upper neighbours)
//   losortStart          int32[n+1]  faces of each neighbour, via losort
//   losortL              int32[nf]   l[losort[k]]: lower neighbour of slot k
//   losort               int32[nf]
//   fwd / bwd schedules  cells grouped by DAG level of the lower / upper
//                        dependency graph, cut into chunks of <= SWEEP_CHUNK
// Coefficients per level (LevelCoeffs<T>, T = double, or float for the
// inner solve of mixed precision):
//   diag[n], upper[nf], lower[nf] (asymmetric only)
//   lowerPerm[nf] = lower[losort[k]] (upper[losort[k]] when symmetric)
//   upperPerm[nf] = upper[losort[k]] (asymmetric only; DILU reciprocal D)
//   rD[n] DIC/DILU reciprocal diagonal
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "cfx.h"

namespace cfx {

constexpr int SWEEP_NT = 256;        // threads of a multi-CTA sweep CTA
constexpr int SWEEP_CHUNK = 256;     // cells per chunk (<= SWEEP_NT)
constexpr int SMALL_NT = 1024;       // threads of a single-CTA sweep
constexpr int RED_NT = 256;          // threads of a streaming/reduction block
constexpr int RED_MAXB = 1216;       // max blocks of a streaming kernel (152 SMs x 8)
constexpr int MAX_LEVELS = 50;       // GAMGAgglomeration::maxLevels_

void set_error(const std::string& msg);
const char* last_error();

#define CFX_CUDA(x)                                                                 \
    do {                                                                            \
        cudaError_t e_ = (x);                                                       \
        if (e_ != cudaSuccess) {                                                    \
            ::cfx::set_error(std::string(#x) + ": " + cudaGetErrorString(e_));       \
            return CFX_ERR_CUDA;                                                    \
        }                                                                           \
    } while (0)

#define CFX_TRY(x)                                \
    do {                                          \
        cfx_status s_ = (x);                      \
        if (s_ != CFX_OK) return s_;              \
    } while (0)

// Level schedule of a dependency DAG (device arrays).
struct Schedule {
    int nLevels = 0, nChunks = 0, nCells = 0, maxLevelWidth = 0;
    int* cells = nullptr;        // [n] cells by level, ascending index within a level
    int* levelStart = nullptr;   // [nLevels+1]
    int* chunkStart = nullptr;   // [nChunks+1]
    int* chunkLevel = nullptr;   // [nChunks]
    int* levelChunks = nullptr;  // [nLevels]
    int* sync = nullptr;         // [2 + nLevels]: ticket, abort, done[level]
};

// Host copy of a level's addressing.
struct HostLevel {
    int n = 0, nf = 0;
    std::vector<int> l, u, ownerStart, losortStart, losort, losortL;
    std::vector<int> fwdCells, fwdLevelStart, bwdCells, bwdLevelStart;
    // restriction to the next coarser level (GAMG)
    int nCoarse = 0, nCoarseFaces = 0;
    std::vector<int> restrictAddr, faceRestrict, faceFlip;
};

// Device addressing of one level.
struct LevelMesh {
    int n = 0, nf = 0;
    int *l = nullptr, *u = nullptr, *ownerStart = nullptr, *losortStart = nullptr;
    int *losort = nullptr, *losortL = nullptr;
    Schedule fwd, bwd;
    // restriction to the next coarser level (valid when nCoarse > 0)
    int nCoarse = 0, nCoarseFaces = 0;
    int* restrictAddr = nullptr;      // [n] fine -> coarse cell
    int* coarseCellStart = nullptr;   // [nCoarse+1]
    int* coarseCellFine = nullptr;    // [n] fine cells of each coarse cell, ascending
    int* faceRestrict = nullptr;      // [nf] >=0 coarse face, <0 -(coarse cell)-1
    int* faceFlip = nullptr;          // [nf]
    int* coarseFaceStart = nullptr;   // [nCoarseFaces+1]
    int* coarseFaceFine = nullptr;    // fine faces of each coarse face, ascending
    int* intFaceStart = nullptr;      // [nCoarse+1]
    int* intFaceFine = nullptr;       // fine faces inside each coarse cell, ascending
};

template <class T>
struct LevelCoeffs {
    bool sym = true;
    T *diag = nullptr, *upper = nullptr, *lower = nullptr;
    T *lowerPerm = nullptr, *upperPerm = nullptr;
    T* rD = nullptr;
};

// Device-resident scalars of one solve.  Kernels read and update them so the
// iteration loop needs no host round trip; `done` predicates every kernel.
struct SolveState {
    double tolerance, relTol;
    int maxIter, minIter;
    double normFactor, initialResidual, finalResidual;
    double wArA, wArAold, alpha, beta, omega, rA0rA, rA0rAold, tAtA;
    double sf, red0, red1, red2;
    int nIterations, converged, singular, done;
    int error, phase, pad0, pad1;
};

// Scratch of a context: reduction partials and counters.
struct Scratch {
    double* partials = nullptr;     // [RED_MAXB * 4]
    unsigned* counters = nullptr;   // [16]
    double* result = nullptr;       // [16]
    double* chunkPartials = nullptr;  // per-chunk partial sums of fused sweeps
    size_t chunkPartialsCap = 0;
};

// ---- launchers (kernels.cu) ----------------------------------------------
template <class T>
struct Ops {
    // y = A x (row gather; per-cell face order as lduMatrix::Amul)
    static void amul(cudaStream_t s, const LevelMesh& m, const LevelCoeffs<T>& a, const T* x, T* y);
    static void tmul(cudaStream_t s, const LevelMesh& m, const LevelCoeffs<T>& a, const T* x, T* y);
    static void residual(cudaStream_t s, const LevelMesh& m, const LevelCoeffs<T>& a, const T* x,
                         const T* b, T* r);
    static void sumA(cudaStream_t s, const LevelMesh& m, const LevelCoeffs<T>& a, T* out);
    // coefficient preparation: lowerPerm/upperPerm gathers
    static void permute(cudaStream_t s, const LevelMesh& m, LevelCoeffs<T>& a);
    // coarse assembly from the fine level coefficients (reference order)
    static void coarsen(cudaStream_t s, const LevelMesh& fine, const LevelCoeffs<T>& fa,
                        const LevelMesh& coarse, LevelCoeffs<T>& ca);
    // cf[c] = sum of ff over the fine cells of c (ascending)
    static void restrict_field(cudaStream_t s, const LevelMesh& fine, const T* ff, T* cf);
    // ff[i] = cf[restrict[i]]
    static void prolong_field(cudaStream_t s, const LevelMesh& fine, const T* cf, T* ff);
    // rD = 1/rD
    static void reciprocal(cudaStream_t s, int n, T* x);
};

void launch_cast_d2f(cudaStream_t s, int64_t n, const double* in, float* out);
void launch_cast_f2d(cudaStream_t s, int64_t n, const float* in, double* out);

// Deterministic reductions: result written to *out (device double).
// which: 0 sum, 1 sumMag, 2 sumSqr, 3 sumProd
template <class T>
void launch_reduce(cudaStream_t s, Scratch& sc, int which, int n, const T* a, const T* b, double* out);

// ---- sweeps (sweeps.cu) ---------------------------------------------------
enum SweepOp {
    SW_DIC_FWD = 0,   // w = rD*r, then w_u -= (rD_u*lp)*w_l in losort order
    SW_BWD = 1,       // w_l -= (rD_l*upper)*w_u, owner faces in reverse order
    SW_GS = 2,        // psi_c = (b - sum lp*psi_l - sum upper*psi_u)/diag
    SW_RD = 3,        // D_u -= (up*lp)/D_l (pivots; reciprocal afterwards)
    SW_T_FWD = 4,     // DILU preconditionT forward: w_u -= (rD_u*upperPerm)*w_l
};

template <class T>
struct SweepArgs {
    const T* rD;        // reciprocal diagonal (DIC/DILU) or nullptr
    const T* diag;      // GS
    const T* lp;        // lowerPerm
    const T* up;        // upperPerm (SW_RD asym, SW_T_FWD)
    const T* upper;     // owner-side coefficients
    const T* in;        // r (fwd) or b (GS) ; D initial for SW_RD = diag
    T* x;               // in/out vector
    // fused dot of the backward sweep result with `dotWith` (per-chunk partials)
    const T* dotWith;
    double* chunkPartials;
    // when non-null and *done != 0 the sweep returns at once (solver predicate)
    const int* done;
};

template <class T>
cfx_status run_sweep(cudaStream_t s, const LevelMesh& m, const Schedule& sch, int op,
                     const SweepArgs<T>& a, int* status, bool forceSmall = false);

// Number of dot partials a fused sweep writes (1 for the single-CTA form).
int sweep_partials(const LevelMesh& m, const Schedule& s, bool forceSmall = false);

// Threshold (cells) below which sweeps run in one CTA with block barriers.
int small_sweep_threshold();
void set_small_sweep_threshold(int n);
void set_num_sms(int n);

// ---- host addressing (host.cpp) ----------------------------------------------
cfx_status build_host_level(int n, int nf, const int* l, const int* u, HostLevel& h, bool validate);
void build_schedules(HostLevel& h);
int pair_agglomerate(int nFine, int nFaces, const int* l, const int* u, const double* w,
                     bool& forward, std::vector<int>& map);
int agglomerate_addressing(int nFaces, const int* l, const int* u, const std::vector<int>& rm,
                           int nCoarse, std::vector<int>& cl, std::vector<int>& cu,
                           std::vector<int>& fra, std::vector<int>& flip);
void face_area_pair_weights(int nFaces, const double* Sf, double* w);

}  // namespace cfx
