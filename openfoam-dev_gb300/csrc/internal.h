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
    // the rows in sliced ELL form (Sell in device.cuh): slice starts, entry
    // counts, columns and each entry's coefficient source (a losort slot, or
    // an owner face | SRC_UPPER; -1 padding); sellCol null when not built
    int* sellStart = nullptr;
    unsigned char* sellCnt = nullptr;
    int *sellCol = nullptr, *sellSrc = nullptr;
    int *sellPat = nullptr, *sellOffs = nullptr;  // offset-pattern slices
    int64_t sellEntries = 0;
    int sellPatterns = 0, sellPatternSlices = 0;
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
    // coupled (cyclic) interfaces: CSR over cells of the interface faces in
    // patch-then-face order (neighbour cell per entry), and the cells that
    // have any (ascending)
    int nIf = 0, nIfCells = 0;
    int* ifStart = nullptr;  // [n+1]
    int* ifNbr = nullptr;    // [nIf]
    int* ifCells = nullptr;  // [nIfCells]
    // coarse levels: the finer level's interface faces (their CSR
    // positions, in ascending patch-then-face order) summed into each of this
    // level's interface faces (CSR order)
    int* ifcStart = nullptr;  // [nIf+1]
    int* ifcFine = nullptr;   // [the finer level's nIf]
    // the dense (direct coarsest) matrix's interface entries, in patch then
    // face order: A[luIfRow[k]][luIfCol[k]] -= ifBou[luIfSrc[k]] (the
    // partner patch's coefficient, a CSR position); luIfN < 0: the
    // interfaces' partner patches are not known
    int luIfN = 0;
    int *luIfRow = nullptr, *luIfCol = nullptr, *luIfSrc = nullptr;
};

template <class T>
struct LevelCoeffs {
    bool sym = true;
    T *diag = nullptr, *upper = nullptr, *lower = nullptr;
    T *lowerPerm = nullptr, *upperPerm = nullptr;
    T* sellCoef = nullptr;  // the coefficients in the level's sliced ELL order
    T* rD = nullptr;
    // interfaceBouCoeffs / interfaceIntCoeffs in the mesh's interface CSR
    // order (null: none set)
    T *ifBou = nullptr, *ifInt = nullptr;
    int ifCap = 0;  // allocated length of ifBou / ifInt (coarse levels)
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

// Coupled (cyclic) interface faces of one cell, in patch-then-face order:
// the neighbour cells and coefficients, CSR over the cells (start == null:
// no interfaces).
template <class T>
struct Iface {
    const int* start = nullptr;
    const int* nbr = nullptr;
    const T* coef = nullptr;
};

// interfaceBouCoeffs (Amul, residual, sumA, smoothers) and
// interfaceIntCoeffs (Tmul) of a level, when both the mesh's interfaces and
// the matrix's coefficients are set
template <class T>
inline Iface<T> if_bou(const LevelMesh& m, const LevelCoeffs<T>& a) {
    Iface<T> f;
    if (m.ifStart && a.ifBou) {
        f.start = m.ifStart;
        f.nbr = m.ifNbr;
        f.coef = a.ifBou;
    }
    return f;
}
template <class T>
inline Iface<T> if_int(const LevelMesh& m, const LevelCoeffs<T>& a) {
    Iface<T> f;
    if (m.ifStart && a.ifInt) {
        f.start = m.ifStart;
        f.nbr = m.ifNbr;
        f.coef = a.ifInt;
    }
    return f;
}

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
    // GAMGSolver::interpolate: psi = -(A - D) psi / D on the fine level,
    // then each coarse cell's diagonal-weighted mean replaced by psiC
    // (Apsi: scratch of the fine level's size)
    static void interpolate(cudaStream_t s, const LevelMesh& fine, const LevelCoeffs<T>& a, T* psi, T* Apsi,
                            const T* psiC);
    // LUscalarMatrix of the level (dense, row-major A[n*n], pivots piv[n];
    // vv: scratch [n]); *status = CFX_ERR_FATAL for an all-zero row
    static void lu_factor(cudaStream_t s, const LevelMesh& m, const LevelCoeffs<T>& a, T* A, T* vv, int* piv,
                          int* status);
    // x = LU^-1 b (LUscalarMatrix::solve)
    static void lu_solve(cudaStream_t s, int n, const T* A, const int* piv, const T* b, T* x);
    // x = b / diag (diagonalSolver)
    static void diag_solve(cudaStream_t s, int n, const T* diag, const T* b, T* x);
    // bp = b - (-bou)*psi[nbr] over the coupled interfaces (the Gauss-Seidel
    // smoothers' bPrime before a sweep)
    static void iface_bprime(cudaStream_t s, int n, const Iface<T>& itf, const T* b, const T* psi, T* bp);
    // GAMGInterface::agglomerateCoeffs: coarse interface coefficients (CSR
    // order of level m) from the finer level's
    static void iface_restrict(cudaStream_t s, const LevelMesh& m, const T* fine, T* coarse);
};

// ---- finite-volume assembly (fvm.cu) -------------------------------------
// Resident face geometry of an fvMesh: internal faces in lduAddressing order,
// boundary faces in patch order; cell -> boundary faces (ascending).
struct FvGeom {
    int nBoundary = 0;
    double *magSf = nullptr, *deltaCoeffs = nullptr, *weights = nullptr, *V = nullptr;
    int* bCell = nullptr;
    double *magSfB = nullptr, *deltaCoeffsB = nullptr;
    int *bStart = nullptr, *bFace = nullptr;  // [n+1], [nBoundary]
};

// The terms of one assembly (device pointers; see cfx_fvm_terms).  first:
// the term that starts the fvMatrix (FVM_*), sgnDiv/sgnLap the signs the
// others enter with (0: absent).
enum { FVM_DDT = 0, FVM_DIV = 1, FVM_LAP = 2 };
struct FvmArgs {
    double rDeltaT;
    const double* psi0;
    const double *phi, *phiB;
    int divScheme;
    int lapSign;
    double gammaUniform;
    const double *gamma, *gammaB;
    const int* bcType;
    const double* bcValue;
    const double* su;
    int hasDdt, hasDiv;
};

// diag, upper, lower (asymmetric results) and source of the assembled
// equation as fvMatrix::solveSegregated hands them to the solver.
// The cyclic boundary faces (bcType 3), in boundary order the interfaces'
// faces in patch order: their boundaryCoeffs and internalCoeffs written to
// ifBou/ifInt at the faces' CSR positions ifPos; *status = CFX_ERR_ARG when
// their count is not nIf or a linear div meets one (one CTA, in order).
void launch_fvm_interfaces(cudaStream_t s, const FvGeom& g, const FvmArgs& a, int nIf, const int* ifPos,
                           double* ifBou, double* ifInt, int* status);
void launch_fvm_assemble(cudaStream_t s, const LevelMesh& m, const FvGeom& g, const FvmArgs& a, double* diag,
                         double* upper, double* lower, double* source);

void launch_cast_d2f(cudaStream_t s, int64_t n, const double* in, float* out);
void launch_cast_f2d(cudaStream_t s, int64_t n, const float* in, double* out);

// Deterministic reductions: result written to *out (device double).
// which: 0 sum, 1 sumMag, 2 sumSqr, 3 sumProd
template <class T>
void launch_reduce(cudaStream_t s, Scratch& sc, int which, int n, const T* a, const T* b, double* out);

// ---- packed sweep schedules (host.cpp builds, sweeps.cu runs) -------------
// SCHED_GSB: the backward Gauss-Seidel pass of symGaussSeidel (the GS
// entries, levels of the upper-neighbour DAG, cells in reverse order)
enum { SCHED_FWD = 0, SCHED_BWD = 1, SCHED_GS = 2, SCHED_GSB = 3 };
constexpr int SRC_UPPER = 1 << 30;       // entry coefficient from upper[f]
constexpr int SCHED_CHUNK_GROUPS = 8;    // most groups of 32 slots per grid chunk (one CTA)
// groups per grid chunk of the schedules built from now on (1..8)
int sched_chunk_groups();
void set_sched_chunk_groups(int g);

struct HostSched {
    int kind = 0, nSweeps = 1, nLevels = 0, n = 0, maxK = 0;
    int64_t maxLevelBytes8 = 0;          // largest level's staged bytes (FP64)
    std::vector<int> levelSlot, levelEntry, groupEntry, cell, cnt, nb, src;
    std::vector<int> chunkGroup, chunkLevel, levelChunks;
    // groups each group's slots read from (CSR, ascending): the wavefront
    // form waits on exactly these
    std::vector<int> depStart, dep;
    bool waveOk = false;
    // per slot: its sweep (combined Gauss-Seidel schedules) and its number
    // of lower-neighbour entries (the losort ones, first in its entries)
    std::vector<int> slotSweep, slotLower;
};

constexpr int LVL_LAUNCH_MAX = 128;  // levels a schedule may have for the level-by-level form
constexpr int LVL_LAUNCH_GROUPS = 8;  // groups (warps) per CTA of the level-by-level form

struct DevSched {
    int kind = 0, nSweeps = 1, nLevels = 0, n = 0, maxK = 0;
    int nSlots = 0, nEntries = 0, nGroups = 0, nChunks = 0;
    int64_t maxLevelBytes8 = 0;
    int *levelSlot = nullptr, *levelEntry = nullptr, *groupEntry = nullptr;
    int *cell = nullptr, *cnt = nullptr, *nb = nullptr, *src = nullptr;
    int *chunkGroup = nullptr, *chunkLevel = nullptr, *levelChunks = nullptr;
    int* sync = nullptr;                 // [2 + LVL_STRIDE_MAX*nLevels]: abort, pad, done[level*lvlStride]
    int lvlStride = 1, pollNs = 0;       // set per launch: counter spacing (ints), poll back-off (ns)
    int *depStart = nullptr, *dep = nullptr;  // group dependencies (wavefront form)
    int* gdone = nullptr;                // [nGroups] group finished flags
    int waveOk = 0;                      // dependencies verified to point backwards
    int *slotSweep = nullptr, *slotLower = nullptr;  // [nSlots] (level-ordered schedules)
    // schedules of at most LVL_LAUNCH_MAX levels (the multicolour ones):
    // each level's first slot and first dot partial, kept on the host for the
    // level-by-level form (one launch per level)
    int levelLaunch = 0;
    int hLvlSlot[LVL_LAUNCH_MAX + 1];
    int hLvlPart[LVL_LAUNCH_MAX + 1];
};

constexpr int LVL_STRIDE_MAX = 32;  // level counters up to one 128-byte line apart

// coefficients packed for one schedule and one operation
template <class T>
struct Packed {
    T* coef = nullptr;    // [nEntries]
    T* scalar = nullptr;  // [nSlots]
    T* inS = nullptr;     // [nSlots] right-hand side in slot order (scratch)
    T* flow = nullptr;    // [nSweeps * n] the dataflow form's per-sweep values (scratch)
    bool valid = false;
};

// withDeps: also the group dependency lists of the wavefront form
// color (not null; SCHED_GS, SCHED_FWD or SCHED_BWD): a multicolour order in
// place of the reference's cell order.  Gauss-Seidel: a cell's "lower"
// neighbours are those of a smaller colour (this sweep's values), the others
// its "upper" ones (the previous sweep's), each group in the reference's
// entry order; the DAG has about nSweeps x colours levels.  Forward: the
// smaller-coloured neighbours (losort slots, then owned faces); backward: the
// larger-coloured ones in the reverse of that order; the coefficient of each
// entry is the matrix entry of the cell's row (src as for Gauss-Seidel)
void build_sched(const HostLevel& h, int kind, int nSweeps, HostSched& o, bool withDeps,
                 const std::vector<int>* color = nullptr);
// A greedy colouring of a level's cells (ascending cells, smallest colour no
// neighbour has); returns the number of colours.
int greedy_colors(const HostLevel& h, std::vector<int>& color);
// Gauss-Seidel smoothing order: 0 the reference's cell order everywhere; 1
// (default) the multicolour order for the FP32 inner cycles of the
// mixed-precision solves; 2 the multicolour order for every Gauss-Seidel
// smoothing (tests)
int colored_gs();
void set_colored_gs(int v);
// DIC / DILU (preconditioners and smoothers) order: 0 the reference's; 1
// (default) the multicolour incomplete factorisation of the same sparsity
// for DIC in the FP32 inner solves; 2 for DIC and DILU there; 3 everywhere
// (tests)
int colored_pre();
void set_colored_pre(int v);
// Schedules of at most this many DAG levels (and too large for one CTA's
// shared memory) run level by level, one ordinary launch per level (0: never)
int sweep_level_launch();
void set_sweep_level_launch(int v);

// ---- sweeps (sweeps.cu) ---------------------------------------------------
enum SweepOp {
    OP_FWD = 0,   // w_c = rD_c*r_c - sum (rD_c*lower)*w_l   (losort order)
    OP_BWD = 1,   // w_c -= sum (rD_c*upper)*w_u              (owner faces, reverse)
    OP_GS = 2,    // psi_c = (b_c - sum lower*psi_l - sum upper*psi_u)/diag_c
    OP_RD = 3,    // D_c = diag_c - sum (upper*lower)/D_l     (pivots; 1/D after)
};

void sweeps_init(int numSms);
template <class T>
bool sweep_is_grid(const DevSched& s);
// number of dot partials a fused backward sweep writes
template <class T>
int sweep_partials(const DevSched& s);
// The execution form a schedule runs in (0 one CTA, 1 cluster in distributed
// shared memory, 2 one CTA with the vector in global memory, 3 cluster in
// global memory, 4 persistent grid, 5 dataflow, 6 one launch per level)
template <class T>
int sweep_mode(const DevSched& s);
template <class T>
cfx_status run_sweep(cudaStream_t st, const DevSched& s, int op, const Packed<T>& p, const T* in, T* x,
                     const T* dotWith, double* partials, const int* done, int* status);
// Failure-path exercise of the grid form's bounded waits (see sweeps.cu).
template <class T>
cfx_status run_sweep_stalled(cudaStream_t st, const DevSched& s, const Packed<T>& p, const T* in, T* x,
                             unsigned long long timeoutNs, int* status);
template <class T>
void pack_sweep(cudaStream_t st, const DevSched& s, int op, const LevelCoeffs<T>& c, Packed<T>& p);

// meshes with at most this many cells sweep in one CTA even when the vector
// does not fit in shared memory
int small_sweep_threshold();
void set_small_sweep_threshold(int n);
size_t sweep_smem_cap();
size_t sweep_smem_cap_max();
int sweep_wave();
void set_sweep_wave(int on);
// dataflow sweeps (level-ordered schedules larger than one CTA)
int sweep_flow();
void set_sweep_flow(int on);
int sweep_flow_ahead();
void set_sweep_flow_ahead(int k);
// level-counter grid form: counter spacing in ints (1..LVL_STRIDE_MAX) and
// the back-off of its polls (ns, 0: none)
// single-CTA form in FP32: 32 entries per slot held in registers for
// schedules with more than 16 (1, default) or 16 (0)
int sweep_cta_xl();
void set_sweep_cta_xl(int on);
int sweep_grid_stride();
void set_sweep_grid_stride(int k);
int sweep_grid_poll_ns();
void set_sweep_grid_poll_ns(int ns);
// A x products: 0 the losort/owner gathers, 1 the sliced ELL rows with
// explicit columns, 2 (default) sliced ELL with offset-pattern slices (1/2
// read when a level's rows are uploaded)
int amul_sell();
void set_amul_sell(int on);
// the dataflow form's value buffers: sweeps x cells of the schedule (0: none)
size_t sweep_flow_values(const DevSched& s, int op);
void set_sweep_smem_cap(size_t b);
int sweep_cluster_size();
void set_sweep_cluster_size(int cs);
int sweep_cluster_pre();
void set_sweep_cluster_pre(int cs);
int cluster_global_cells();
void set_cluster_global_cells(int n);

// ---- host addressing (host.cpp) ----------------------------------------------
cfx_status build_host_level(int n, int nf, const int* l, const int* u, HostLevel& h, bool validate);
// A level's rows in sliced ELL form (Sell in device.cuh), built on the host.
struct HostSell {
    std::vector<int> start, pat, offs, col, src;
    std::vector<unsigned char> cnt;
    int64_t entries = 0;
    int patterns = 0, patternSlices = 0;
};
bool build_sell(const HostLevel& h, bool patterns, HostSell& out);
void build_schedules(HostLevel& h);
int pair_agglomerate(int nFine, int nFaces, const int* l, const int* u, const double* w,
                     bool& forward, std::vector<int>& map);
int agglomerate_addressing(int nFaces, const int* l, const int* u, const std::vector<int>& rm,
                           int nCoarse, std::vector<int>& cl, std::vector<int>& cu,
                           std::vector<int>& fra, std::vector<int>& flip);
void face_area_pair_weights(int nFaces, const double* Sf, double* w);

}  // namespace cfx
