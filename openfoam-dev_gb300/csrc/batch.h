// batch.h - resident small systems solved by one thread group each
// (cfx_batch_*, and the systems of the solve server).
//
// A BSys is one lduMatrix system held on the device in slot order (SlotSys:
// cells ordered by forward level of the DIC/DILU lower DAG, neighbours and
// coefficients in column-major ELL), in two allocations:
//   addressing (set at creation): cnt, loSrc, upSrc, cellOf, the forward
//     level ranges and the backward level schedule;
//   coefficients + work (set with the coefficients): FP64 diag, lo, up,
//     upLo (asymmetric only), the same in FP32 for the inner solves of mixed
//     precision, then the FP64 and FP32 work vectors (slot order).
// The right-hand side and solution in cell order live with the owner (a
// batch keeps them concatenated, a server request keeps its own).
#pragma once

#include <vector>

#include "objects.h"

namespace cfx {

struct BSys {
    int n = 0, nf = 0, nFwd = 0, nBwd = 0, wLo = 0, wUp = 0;
    bool sym = true, hasCoeffs = false;
    char* dAddr = nullptr;    // addressing allocation
    char* dCoef = nullptr;    // coefficients + work allocation
    // with a pool, both allocations are stream-ordered on poolStream (no
    // device-wide synchronisation when they are made or freed)
    cudaMemPool_t pool = nullptr;
    cudaStream_t poolStream = nullptr;
    size_t addrBytes = 0, coefBytes = 0;
    SlotSys<double> h64{};    // pointers into the allocations (bCell, psiCell unset)
    SlotSys<float> h32{};
    // host maps for coefficient uploads: face of each ELL entry (-1: padding)
    std::vector<int> loFace, upFace, cellOf;
    BSys() = default;
    BSys(const BSys&) = delete;
    BSys& operator=(const BSys&) = delete;
    ~BSys();
};

// Device bytes of a system with n cells and nf faces (both allocations,
// upper bound for any ELL width up to 3 + 3 and any level count <= n).
size_t bsys_bytes_estimate(int n, int nf, bool sym);
// Validates and uploads the addressing (throws on CUDA errors; returns the
// addressing status otherwise).
cfx_status bsys_create(cudaStream_t s, int n, int nf, const int32_t* l, const int32_t* u, BSys& sys);
// Uploads the coefficients (lower == nullptr: symmetric), allocating the
// coefficient + work block when absent or when the symmetry changed.
void bsys_set_coeffs(cudaStream_t s, BSys& sys, const double* diag, const double* upper, const double* lower);
// Fills the launch records of one solve of sys with the given controls;
// psi / b are the system's cell-order device vectors.
void bsys_records(const BSys& sys, const cfx_controls& c, double* psi, const double* b, SlotSys<double>& r64,
                  SlotSys<float>& r32);
// Solver name as SolverPerformance prints it, e.g. "DICPCG".
const char* bsys_solver_name(const cfx_controls& c);
// Batch controls check: PCG (symmetric) or PBiCGStab; any preconditioner.
cfx_status bsys_check_controls(const cfx_controls* c, bool sym);

// FP32 inner solves of mixed-precision batches reduce the residual by
// 10^-digits (default 3).
void batch_set_inner_digits(int d);
int batch_inner_digits();

}  // namespace cfx
