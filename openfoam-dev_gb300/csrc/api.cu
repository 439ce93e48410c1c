// api.cu - the C ABI (include/cfx.h): contexts, resident meshes and matrices,
// and the host drivers of cudaPCG / cudaPBiCGStab / cudaGAMG.
//
// The drivers enqueue device work only; the host reads the device SolveState
// once per batch of iterations (Krylov) or once per V-cycle (GAMG).  One
// iteration (or one V-cycle) is captured once into a CUDA graph and replayed,
// so launch overhead is paid once per graph, not per kernel.

#include <algorithm>
#include <cstring>
#include <memory>
#include <map>
#include <mutex>
#include <new>
#include <stdexcept>

#include "internal.h"
#include "batch.h"
#include "objects.h"
#include "solvers.h"

namespace cfx {

namespace {
thread_local std::string g_err;
}

void set_error(const std::string& msg) { g_err = msg; }
const char* last_error() { return g_err.c_str(); }


}  // namespace cfx

using namespace cfx;

// ------------------------------------------------------------------ objects

struct cfx_mesh {
    cfx_ctx* ctx = nullptr;  // retained while the mesh lives
    // The creator's handle plus one reference per matrix on this mesh:
    // cfx_mesh_destroy drops the creator's and the mesh is freed with its
    // last matrix, so matrices may be destroyed after their mesh.
    std::atomic<int> refs{1};
    Arena arena;
    std::vector<HostLevel> host;   // [0] = the mesh, then GAMG coarse levels
    std::vector<LevelMesh> dev;
    int nCoarseLevels = 0;         // GAMG levels below the mesh (0: none)
    uint64_t version = 1;          // bumped when the level hierarchy changes
    // packed sweep schedules per level, built on first use
    struct Scheds {
        DevSched fwd, bwd;
        bool hasFwd = false, hasBwd = false;
        DevSched fwdC, bwdC;  // the multicolour forward / backward schedules
        bool hasFwdC = false, hasBwdC = false;
        std::map<int, DevSched> gs;
    };
    std::vector<Scheds> sched;
    Arena schedArena;
    FvGeom fv;  // finite-volume face geometry (cfx_fv_geometry)
    bool hasFv = false;
    Arena fvArena;
    // coupled interfaces (cfx_mesh_set_interfaces): the CSR position of each
    // interface face given in patch order
    int nIf = 0;
    std::vector<int> ifPos;
    int* d_ifPos = nullptr;  // the same on the device (device assembly of cyclic faces)
    Arena ifArena;
    // the same interfaces on the host (patch sizes, face cells, partner
    // cells, patch order) and the GAMG levels' coarse interfaces; each
    // patch's partner patch when known (cfx_mesh_set_interface_partners)
    std::vector<int> ifPatchSize, ifFaceCell, ifNbrCell, ifNbrPatch;
    Arena ifCoarseArena;
};

template <class T>
struct LevelPack {
    Packed<T> rd, fwd, bwd;
    Packed<T> fwdT, bwdT;  // DILU preconditionT: the packs of the transpose
    Packed<T> rdC, fwdC, bwdC, fwdTC, bwdTC;  // the same on the multicolour schedules
    std::map<int, Packed<T>> gs;
};

// Named device work vectors of one precision; slot i keeps its allocation
// (grown when a larger size is asked for), so captured graphs stay valid.
template <class T>
struct Work {
    Arena arena;
    int n = 0;
    std::vector<T*> v;
    std::vector<int> sz;
    T* get(int i, int nn) {
        if ((int)v.size() <= i) {
            v.resize(i + 1, nullptr);
            sz.resize(i + 1, 0);
        }
        if (!v[i] || sz[i] < nn) {
            v[i] = arena.template get<T>(nn);
            sz[i] = nn;
        }
        return v[i];
    }
};

namespace cfx {
struct PcGamg;  // the GAMG preconditioner's cycles (defined with the V-cycle)
void pc_gamg_free(PcGamg* p);
}  // namespace cfx

struct cfx_matrix {
    cfx_mesh* mesh = nullptr;
    PcGamg* pcGamg = nullptr;
    Arena arena;
    bool sym = true;
    bool diagonal = false;  // lduMatrix::diagonal(): no off-diagonal coefficients
    std::vector<LevelCoeffs<double>> c64;   // per level
    std::vector<LevelCoeffs<float>> c32;
    bool coarse64 = false, coarse32 = false, fine32 = false;
    // host<->device staging and work vectors
    double *d_psi = nullptr, *d_src = nullptr;
    Work<double> w64;
    Work<float> w32;
    std::vector<Work<double>> lv64;  // per-level GAMG vectors
    std::vector<Work<float>> lv32;
    Arena blockArena;
    std::vector<LevelPack<double>> p64;
    std::vector<LevelPack<float>> p32;
    BlockSys<double>* d_blk64 = nullptr;
    BlockSys<float>* d_blk32 = nullptr;
    int* luPiv = nullptr;  // directSolveCoarsest pivots
    int luPivN = 0;
    int ifN = 0;  // interface coefficients held (cfx_matrix_set_interface_coeffs)
    GraphCache gPCG, gBiCG, gGAMG, gMixed;
    GraphCache gDiag32;  // cfx_diag_smooth_f32: the smoothing as the V-cycle graph replays it
};

// --------------------------------------------------------------- utilities
namespace {


void upload_schedule(Arena& ar, cudaStream_t s, const std::vector<int>& cells, const std::vector<int>& levelStart,
                     Schedule& sch) {
    const int nl = int(levelStart.size()) - 1;
    std::vector<int> chunkStart{0}, chunkLevel, levelChunks(std::max(nl, 0), 0);
    int maxw = 0;
    for (int L = 0; L < nl; ++L) {
        const int b = levelStart[L], e = levelStart[L + 1];
        maxw = std::max(maxw, e - b);
        for (int i = b; i < e; i += SWEEP_CHUNK) {
            chunkStart.push_back(std::min(i + SWEEP_CHUNK, e));
            chunkLevel.push_back(L);
            levelChunks[L]++;
        }
    }
    sch.nLevels = nl;
    sch.nCells = int(cells.size());
    sch.nChunks = int(chunkLevel.size());
    sch.maxLevelWidth = maxw;
    sch.cells = ar.upload(cells, s);
    sch.levelStart = ar.upload(levelStart, s);
    sch.chunkStart = ar.upload(chunkStart, s);
    sch.chunkLevel = ar.upload(chunkLevel, s);
    sch.levelChunks = ar.upload(levelChunks, s);
    sch.sync = ar.get<int>(2 + std::max(nl, 1));
    CK(cudaMemsetAsync(sch.sync, 0, sizeof(int) * (2 + std::max(nl, 1)), s));
}

// The level's rows in sliced ELL form (build_sell), when every row has at
// most 255 neighbours.
void upload_sell(Arena& ar, cudaStream_t s, const HostLevel& h, LevelMesh& m) {
    HostSell hs;
    if (!build_sell(h, amul_sell() == 2, hs)) return;
    m.sellStart = ar.upload(hs.start, s);
    m.sellCnt = ar.upload(hs.cnt, s);
    m.sellCol = ar.upload(hs.col, s);
    m.sellSrc = ar.upload(hs.src, s);
    m.sellPat = ar.upload(hs.pat, s);
    m.sellOffs = hs.offs.empty() ? nullptr : ar.upload(hs.offs, s);
    m.sellEntries = hs.entries;
    m.sellPatterns = hs.patterns;
    m.sellPatternSlices = hs.patternSlices;
}

void upload_level(Arena& ar, cudaStream_t s, const HostLevel& h, LevelMesh& m) {
    m.n = h.n;
    m.nf = h.nf;
    m.l = ar.upload(h.l, s);
    m.u = ar.upload(h.u, s);
    m.ownerStart = ar.upload(h.ownerStart, s);
    m.losortStart = ar.upload(h.losortStart, s);
    m.losort = ar.upload(h.losort, s);
    m.losortL = ar.upload(h.losortL, s);
    upload_schedule(ar, s, h.fwdCells, h.fwdLevelStart, m.fwd);
    upload_schedule(ar, s, h.bwdCells, h.bwdLevelStart, m.bwd);
    upload_sell(ar, s, h, m);
}

// Inverse restriction maps of level h (fine) -> coarse, for the gathers.
void upload_restriction(Arena& ar, cudaStream_t s, const HostLevel& h, LevelMesh& m) {
    const int n = h.n, nf = h.nf, nc = h.nCoarse, ncf = h.nCoarseFaces;
    m.nCoarse = nc;
    m.nCoarseFaces = ncf;
    auto group = [](int nKeys, const std::vector<int>& key, std::vector<int>& start, std::vector<int>& items,
                     bool negative) {
        start.assign(nKeys + 1, 0);
        for (size_t i = 0; i < key.size(); ++i) {
            const int k = key[i];
            if (negative ? k < 0 : k >= 0) start[(negative ? -1 - k : k) + 1]++;
        }
        for (int c = 0; c < nKeys; ++c) start[c + 1] += start[c];
        items.resize(start[nKeys]);
        std::vector<int> fill(start.begin(), start.end() - 1);
        for (size_t i = 0; i < key.size(); ++i) {
            const int k = key[i];
            if (negative ? k < 0 : k >= 0) items[fill[negative ? -1 - k : k]++] = int(i);
        }
    };
    std::vector<int> ccStart, ccFine, cfStart, cfFine, ifStart, ifFine;
    group(nc, h.restrictAddr, ccStart, ccFine, false);
    group(ncf, h.faceRestrict, cfStart, cfFine, false);
    group(nc, h.faceRestrict, ifStart, ifFine, true);
    (void)n;
    (void)nf;
    m.restrictAddr = ar.upload(h.restrictAddr, s);
    m.coarseCellStart = ar.upload(ccStart, s);
    m.coarseCellFine = ar.upload(ccFine, s);
    m.faceRestrict = ar.upload(h.faceRestrict, s);
    m.faceFlip = ar.upload(h.faceFlip, s);
    m.coarseFaceStart = ar.upload(cfStart, s);
    m.coarseFaceFine = ar.upload(cfFine, s);
    m.intFaceStart = ar.upload(ifStart, s);
    m.intFaceFine = ar.upload(ifFine, s);
}

template <class T>
void alloc_coeffs(Arena& ar, const LevelMesh& m, bool sym, LevelCoeffs<T>& c) {
    c.sym = sym;
    c.diag = ar.get<T>(m.n);
    c.upper = ar.get<T>(m.nf);
    c.lower = sym ? nullptr : ar.get<T>(m.nf);
    c.lowerPerm = ar.get<T>(m.nf);
    c.upperPerm = sym ? nullptr : ar.get<T>(m.nf);
    c.rD = ar.get<T>(m.n);
    c.sellCoef = m.sellCol ? ar.get<T>(m.sellEntries) : nullptr;
}

// GAMG hierarchy from level-0 restriction maps (host), then upload.
void build_coarse_interfaces(cfx_mesh* mesh);

cfx_status build_hierarchy(cfx_mesh* mesh, const std::vector<std::vector<int>>& maps, const std::vector<int>& nCoarse) {
    cudaStream_t s = mesh->ctx->stream;
    mesh->host.resize(1);
    for (size_t i = 0; i < maps.size(); ++i) {
        HostLevel& f = mesh->host[i];
        if ((int)maps[i].size() != f.n) {
            set_error("restrict map " + std::to_string(i) + " has wrong size");
            return CFX_ERR_ARG;
        }
        for (int v : maps[i])
            if (v < 0 || v >= nCoarse[i]) {
                set_error("restrict map " + std::to_string(i) + " out of range");
                return CFX_ERR_ARG;
            }
        std::vector<int> cl, cu, fra, flip;
        const int ncf = agglomerate_addressing(f.nf, f.l.data(), f.u.data(), maps[i], nCoarse[i], cl, cu, fra, flip);
        f.restrictAddr = maps[i];
        f.nCoarse = nCoarse[i];
        f.nCoarseFaces = ncf;
        f.faceRestrict = std::move(fra);
        f.faceFlip = std::move(flip);
        HostLevel c;
        CFX_TRY(build_host_level(nCoarse[i], ncf, cl.data(), cu.data(), c, false));
        mesh->host.push_back(std::move(c));
    }
    mesh->nCoarseLevels = int(maps.size());
    mesh->version++;
    // upload: keep level 0's device mesh, rebuild the rest
    mesh->dev.resize(1);
    upload_restriction(mesh->arena, s, mesh->host[0], mesh->dev[0]);
    for (size_t i = 1; i < mesh->host.size(); ++i) {
        LevelMesh m;
        upload_level(mesh->arena, s, mesh->host[i], m);
        if (mesh->host[i].nCoarse > 0) upload_restriction(mesh->arena, s, mesh->host[i], m);
        mesh->dev.push_back(m);
    }
    build_coarse_interfaces(mesh);
    return CFX_OK;
}

// The GAMG levels' cyclic interfaces (cyclicGAMGInterface.C:87-151): on
// each coarse level every patch's faces are grouped by the pair (coarse cell,
// coarse partner cell) in order of first appearance, the partner cell read
// through the partner patch's restricted face cells (its
// internalFieldTransfer); per level, the coarse faces' CSR over cells (in
// patch-then-face order, as updateMatrixInterfaces adds them) and, for the
// coefficient sums (GAMGInterface::agglomerateCoeffs), each coarse face's
// fine faces in ascending order.
// One level's grouping (cyclicGAMGInterface.C:87-151): size/cell/nbr of the
// finer level in patch order and its restriction map R.
void coarse_interface_faces(const int* R, const std::vector<int>& size, const std::vector<int>& cell,
                            const std::vector<int>& nbr, std::vector<int>& cSize, std::vector<int>& cCell,
                            std::vector<int>& cNbr, std::vector<int>& toCoarse) {
    cSize.clear();
    cCell.clear();
    cNbr.clear();
    toCoarse.assign(cell.size(), 0);
    int off = 0;
    for (size_t p = 0; p < size.size(); ++p) {
        const int c0 = int(cCell.size());
        std::map<std::pair<int, int>, int> seen;
        for (int k = off; k < off + size[p]; ++k) {
            const std::pair<int, int> key(R[cell[k]], R[nbr[k]]);
            auto it = seen.find(key);
            if (it == seen.end()) {
                const int j = int(cCell.size());
                seen.emplace(key, j);
                cCell.push_back(key.first);
                cNbr.push_back(key.second);
                toCoarse[k] = j;
            } else {
                toCoarse[k] = it->second;
            }
        }
        cSize.push_back(int(cCell.size()) - c0);
        off += size[p];
    }
}

// LUscalarMatrix::convert's interface entries (LUscalarMatrix.C:236-262) of
// one level: per patch p with partner q and face f, row faceCells_p[f],
// column faceCells_q[f], coefficient interfaceBouCoeffs_q[f] (its CSR
// position).  False when a partner is unknown or of another size.
bool lu_interface_entries(const std::vector<int>& partner, const std::vector<int>& size,
                          const std::vector<int>& cell, const std::vector<int>& pos, std::vector<int>& row,
                          std::vector<int>& col, std::vector<int>& src) {
    const int nP = int(size.size());
    if (int(partner.size()) != nP) return false;
    std::vector<int> off(static_cast<size_t>(nP) + 1, 0);
    for (int p = 0; p < nP; ++p) off[p + 1] = off[p] + size[p];
    row.clear();
    col.clear();
    src.clear();
    for (int p = 0; p < nP; ++p) {
        const int q = partner[p];
        if (q < 0 || q >= nP || size[q] != size[p]) return false;
        for (int f = 0; f < size[p]; ++f) {
            row.push_back(cell[off[p] + f]);
            col.push_back(cell[off[q] + f]);
            src.push_back(pos[off[q] + f]);
        }
    }
    return true;
}

void set_lu_interfaces(cfx_mesh* mesh, LevelMesh& m, const std::vector<int>& size, const std::vector<int>& cell,
                       const std::vector<int>& pos, cudaStream_t s) {
    std::vector<int> row, col, src;
    m.luIfRow = m.luIfCol = m.luIfSrc = nullptr;
    if (!lu_interface_entries(mesh->ifNbrPatch, size, cell, pos, row, col, src)) {
        m.luIfN = -1;
        return;
    }
    m.luIfN = int(row.size());
    m.luIfRow = mesh->ifCoarseArena.upload(row, s);
    m.luIfCol = mesh->ifCoarseArena.upload(col, s);
    m.luIfSrc = mesh->ifCoarseArena.upload(src, s);
}

void build_coarse_interfaces(cfx_mesh* mesh) {
    cudaStream_t s = mesh->ctx->stream;
    CK(cudaStreamSynchronize(s));
    mesh->ifCoarseArena.release();
    const int nl = int(mesh->dev.size());
    for (int i = 0; i < nl; ++i) {
        LevelMesh& m = mesh->dev[i];
        m.luIfN = 0;
        m.luIfRow = m.luIfCol = m.luIfSrc = nullptr;
        if (i == 0) continue;
        m.nIf = 0;
        m.ifStart = m.ifNbr = m.ifcStart = m.ifcFine = nullptr;
    }
    if (!mesh->nIf) return;
    std::vector<int> size = mesh->ifPatchSize, cell = mesh->ifFaceCell, nbr = mesh->ifNbrCell, pos = mesh->ifPos;
    set_lu_interfaces(mesh, mesh->dev[0], size, cell, pos, s);
    for (int i = 1; i < nl; ++i) {
        const int nFine = int(cell.size());
        std::vector<int> cSize, cCell, cNbr, toCoarse;
        coarse_interface_faces(mesh->host[i - 1].restrictAddr.data(), size, cell, nbr, cSize, cCell, cNbr, toCoarse);
        const int n = mesh->host[i].n, nc = int(cCell.size());
        std::vector<int> start(static_cast<size_t>(n) + 1, 0), cnbr(nc), cpos(nc);
        for (int k = 0; k < nc; ++k) start[cCell[k] + 1]++;
        for (int c = 0; c < n; ++c) start[c + 1] += start[c];
        std::vector<int> fill(start.begin(), start.end() - 1);
        for (int k = 0; k < nc; ++k) {
            const int j = fill[cCell[k]]++;
            cnbr[j] = cNbr[k];
            cpos[k] = j;
        }
        std::vector<int> gStart(static_cast<size_t>(nc) + 1, 0), gFine(static_cast<size_t>(nFine));
        for (int k = 0; k < nFine; ++k) gStart[cpos[toCoarse[k]] + 1]++;
        for (int j = 0; j < nc; ++j) gStart[j + 1] += gStart[j];
        std::vector<int> gfill(gStart.begin(), gStart.end() - 1);
        for (int k = 0; k < nFine; ++k) gFine[gfill[cpos[toCoarse[k]]]++] = pos[k];
        LevelMesh& m = mesh->dev[i];
        m.nIf = nc;
        m.ifStart = mesh->ifCoarseArena.upload(start, s);
        m.ifNbr = mesh->ifCoarseArena.upload(cnbr, s);
        m.ifcStart = mesh->ifCoarseArena.upload(gStart, s);
        m.ifcFine = mesh->ifCoarseArena.upload(gFine, s);
        size.swap(cSize);
        cell.swap(cCell);
        nbr.swap(cNbr);
        pos.swap(cpos);
        set_lu_interfaces(mesh, m, size, cell, pos, s);
    }
    CK(cudaStreamSynchronize(s));  // the host vectors are temporaries
}

void set_state(cfx_ctx* ctx, int slot, const cfx_controls& c, double tol, double relTol, int maxIter, int minIter) {
    SolveState h{};
    h.tolerance = tol;
    h.relTol = relTol;
    h.maxIter = maxIter;
    h.minIter = minIter;
    (void)c;
    ctx->h_state[slot] = h;
    CK(cudaMemcpyAsync(ctx->d_state + slot, ctx->h_state + slot, sizeof(SolveState), cudaMemcpyHostToDevice,
                       ctx->stream));
}

SolveState read_state(cfx_ctx* ctx, int slot) {
    CK(cudaMemcpyAsync(ctx->h_state + slot, ctx->d_state + slot, sizeof(SolveState), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return ctx->h_state[slot];
}

int read_status(cfx_ctx* ctx) {
    int h = 0;
    CK(cudaMemcpyAsync(&h, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return h;
}


uint64_t hkey(std::initializer_list<uint64_t> v) {
    uint64_t h = 1469598103934665603ull;
    for (uint64_t x : v) {
        h ^= x;
        h *= 1099511628211ull;
    }
    return h;
}

template <class T>
LevelCoeffs<T>& coeffs(cfx_matrix* mat, int lv);
template <>
LevelCoeffs<double>& coeffs<double>(cfx_matrix* mat, int lv) {
    return mat->c64[lv];
}
template <>
LevelCoeffs<float>& coeffs<float>(cfx_matrix* mat, int lv) {
    return mat->c32[lv];
}

// Ensure coefficients of all levels exist in precision T (coarse assembly on
// device from the level-0 FP64 coefficients; FP32 copies are cast from FP64).
void prepare_levels(cfx_matrix* mat, bool want32) {
    cfx_mesh* mesh = mat->mesh;
    cudaStream_t s = mesh->ctx->stream;
    const int nl = int(mesh->dev.size());
    if ((int)mat->c64.size() < nl) {
        for (int i = int(mat->c64.size()); i < nl; ++i) {
            LevelCoeffs<double> c;
            alloc_coeffs(mat->arena, mesh->dev[i], mat->sym, c);
            mat->c64.push_back(c);
        }
        mat->coarse64 = false;
    }
    if (!mat->coarse64) {
        for (int i = 1; i < nl; ++i) {
            Ops<double>::coarsen(s, mesh->dev[i - 1], mat->c64[i - 1], mesh->dev[i], mat->c64[i]);
            // the coarse interfaces' coefficients
            // (GAMGSolverAgglomerateMatrix.C:196-268)
            const LevelMesh& cm = mesh->dev[i];
            LevelCoeffs<double>& cc = mat->c64[i];
            const LevelCoeffs<double>& fc = mat->c64[i - 1];
            if (cm.nIf && fc.ifBou) {
                if (cc.ifCap < cm.nIf) {
                    cc.ifBou = mat->arena.get<double>(cm.nIf);
                    cc.ifInt = mat->arena.get<double>(cm.nIf);
                    cc.ifCap = cm.nIf;
                }
                Ops<double>::iface_restrict(s, cm, fc.ifBou, cc.ifBou);
                Ops<double>::iface_restrict(s, cm, fc.ifInt ? fc.ifInt : fc.ifBou, cc.ifInt);
            } else {
                cc.ifBou = cc.ifInt = nullptr;
            }
        }
        mat->coarse64 = true;
    }
    if (want32) {
        if ((int)mat->c32.size() < nl) {
            for (int i = int(mat->c32.size()); i < nl; ++i) {
                LevelCoeffs<float> c;
                alloc_coeffs(mat->arena, mesh->dev[i], mat->sym, c);
                mat->c32.push_back(c);
            }
            mat->fine32 = mat->coarse32 = false;
        }
        if (!mat->fine32 || !mat->coarse32) {
            for (int i = 0; i < nl; ++i) {
                const LevelMesh& m = mesh->dev[i];
                launch_cast_d2f(s, m.n, mat->c64[i].diag, mat->c32[i].diag);
                launch_cast_d2f(s, m.nf, mat->c64[i].upper, mat->c32[i].upper);
                launch_cast_d2f(s, m.nf, mat->c64[i].lowerPerm, mat->c32[i].lowerPerm);
                if (m.sellCol) launch_cast_d2f(s, m.sellEntries, mat->c64[i].sellCoef, mat->c32[i].sellCoef);
                if (!mat->sym) {
                    launch_cast_d2f(s, m.nf, mat->c64[i].lower, mat->c32[i].lower);
                    launch_cast_d2f(s, m.nf, mat->c64[i].upperPerm, mat->c32[i].upperPerm);
                }
                // the interface coefficients of the FP32 inner solves
                LevelCoeffs<float>& f32 = mat->c32[i];
                const LevelCoeffs<double>& f64 = mat->c64[i];
                if (m.nIf && f64.ifBou) {
                    if (f32.ifCap < m.nIf) {
                        f32.ifBou = mat->arena.get<float>(m.nIf);
                        f32.ifInt = mat->arena.get<float>(m.nIf);
                        f32.ifCap = m.nIf;
                    }
                    launch_cast_d2f(s, m.nIf, f64.ifBou, f32.ifBou);
                    launch_cast_d2f(s, m.nIf, f64.ifInt ? f64.ifInt : f64.ifBou, f32.ifInt);
                } else {
                    f32.ifBou = f32.ifInt = nullptr;
                }
            }
            mat->fine32 = mat->coarse32 = true;
        }
    }
}

void invalidate_packs(cfx_matrix* mat);

void coefficients_changed(cfx_matrix* mat) {
    Ops<double>::permute(mat->mesh->ctx->stream, mat->mesh->dev[0], mat->c64[0]);
    mat->coarse64 = mat->coarse32 = mat->fine32 = false;
    invalidate_packs(mat);
}

void set_coefficients(cfx_matrix* mat, const double* diag, const double* upper, const double* lower,
                      cudaMemcpyKind kind) {
    cfx_mesh* mesh = mat->mesh;
    cudaStream_t s = mesh->ctx->stream;
    const LevelMesh& m = mesh->dev[0];
    LevelCoeffs<double>& c = mat->c64[0];
    CK(cudaMemcpyAsync(c.diag, diag, sizeof(double) * m.n, kind, s));
    if (m.nf && upper) CK(cudaMemcpyAsync(c.upper, upper, sizeof(double) * m.nf, kind, s));
    if (m.nf && !upper) CK(cudaMemsetAsync(c.upper, 0, sizeof(double) * m.nf, s));  // diagonal matrix
    if (!mat->sym && m.nf) CK(cudaMemcpyAsync(c.lower, lower, sizeof(double) * m.nf, kind, s));
    coefficients_changed(mat);
}

// ---- packed sweep schedules and coefficients ------------------------------
DevSched upload_sched(Arena& ar, cudaStream_t s, const HostSched& h) {
    DevSched d;
    d.kind = h.kind;
    d.nSweeps = h.nSweeps;
    d.nLevels = h.nLevels;
    d.n = h.n;
    d.maxK = h.maxK;
    d.nSlots = int(h.cell.size());
    d.nEntries = int(h.nb.size());
    d.nGroups = int(h.groupEntry.size()) - 1;
    d.nChunks = int(h.chunkLevel.size());
    d.maxLevelBytes8 = h.maxLevelBytes8;
    d.levelSlot = ar.upload(h.levelSlot, s);
    d.levelEntry = ar.upload(h.levelEntry, s);
    d.groupEntry = ar.upload(h.groupEntry, s);
    d.cell = ar.upload(h.cell, s);
    d.cnt = ar.upload(h.cnt, s);
    d.nb = ar.upload(h.nb, s);
    d.src = ar.upload(h.src, s);
    d.chunkGroup = ar.upload(h.chunkGroup, s);
    d.chunkLevel = ar.upload(h.chunkLevel, s);
    d.levelChunks = ar.upload(h.levelChunks, s);
    d.depStart = ar.upload(h.depStart, s);
    d.dep = ar.upload(h.dep, s);
    d.slotSweep = ar.upload(h.slotSweep, s);
    d.slotLower = ar.upload(h.slotLower, s);
    d.gdone = ar.get<int>(std::max(d.nGroups, 1));
    d.waveOk = h.waveOk ? 1 : 0;
    d.levelLaunch = h.nLevels <= LVL_LAUNCH_MAX ? 1 : 0;
    if (d.levelLaunch) {
        d.hLvlPart[0] = 0;
        for (int L = 0; L <= h.nLevels; ++L) {
            d.hLvlSlot[L] = h.levelSlot[L];
            if (L < h.nLevels) {
                const int groups = (h.levelSlot[L + 1] - h.levelSlot[L]) / 32;
                d.hLvlPart[L + 1] = d.hLvlPart[L] + (groups + LVL_LAUNCH_GROUPS - 1) / LVL_LAUNCH_GROUPS;
            }
        }
    }
    d.sync = ar.get<int>(2 + size_t(LVL_STRIDE_MAX) * std::max(h.nLevels, 1));
    CK(cudaMemsetAsync(d.sync, 0, sizeof(int) * (2 + size_t(LVL_STRIDE_MAX) * std::max(h.nLevels, 1)), s));
    return d;
}

// A level's schedule, built on first use and kept with the mesh.
DevSched build_and_upload(cfx_mesh* mesh, int lv, int kind, int S) {
    HostSched h;
    build_sched(mesh->host[lv], kind, S, h, sweep_wave() != 0);
    return upload_sched(mesh->schedArena, mesh->ctx->stream, h);
}

// Schedule of level lv (kind SCHED_*, S combined Gauss-Seidel sweeps).
const DevSched& sched(cfx_mesh* mesh, int lv, int kind, int S = 1) {
    if ((int)mesh->sched.size() < (int)mesh->host.size()) mesh->sched.resize(mesh->host.size());
    cfx_mesh::Scheds& sc = mesh->sched[lv];
    if (kind == SCHED_FWD) {
        if (!sc.hasFwd) {
            sc.fwd = build_and_upload(mesh, lv, SCHED_FWD, 1);
            sc.hasFwd = true;
        }
        return sc.fwd;
    }
    if (kind == SCHED_BWD) {
        if (!sc.hasBwd) {
            sc.bwd = build_and_upload(mesh, lv, SCHED_BWD, 1);
            sc.hasBwd = true;
        }
        return sc.bwd;
    }
    // Gauss-Seidel schedules by sweep count; key -1 = the backward pass
    if (kind == SCHED_GSB) S = -1;
    auto it = sc.gs.find(S);
    if (it == sc.gs.end())
        it = sc.gs.emplace(S, S < 0 ? build_and_upload(mesh, lv, SCHED_GSB, 1)
                                    : build_and_upload(mesh, lv, SCHED_GS, S)).first;
    return it->second;
}

// The multicolour forward or backward schedule of level lv (kind SCHED_FWD
// or SCHED_BWD), built on first use.
const DevSched& sched_pre_colored(cfx_mesh* mesh, int lv, int kind) {
    if ((int)mesh->sched.size() < (int)mesh->host.size()) mesh->sched.resize(mesh->host.size());
    cfx_mesh::Scheds& sc = mesh->sched[lv];
    const bool fwd = kind == SCHED_FWD;
    if (!(fwd ? sc.hasFwdC : sc.hasBwdC)) {
        std::vector<int> color;
        greedy_colors(mesh->host[lv], color);
        HostSched h;
        build_sched(mesh->host[lv], kind, 1, h, false, &color);
        (fwd ? sc.fwdC : sc.bwdC) = upload_sched(mesh->schedArena, mesh->ctx->stream, h);
        (fwd ? sc.hasFwdC : sc.hasBwdC) = true;
    }
    return fwd ? sc.fwdC : sc.bwdC;
}

// Whether precision T's DIC (sym) / DILU take the multicolour order
// (colored_pre(): 1 DIC in the FP32 inner solves, 2 DIC and DILU in the
// FP32 inner solves, 3 both in every solve).
template <class T>
bool pre_colored(bool sym) {
    const int k = colored_pre();
    if (k == 3) return true;
    return k > 0 && sizeof(T) == 4 && (sym || k == 2);
}

// The forward / backward schedule DIC and DILU of precision T run on.
template <class T>
const DevSched& sched_pre(cfx_mesh* mesh, int lv, int kind, bool col) {
    return col ? sched_pre_colored(mesh, lv, kind) : sched(mesh, lv, kind);
}

// The multicolour Gauss-Seidel schedule of level lv (S combined sweeps),
// built on first use; kept under key COLORED_KEY + S.
constexpr int COLORED_KEY = 1 << 16;
const DevSched& sched_colored(cfx_mesh* mesh, int lv, int S) {
    if ((int)mesh->sched.size() < (int)mesh->host.size()) mesh->sched.resize(mesh->host.size());
    cfx_mesh::Scheds& sc = mesh->sched[lv];
    auto it = sc.gs.find(COLORED_KEY + S);
    if (it == sc.gs.end()) {
        std::vector<int> color;
        greedy_colors(mesh->host[lv], color);
        HostSched h;
        build_sched(mesh->host[lv], SCHED_GS, S, h, false, &color);
        it = sc.gs.emplace(COLORED_KEY + S, upload_sched(mesh->schedArena, mesh->ctx->stream, h)).first;
    }
    return it->second;
}

// Whether precision T's Gauss-Seidel smoothing takes the multicolour order
// (colored_gs(): 1 for the FP32 inner cycles, 2 for every smoothing).
template <class T>
bool gs_colored() {
    return colored_gs() == 2 || (colored_gs() == 1 && sizeof(T) == 4);
}

template <class T>
std::vector<LevelPack<T>>& packs_of(cfx_matrix* mat);
template <>
std::vector<LevelPack<double>>& packs_of<double>(cfx_matrix* mat) {
    return mat->p64;
}
template <>
std::vector<LevelPack<float>>& packs_of<float>(cfx_matrix* mat) {
    return mat->p32;
}

template <class T>
Packed<T>& packed(cfx_matrix* mat, int lv, int op, int S, const DevSched& sd, int colPre = -1) {
    auto& v = packs_of<T>(mat);
    if ((int)v.size() <= lv) v.resize(lv + 1);
    LevelPack<T>& lp = v[lv];
    // the forward, backward and pivot packs of the multicolour schedules
    // are kept apart (their entry counts differ)
    const bool col = op != OP_GS && (colPre < 0 ? pre_colored<T>(mat->sym) : colPre != 0);
    Packed<T>* p = op == OP_RD ? (col ? &lp.rdC : &lp.rd)
                 : op == OP_FWD ? (col ? &lp.fwdC : &lp.fwd)
                 : op == OP_BWD ? (col ? &lp.bwdC : &lp.bwd) : &lp.gs[S];
    if (!p->coef) {
        p->coef = mat->arena.get<T>(sd.nEntries);
        p->scalar = mat->arena.get<T>(sd.nSlots);
        p->inS = mat->arena.get<T>(sd.nSlots);
    }
    const size_t fv = sweep_flow_values(sd, op);
    if (fv && !p->flow) p->flow = mat->arena.get<T>(fv);
    return *p;
}

// The transpose's DILU packs (forward: rD*upper of the neighbour faces,
// backward: rD*lower of the owned faces) for preconditionT.
template <class T>
Packed<T>& packedT(cfx_matrix* mat, int lv, int op, const DevSched& sd) {
    auto& v = packs_of<T>(mat);
    if ((int)v.size() <= lv) v.resize(lv + 1);
    const bool col = pre_colored<T>(mat->sym);
    Packed<T>* p = op == OP_FWD ? (col ? &v[lv].fwdTC : &v[lv].fwdT) : (col ? &v[lv].bwdTC : &v[lv].bwdT);
    if (!p->coef) {
        p->coef = mat->arena.get<T>(sd.nEntries);
        p->scalar = mat->arena.get<T>(sd.nSlots);
        p->inS = mat->arena.get<T>(sd.nSlots);
    }
    const size_t fv = sweep_flow_values(sd, op);
    if (fv && !p->flow) p->flow = mat->arena.get<T>(fv);
    return *p;
}

void invalidate_packs(cfx_matrix* mat) {
    for (auto& l : mat->p64) {
        l.rd.valid = l.fwd.valid = l.bwd.valid = l.fwdT.valid = l.bwdT.valid = false;
        l.rdC.valid = l.fwdC.valid = l.bwdC.valid = l.fwdTC.valid = l.bwdTC.valid = false;
        for (auto& kv : l.gs) kv.second.valid = false;
    }
    for (auto& l : mat->p32) {
        l.rd.valid = l.fwd.valid = l.bwd.valid = l.fwdT.valid = l.bwdT.valid = false;
        l.rdC.valid = l.fwdC.valid = l.bwdC.valid = l.fwdTC.valid = l.bwdTC.valid = false;
        for (auto& kv : l.gs) kv.second.valid = false;
    }
}

void ensure_chunk_partials(cfx_ctx* ctx, size_t chunks) {
    const size_t need = std::max<size_t>(chunks, RED_MAXB) + 16;
    if (ctx->sc.chunkPartialsCap < need) {
        ctx->sc.chunkPartials = ctx->arena.get<double>(need);
        ctx->sc.chunkPartialsCap = need;
    }
}

// rD of DIC / DILU (DICPreconditioner.C:57-84, DILUPreconditioner.C:57-85):
// pivot sweep in level order, then the reciprocal; then the forward and
// backward coefficients (rD_c*lower, rD_c*upper) are packed.  col: in the
// multicolour order (the coarsest level's one-CTA solve sweeps in the
// reference's order and takes the reference's pivots).
template <class T>
void compute_rD(cfx_matrix* mat, int lv, int colored = -1) {
    const bool col = colored < 0 ? pre_colored<T>(mat->sym) : colored != 0;
    cfx_ctx* ctx = mat->mesh->ctx;
    cudaStream_t s = ctx->stream;
    const LevelMesh& m = mat->mesh->dev[lv];
    LevelCoeffs<T>& c = coeffs<T>(mat, lv);
    const DevSched& f = sched_pre<T>(mat->mesh, lv, SCHED_FWD, col);
    const DevSched& b = sched_pre<T>(mat->mesh, lv, SCHED_BWD, col);
    // dot partials of the fused backward sweep: one per chunk or per
    // dataflow CTA, whichever form runs
    ensure_chunk_partials(ctx, std::max({size_t(f.nChunks), size_t(b.nChunks), size_t(sweep_partials<T>(b)),
                                         size_t(sweep_partials<T>(f))}));
    Packed<T>& prd = packed<T>(mat, lv, OP_RD, 1, f, int(col));
    pack_sweep<T>(s, f, OP_RD, c, prd);
    if (run_sweep<T>(s, f, OP_RD, prd, nullptr, c.rD, nullptr, nullptr, nullptr, ctx->d_status) != CFX_OK)
        throw CudaError(last_error());
    Ops<T>::reciprocal(s, m.n, c.rD);
    pack_sweep<T>(s, f, OP_FWD, c, packed<T>(mat, lv, OP_FWD, 1, f, int(col)));
    pack_sweep<T>(s, b, OP_BWD, c, packed<T>(mat, lv, OP_BWD, 1, b, int(col)));
}

template <class T>
void diag_reciprocal(cfx_ctx* ctx, const LevelMesh& m, LevelCoeffs<T>& c) {
    Kern<T>::copy(ctx->stream, m.n, c.diag, c.rD, nullptr);
    Ops<T>::reciprocal(ctx->stream, m.n, c.rD);
}

template <class T>
int pc_gamg_apply(cfx_matrix* mat, const T* r, T* w, const int* done, bool dot);
template <class T>
void pc_gamg_setup(cfx_matrix* mat);

// w = M^-1 r with the w.r dot partials in ctx->sc.chunkPartials when dot.
// Returns the number of partials.  DIC/DILU packs must be current
// (compute_rD).
template <class T>
int precondition(cfx_matrix* mat, int lv, int kind, const T* r, T* w, const int* done, bool dot) {
    cfx_ctx* ctx = mat->mesh->ctx;
    cudaStream_t s = ctx->stream;
    const LevelMesh& m = mat->mesh->dev[lv];
    LevelCoeffs<T>& c = coeffs<T>(mat, lv);
    if (kind == CFX_PRE_GAMG) return pc_gamg_apply<T>(mat, r, w, done, dot);
    if (kind == CFX_PRE_DIC || kind == CFX_PRE_DILU) {
        const DevSched& f = sched_pre<T>(mat->mesh, lv, SCHED_FWD, pre_colored<T>(mat->sym));
        const DevSched& b = sched_pre<T>(mat->mesh, lv, SCHED_BWD, pre_colored<T>(mat->sym));
        if (run_sweep<T>(s, f, OP_FWD, packed<T>(mat, lv, OP_FWD, 1, f), r, w, nullptr, nullptr, done,
                         ctx->d_status) != CFX_OK)
            throw CudaError(last_error());
        if (run_sweep<T>(s, b, OP_BWD, packed<T>(mat, lv, OP_BWD, 1, b), nullptr, w, dot ? r : nullptr,
                         ctx->sc.chunkPartials, done, ctx->d_status) != CFX_OK)
            throw CudaError(last_error());
        return sweep_partials<T>(b);
    }
    Kern<T>::precond_pointwise(s, m.n, kind == CFX_PRE_DIAGONAL ? c.rD : nullptr, r, w, ctx->sc.chunkPartials,
                               done);
    int g = (m.n + RED_NT - 1) / RED_NT;
    return std::max(1, std::min(g, RED_MAXB));
}

// DILUPreconditioner::preconditionT (DILUPreconditioner.C:138-185) is the
// DILU sweep pair of the transpose: the forward pass subtracts
// rD[u]*upper*w[l] per cell in face order (the order the losort forward
// pass of precondition uses for lower), the backward pass rD[l]*lower*w[u]
// in the reverse order of the owned faces, and rD (upper*lower products)
// is the same.  Other preconditioners' preconditionT is precondition.
template <class T>
void preconditionT(cfx_matrix* mat, int lv, int kind, const T* r, T* w, const int* done) {
    if (kind != CFX_PRE_DILU) {
        precondition<T>(mat, lv, kind, r, w, done, false);
        return;
    }
    cfx_ctx* ctx = mat->mesh->ctx;
    cudaStream_t s = ctx->stream;
    const DevSched& f = sched_pre<T>(mat->mesh, lv, SCHED_FWD, pre_colored<T>(mat->sym));
    const DevSched& b = sched_pre<T>(mat->mesh, lv, SCHED_BWD, pre_colored<T>(mat->sym));
    if (run_sweep<T>(s, f, OP_FWD, packedT<T>(mat, lv, OP_FWD, f), r, w, nullptr, nullptr, done, ctx->d_status) !=
        CFX_OK)
        throw CudaError(last_error());
    if (run_sweep<T>(s, b, OP_BWD, packedT<T>(mat, lv, OP_BWD, b), nullptr, w, nullptr, nullptr, done,
                     ctx->d_status) != CFX_OK)
        throw CudaError(last_error());
}

// Packs for preconditionT of DILU (compute_rD must have run).
template <class T>
void setup_preconditioner_t(cfx_matrix* mat, int lv, int kind) {
    if (kind != CFX_PRE_DILU) return;
    cudaStream_t s = mat->mesh->ctx->stream;
    const LevelCoeffs<T>& c = coeffs<T>(mat, lv);
    LevelCoeffs<T> t = c;  // the transpose: upper <-> lower
    t.sym = false;
    t.lower = c.upper;
    t.upper = c.lower;
    t.lowerPerm = c.upperPerm;
    t.upperPerm = c.lowerPerm;
    t.sellCoef = nullptr;
    const DevSched& f = sched_pre<T>(mat->mesh, lv, SCHED_FWD, pre_colored<T>(mat->sym));
    const DevSched& b = sched_pre<T>(mat->mesh, lv, SCHED_BWD, pre_colored<T>(mat->sym));
    pack_sweep<T>(s, f, OP_FWD, t, packedT<T>(mat, lv, OP_FWD, f));
    pack_sweep<T>(s, b, OP_BWD, t, packedT<T>(mat, lv, OP_BWD, b));
}

template <class T>
void setup_preconditioner(cfx_matrix* mat, int lv, int kind) {
    cfx_ctx* ctx = mat->mesh->ctx;
    if (kind == CFX_PRE_DIC || kind == CFX_PRE_DILU) {
        compute_rD<T>(mat, lv);
    } else if (kind == CFX_PRE_DIAGONAL) {
        diag_reciprocal<T>(ctx, mat->mesh->dev[lv], coeffs<T>(mat, lv));
    } else if (kind == CFX_PRE_GAMG) {
        pc_gamg_setup<T>(mat);
    }
    ensure_chunk_partials(ctx, RED_MAXB);
}

// Gauss-Seidel coefficients for S fused sweeps on level lv (colored: the
// multicolour schedule's).
template <class T>
void prepare_gs(cfx_matrix* mat, int lv, int S, bool colored = false) {
    const DevSched& g = colored ? sched_colored(mat->mesh, lv, S) : sched(mat->mesh, lv, SCHED_GS, S);
    Packed<T>& p = packed<T>(mat, lv, OP_GS, colored ? COLORED_KEY + S : S, g);
    if (!p.valid) pack_sweep<T>(mat->mesh->ctx->stream, g, OP_GS, coeffs<T>(mat, lv), p);
}

constexpr int MAX_FUSED_SWEEPS = 4;

// ----------------------------------------------------------- PCG / PBiCGStab
// One Krylov solve in precision T on level lv of the matrix.  psi/b are T
// device vectors; state in slot.
template <class T>
cfx_status krylov(cfx_matrix* mat, Work<T>& W, GraphCache& gc, int lv, int solver, int precond, T* psi, const T* b,
                  int slot, double tol, double relTol, int maxIter, int minIter, const cfx_controls& ctl,
                  SolveState* out) {
    cfx_ctx* ctx = mat->mesh->ctx;
    cudaStream_t s = ctx->stream;
    const LevelMesh& m = mat->mesh->dev[lv];
    LevelCoeffs<T>& c = coeffs<T>(mat, lv);
    const int n = m.n;
    W.n = std::max(W.n, n);
    SolveState* st = ctx->d_state + slot;
    set_state(ctx, slot, ctl, tol, relTol, maxIter, minIter);
    T* r = W.get(0, n);
    T* w = W.get(1, n);
    T* p = W.get(2, n);
    T* r0 = solver == CFX_SOLVER_PBICGSTAB ? W.get(3, n) : nullptr;
    // Apsi into w; normFactor; r = b - Apsi
    launch_reduce<T>(s, ctx->sc, 0, n, psi, nullptr, &st->red0);
    count_launch();
    Ops<T>::amul(s, m, c, psi, w);
    Kern<T>::norm_init(s, ctx->sc, m, c, w, b, r, r0, st);
    setup_preconditioner<T>(mat, lv, precond);
    const int* done = &st->done;
    int iters = 0;
    if (solver == CFX_SOLVER_PBICGSTAB)
        for (int i = 4; i < 8; ++i) W.get(i, n);
    T *rT = nullptr, *wT = nullptr, *pT = nullptr;
    if (solver == CFX_SOLVER_PBICG) {
        // PBiCG.C:108-125: rT = source - A^T psi (pT starts at zero; the
        // first iteration overwrites it)
        rT = W.get(20, n);
        wT = W.get(21, n);
        pT = W.get(22, n);
        setup_preconditioner_t<T>(mat, lv, precond);
        Ops<T>::tmul(s, m, c, psi, wT);
        Kern<T>::copy(s, n, b, rT, nullptr);
        Kern<T>::axpy(s, n, T(-1), wT, rT, nullptr);
        Kern<T>::fill(s, n, T(0), pT, nullptr);
    }
    uint64_t pcKey = 0;
    if (precond == CFX_PRE_GAMG) {
        double pt = ctl.pcTolerance, pr = ctl.pcRelTol;
        uint64_t a = 0, b2 = 0;
        std::memcpy(&a, &pt, 8);
        std::memcpy(&b2, &pr, 8);
        pcKey = hkey({a, b2, uint64_t(ctl.nVcycles), uint64_t(ctl.smoother), uint64_t(ctl.nPreSweeps),
                      uint64_t(ctl.nPostSweeps), uint64_t(ctl.nFinestSweeps), uint64_t(ctl.maxPreSweeps),
                      uint64_t(ctl.maxPostSweeps), uint64_t(ctl.preSweepsLevelMultiplier),
                      uint64_t(ctl.postSweepsLevelMultiplier), uint64_t(ctl.scaleCorrection + 7),
                      uint64_t(ctl.interpolateCorrection), uint64_t(ctl.directSolveCoarsest),
                      uint64_t(mat->mesh->nCoarseLevels)});
    }
    const uint64_t key = hkey({mat->mesh->version, pcKey, uint64_t(small_sweep_threshold()), uint64_t(cluster_global_cells()), uint64_t(sweep_cluster_size()), uint64_t(sweep_cluster_pre()), uint64_t(sweep_flow()), uint64_t(sweep_flow_ahead()), uint64_t(amul_sell()), uint64_t(sweep_grid_stride()), uint64_t(sweep_grid_poll_ns()), uint64_t(sweep_cta_xl()), uint64_t(colored_gs()), uint64_t(colored_pre()), uint64_t(sweep_level_launch()), uint64_t(sweep_smem_cap()), uint64_t(sweep_wave()), uint64_t(sched_chunk_groups()), uint64_t(lv), uint64_t(solver), uint64_t(precond), uint64_t(slot), uint64_t(n),
                               reinterpret_cast<uint64_t>(psi), reinterpret_cast<uint64_t>(b),
                               reinterpret_cast<uint64_t>(r), reinterpret_cast<uint64_t>(c.rD),
                               reinterpret_cast<uint64_t>(c.ifBou), reinterpret_cast<uint64_t>(m.ifStart)});
    auto body = [&]() {
        if (solver == CFX_SOLVER_PCG) {
            const int np = precondition<T>(mat, lv, precond, r, w, done, true);
            Kern<T>::pcg_beta(s, np, ctx->sc.chunkPartials, st);
            Kern<T>::pcg_p(s, n, w, p, st);
            Kern<T>::pcg_amul(s, ctx->sc, m, c, p, w, st);
            Kern<T>::pcg_update(s, ctx->sc, n, p, w, psi, r, st);
        } else if (solver == CFX_SOLVER_PBICG) {
            // PBiCG.C:131-200
            precondition<T>(mat, lv, precond, r, w, done, false);
            preconditionT<T>(mat, lv, precond, rT, wT, done);
            launch_reduce<T>(s, ctx->sc, 3, n, w, rT, ctx->sc.chunkPartials);  // wArT
            count_launch();
            Kern<T>::pcg_beta(s, 1, ctx->sc.chunkPartials, st);
            Kern<T>::pbicg_p(s, n, w, wT, p, pT, st);
            Ops<T>::amul(s, m, c, p, w);
            Kern<T>::pbicg_tmul(s, ctx->sc, m, c, pT, wT, w, st);
            Kern<T>::pbicg_update(s, ctx->sc, n, p, w, wT, psi, r, rT, st);
        } else {
            T* AyA = W.get(4, n);
            T* sA = W.get(5, n);
            T* zA = W.get(6, n);
            T* tA = W.get(7, n);
            T* yA = w;
            Kern<T>::bicg_rho(s, ctx->sc, n, r0, r, st);
            Kern<T>::bicg_p(s, n, r, AyA, p, st);
            precondition<T>(mat, lv, precond, p, yA, done, false);
            Kern<T>::bicg_amul_alpha(s, ctx->sc, m, c, yA, AyA, r0, st);
            Kern<T>::bicg_s(s, ctx->sc, n, r, AyA, sA, st);
            Kern<T>::bicg_early(s, n, yA, psi, st);
            precondition<T>(mat, lv, precond, sA, zA, done, false);
            Kern<T>::bicg_amul_omega(s, ctx->sc, m, c, zA, tA, sA, st);
            Kern<T>::bicg_update(s, ctx->sc, n, yA, zA, sA, tA, psi, r, st);
        }
    };
    // first read: was it converged at start?
    SolveState h = read_state(ctx, slot);
    int batch = 4;
    while (!h.done) {
        for (int k = 0; k < batch; ++k) graph_launch(gc, key, s, body);
        iters += batch;
        h = read_state(ctx, slot);
        const int stc = read_status(ctx);
        if (stc != 0) return cfx_status(stc);
        batch = std::min(64, std::max(4, h.nIterations / 4));
        if (iters > 4 * maxIter + 1024) {
            set_error("iteration loop did not terminate");
            return CFX_ERR_STATE;
        }
        if (ctx->yield && !h.done) ctx->yield(ctx->yieldArg);
    }
    *out = h;
    return CFX_OK;
}

// ---------------------------------------------------------------------- GAMG
// nSweeps of GaussSeidel (fused in passes of up to MAX_FUSED_SWEEPS, packs
// prepared by prepare_gs) or DIC (packs prepared by compute_rD).
template <class T>
void smooth(cfx_ctx* ctx, cfx_matrix* mat, int lv, int kind, T* psi, const T* b, int nSweeps, Work<T>& LW) {
    const LevelMesh& m = mat->mesh->dev[lv];
    LevelCoeffs<T>& c = coeffs<T>(mat, lv);
    cudaStream_t s = ctx->stream;
    if (kind == CFX_SMOOTH_DICGS || kind == CFX_SMOOTH_DILUGS) {
        // DICGaussSeidelSmoother.C:79-92, DILUGaussSeidelSmoother.C:79-92
        smooth<T>(ctx, mat, lv, kind == CFX_SMOOTH_DICGS ? CFX_SMOOTH_DIC : CFX_SMOOTH_DILU, psi, b, nSweeps, LW);
        smooth<T>(ctx, mat, lv, CFX_SMOOTH_GS, psi, b, nSweeps, LW);
        return;
    }
    if (kind == CFX_SMOOTH_SYMGS) {
        // symGaussSeidelSmoother.C:130-199: a forward pass, then a backward
        // pass over the reverse order starting from the forward bPrime, which
        // is the same per-cell formula on the upper-neighbour DAG
        // With coupled interfaces both passes start from bPrime = source
        // minus the (negated) interface terms of psi at the sweep's start.
        const DevSched& f = sched(mat->mesh, lv, SCHED_GS, 1);
        const DevSched& g = sched(mat->mesh, lv, SCHED_GSB, 1);
        const Iface<T> itf = if_bou(m, c);
        for (int k = 0; k < nSweeps; ++k) {
            const T* bk = b;
            if (itf.start) {
                T* bp = LW.get(2, m.n);
                Ops<T>::iface_bprime(s, m.n, itf, b, psi, bp);
                bk = bp;
            }
            if (run_sweep<T>(s, f, OP_GS, packed<T>(mat, lv, OP_GS, 1, f), bk, psi, nullptr, nullptr, nullptr,
                             ctx->d_status) != CFX_OK ||
                run_sweep<T>(s, g, OP_GS, packed<T>(mat, lv, OP_GS, -1, g), bk, psi, nullptr, nullptr, nullptr,
                             ctx->d_status) != CFX_OK)
                throw CudaError(last_error());
        }
        return;
    }
    if (kind == CFX_SMOOTH_GS && if_bou(m, c).start) {
        // GaussSeidelSmoother.C:118-177 with coupled interfaces: each sweep
        // starts from bPrime = source - (-bou)*psi[nbr] (psi at the sweep's
        // start), so the sweeps are not fused
        const DevSched& g = sched(mat->mesh, lv, SCHED_GS, 1);
        T* bp = LW.get(2, m.n);
        for (int k = 0; k < nSweeps; ++k) {
            Ops<T>::iface_bprime(s, m.n, if_bou(m, c), b, psi, bp);
            if (run_sweep<T>(s, g, OP_GS, packed<T>(mat, lv, OP_GS, 1, g), bp, psi, nullptr, nullptr, nullptr,
                             ctx->d_status) != CFX_OK)
                throw CudaError(last_error());
        }
        return;
    }
    if (kind == CFX_SMOOTH_GS) {
        // GaussSeidelSmoother.C:125-177; the FP32 inner cycles of the
        // mixed-precision solves (by default) in the multicolour order
        const bool colored = gs_colored<T>();
        for (int left = nSweeps; left > 0;) {
            const int S = std::min(left, MAX_FUSED_SWEEPS);
            const DevSched& g = colored ? sched_colored(mat->mesh, lv, S) : sched(mat->mesh, lv, SCHED_GS, S);
            Packed<T>& p = packed<T>(mat, lv, OP_GS, colored ? COLORED_KEY + S : S, g);
            if (run_sweep<T>(s, g, OP_GS, p, b, psi, nullptr, nullptr, nullptr, ctx->d_status) != CFX_OK)
                throw CudaError(last_error());
            left -= S;
        }
        return;
    }
    for (int k = 0; k < nSweeps; ++k) {
        // DICSmoother.C:86-115, DILUSmoother.C:86-117: rA = b - A psi;
        // rA = M^-1 rA; psi += rA
        T* rA = LW.get(0, m.n);
        T* wA = LW.get(1, m.n);
        Ops<T>::residual(s, m, c, psi, b, rA);
        precondition<T>(mat, lv, kind == CFX_SMOOTH_DILU ? CFX_PRE_DILU : CFX_PRE_DIC, rA, wA, nullptr, false);
        Kern<T>::axpy(s, m.n, T(1), wA, psi, nullptr);
    }
}

// Set up what smooth() needs on level lv for nSweeps (outside graph capture).
template <class T>
void prepare_smooth(cfx_matrix* mat, int lv, int kind, int nSweeps, Work<T>& LW) {
    if (kind == CFX_SMOOTH_DICGS || kind == CFX_SMOOTH_DILUGS) {
        prepare_smooth<T>(mat, lv, kind == CFX_SMOOTH_DICGS ? CFX_SMOOTH_DIC : CFX_SMOOTH_DILU, nSweeps, LW);
        prepare_smooth<T>(mat, lv, CFX_SMOOTH_GS, nSweeps, LW);
        return;
    }
    const bool itf = if_bou(mat->mesh->dev[lv], coeffs<T>(mat, lv)).start != nullptr;
    if (itf && (kind == CFX_SMOOTH_SYMGS || kind == CFX_SMOOTH_GS)) LW.get(2, mat->mesh->dev[lv].n);
    if (kind == CFX_SMOOTH_SYMGS) {
        prepare_gs<T>(mat, lv, 1);
        const DevSched& g = sched(mat->mesh, lv, SCHED_GSB, 1);
        Packed<T>& p = packed<T>(mat, lv, OP_GS, -1, g);
        if (!p.valid) pack_sweep<T>(mat->mesh->ctx->stream, g, OP_GS, coeffs<T>(mat, lv), p);
        return;
    }
    if (kind == CFX_SMOOTH_GS && itf) {
        prepare_gs<T>(mat, lv, 1);
        return;
    }
    if (kind == CFX_SMOOTH_GS) {
        for (int left = nSweeps; left > 0;) {
            const int S = std::min(left, MAX_FUSED_SWEEPS);
            prepare_gs<T>(mat, lv, S, gs_colored<T>());
            left -= S;
        }
    } else {
        LW.get(0, mat->mesh->dev[lv].n);
        LW.get(1, mat->mesh->dev[lv].n);
    }
}

// GAMGSolver::scale (GAMGSolverScale.C:31-76), optionally adding `pre`.
template <class T>
void scale(cfx_ctx* ctx, cfx_matrix* mat, int lv, T* field, T* Acf, const T* source, const T* pre, SolveState* st) {
    const LevelMesh& m = mat->mesh->dev[lv];
    LevelCoeffs<T>& c = coeffs<T>(mat, lv);
    Kern<T>::gamg_scale_sf(ctx->stream, ctx->sc, m, c, field, Acf, source, st);
    Kern<T>::gamg_scale_apply(ctx->stream, m.n, field, Acf, source, c.diag, pre, st);
}

template <class T>
struct GamgCycle {
    cfx_ctx* ctx;
    cfx_matrix* mat;
    const cfx_controls* ctl;
    int coarsest;         // index of the coarsest coarse level li (matrix level coarsest+1)
    bool scaleCorr;
    bool interp;  // interpolateCorrection
    T* lu = nullptr;  // directSolveCoarsest: the factorised coarsest matrix
    int* piv = nullptr;
    std::vector<T*> corr, src;
    T *Apsi, *fcorr, *scratch2;
    BlockSys<T>* d_blk;
    SolveState* st;

    // One V-cycle (GAMGSolverSolve.C:148-443) for psi with source b and
    // current finest residual fres.
    void enqueue(T* psi, const T* b, const T* fres) {
        cudaStream_t s = ctx->stream;
        cfx_mesh* mesh = mat->mesh;
        const int smoother = ctl->smoother;
        Ops<T>::restrict_field(s, mesh->dev[0], fres, src[0]);
        for (int li = 0; li < coarsest; ++li) {
            const int lv = li + 1;
            const int nc = mesh->dev[lv].n;
            if (ctl->nPreSweeps) {
                Kern<T>::fill(s, nc, T(0), corr[li], nullptr);
                smooth<T>(ctx, mat, lv, smoother, corr[li], src[li],
                          std::min(ctl->nPreSweeps + ctl->preSweepsLevelMultiplier * li, ctl->maxPreSweeps),
                          workFor(lv));
                if (scaleCorr && li < coarsest - 1) scale<T>(ctx, mat, lv, corr[li], Apsi, src[li], nullptr, st);
                Ops<T>::amul(s, mesh->dev[lv], coeffs<T>(mat, lv), corr[li], Apsi);
                Kern<T>::axpy(s, nc, T(-1), Apsi, src[li], nullptr);
            }
            Ops<T>::restrict_field(s, mesh->dev[lv], src[li], src[li + 1]);
        }
        // solveCoarsestLevel (GAMGSolverSolve.C:520-552): PCG+DIC or
        // PBiCGStab+DILU from zero at the GAMG tolerances, one CTA.
        if (lu) {
            // LUscalarMatrix::solve (LUscalarMatrixTemplates.C:29-139)
            Ops<T>::lu_solve(s, mesh->dev[coarsest + 1].n, lu, piv, src[coarsest], corr[coarsest]);
        } else {
            Kern<T>::fill(s, mesh->dev[coarsest + 1].n, T(0), corr[coarsest], nullptr);
            Kern<T>::block_solve(s, d_blk, 1, nullptr);
        }
        for (int li = coarsest - 1; li >= 0; --li) {
            const int lv = li + 1;
            const int nc = mesh->dev[lv].n;
            T* pre = nullptr;
            if (ctl->nPreSweeps) {
                Kern<T>::copy(s, nc, corr[li], scratch2, nullptr);
                pre = scratch2;
            }
            Ops<T>::prolong_field(s, mesh->dev[lv], corr[li + 1], corr[li]);
            if (interp) Ops<T>::interpolate(s, mesh->dev[lv], coeffs<T>(mat, lv), corr[li], Apsi, corr[li + 1]);
            if (scaleCorr && (interp || li < coarsest - 1)) {
                scale<T>(ctx, mat, lv, corr[li], Apsi, src[li], pre, st);
            } else if (pre) {
                Kern<T>::axpy(s, nc, T(1), pre, corr[li], nullptr);
            }
            smooth<T>(ctx, mat, lv, smoother, corr[li], src[li],
                      std::min(ctl->nPostSweeps + ctl->postSweepsLevelMultiplier * li, ctl->maxPostSweeps),
                      workFor(lv));
        }
        Ops<T>::prolong_field(s, mesh->dev[0], corr[0], fcorr);
        if (interp) Ops<T>::interpolate(s, mesh->dev[0], coeffs<T>(mat, 0), fcorr, Apsi, corr[0]);
        if (scaleCorr) scale<T>(ctx, mat, 0, fcorr, Apsi, fres, nullptr, st);
    }

    Work<T>& workFor(int lv);
};

template <>
Work<double>& GamgCycle<double>::workFor(int lv) {
    return mat->lv64[lv];
}
template <>
Work<float>& GamgCycle<float>::workFor(int lv) {
    return mat->lv32[lv];
}

template <class T>
BlockSys<T>* block_sys(cfx_matrix* mat);
template <>
BlockSys<double>* block_sys<double>(cfx_matrix* mat) {
    if (!mat->d_blk64) mat->d_blk64 = mat->blockArena.get<BlockSys<double>>(1);
    return mat->d_blk64;
}
template <>
BlockSys<float>* block_sys<float>(cfx_matrix* mat) {
    if (!mat->d_blk32) mat->d_blk32 = mat->blockArena.get<BlockSys<float>>(1);
    return mat->d_blk32;
}

constexpr int G0 = 1000;  // GAMG work-vector slots (apart from the Krylov ones)

template <class T>
void setup_cycle(GamgCycle<T>& cy, cfx_matrix* mat, const cfx_controls* ctl, Work<T>& W, SolveState* st) {
    cfx_mesh* mesh = mat->mesh;
    cfx_ctx* ctx = mesh->ctx;
    cudaStream_t s = ctx->stream;
    const int nl = int(mesh->dev.size());
    cy.ctx = ctx;
    cy.mat = mat;
    cy.ctl = ctl;
    cy.coarsest = nl - 2;
    cy.scaleCorr = ctl->scaleCorrection < 0 ? mat->sym : ctl->scaleCorrection != 0;
    cy.interp = ctl->interpolateCorrection != 0;
    cy.st = st;
    int maxSize = 0;
    for (int i = 0; i < nl; ++i) maxSize = std::max(maxSize, mesh->dev[i].n);
    W.n = std::max(W.n, maxSize);
    cy.corr.assign(nl - 1, nullptr);
    cy.src.assign(nl - 1, nullptr);
    for (int li = 0; li < nl - 1; ++li) {
        cy.corr[li] = W.get(G0 + 10 + 2 * li, mesh->dev[li + 1].n);
        cy.src[li] = W.get(G0 + 11 + 2 * li, mesh->dev[li + 1].n);
    }
    cy.Apsi = W.get(G0 + 0, maxSize);
    cy.fcorr = W.get(G0 + 1, maxSize);
    cy.scratch2 = W.get(G0 + 2, maxSize);
    // smoother / coarsest-solver set-up on every level (initVcycle: the
    // smoothers are constructed per solve, so DIC rD is recomputed)
    // sweep counts used on each level (Vcycle, GAMGSolverSolve.C:179-390)
    for (int lv = 0; lv < nl - 1; ++lv) {
        if (ctl->smoother == CFX_SMOOTH_DIC || ctl->smoother == CFX_SMOOTH_DILU || ctl->smoother == CFX_SMOOTH_DICGS ||
            ctl->smoother == CFX_SMOOTH_DILUGS)
            compute_rD<T>(mat, lv);  // DIC pivots when symmetric, DILU otherwise
        if (lv == 0) {
            prepare_smooth<T>(mat, 0, ctl->smoother, ctl->nFinestSweeps, cy.workFor(0));
            continue;
        }
        const int li = lv - 1;
        if (ctl->nPreSweeps)
            prepare_smooth<T>(mat, lv, ctl->smoother,
                              std::min(ctl->nPreSweeps + ctl->preSweepsLevelMultiplier * li, ctl->maxPreSweeps),
                              cy.workFor(lv));
        prepare_smooth<T>(mat, lv, ctl->smoother,
                          std::min(ctl->nPostSweeps + ctl->postSweepsLevelMultiplier * li, ctl->maxPostSweeps),
                          cy.workFor(lv));
    }
    ensure_chunk_partials(ctx, RED_MAXB);
    const int lc = nl - 1;
    const LevelMesh& m = mesh->dev[lc];
    LevelCoeffs<T>& c = coeffs<T>(mat, lc);
    cy.lu = nullptr;
    cy.piv = nullptr;
    if (ctl->directSolveCoarsest) {
        // GAMGSolver.C:257-267: the coarsest matrix factorised once per
        // solver construction (here: per solve), in the cycle's precision
        if (m.n > 8192) throw StatusError(CFX_ERR_CONFIG, "directSolveCoarsest: the coarsest level has more "
                                                          "than 8192 cells");
        if (m.nIf && m.luIfN < 0)
            throw StatusError(CFX_ERR_CONFIG, "directSolveCoarsest: a coarsest-level interface has no partner "
                                              "patch of its size");
        cy.lu = W.get(G0 + 700, m.n * m.n);
        T* vv = W.get(G0 + 701, m.n);
        if (mat->luPivN < m.n) {
            mat->luPiv = mat->arena.get<int>(m.n);
            mat->luPivN = m.n;
        }
        cy.piv = mat->luPiv;
        CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), s));
        Ops<T>::lu_factor(s, m, c, cy.lu, vv, cy.piv, ctx->d_status);
        if (read_status(ctx) == CFX_ERR_FATAL) {
            CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), s));
            throw StatusError(CFX_ERR_FATAL, "Singular matrix");
        }
        return;
    }
    compute_rD<T>(mat, lc, 0);  // coarsest PCG+DIC / PBiCGStab+DILU
    BlockSys<T> h{};
    h.n = m.n;
    h.nf = m.nf;
    h.ownerStart = m.ownerStart;
    h.losortStart = m.losortStart;
    h.losortL = m.losortL;
    h.u = m.u;
    h.fwdCells = m.fwd.cells;
    h.fwdLevelStart = m.fwd.levelStart;
    h.nFwd = m.fwd.nLevels;
    h.bwdCells = m.bwd.cells;
    h.bwdLevelStart = m.bwd.levelStart;
    h.nBwd = m.bwd.nLevels;
    h.diag = c.diag;
    h.lp = c.lowerPerm;
    h.upper = c.upper;
    h.rD = c.rD;
    h.itf = if_bou(m, c);  // the coarsest level's interfaces (solveCoarsestLevel)
    h.b = cy.src[lc - 1];
    h.psi = cy.corr[lc - 1];
    h.r = W.get(G0 + 3, m.n);
    h.w = W.get(G0 + 4, m.n);
    h.p = W.get(G0 + 5, m.n);
    h.q = W.get(G0 + 6, m.n);
    h.s = W.get(G0 + 7, m.n);
    h.t = W.get(G0 + 8, m.n);
    h.r0 = W.get(G0 + 9, m.n);
    h.tolerance = ctl->tolerance;
    h.relTol = ctl->relTol;
    h.maxIter = 1000;  // lduMatrix::solver::defaultMaxIter_ (lduMatrix.C:38)
    h.minIter = 0;
    h.precond = mat->sym ? CFX_PRE_DIC : CFX_PRE_DILU;
    h.solver = mat->sym ? CFX_SOLVER_PCG : CFX_SOLVER_PBICGSTAB;
    cy.d_blk = block_sys<T>(mat);
    CK(cudaMemcpyAsync(cy.d_blk, &h, sizeof(h), cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));  // h is a stack object
}

}  // namespace

namespace cfx {
// GAMGPreconditioner (GAMGPreconditioner.C:40-148): its own GAMG controls
// (the preconditioner dictionary's smoother, sweeps, tolerance and relTol)
// and one V-cycle object per precision.
struct PcGamg {
    cfx_controls ctl{};
    GamgCycle<double> c64{};
    GamgCycle<float> c32{};
};
void pc_gamg_free(PcGamg* p) { delete p; }
}  // namespace cfx

namespace {

template <class T>
GamgCycle<T>& pc_cycle(PcGamg* p);
template <>
GamgCycle<double>& pc_cycle<double>(PcGamg* p) {
    return p->c64;
}
template <>
GamgCycle<float>& pc_cycle<float>(PcGamg* p) {
    return p->c32;
}
template <class T>
Work<T>& work_of(cfx_matrix* mat);
template <>
Work<double>& work_of<double>(cfx_matrix* mat) {
    return mat->w64;
}
template <>
Work<float>& work_of<float>(cfx_matrix* mat) {
    return mat->w32;
}

constexpr int PC_SLOT = 3;  // SolveState of the preconditioner's V-cycles

template <class T>
void pc_gamg_setup(cfx_matrix* mat) {
    PcGamg* P = mat->pcGamg;
    cfx_ctx* ctx = mat->mesh->ctx;
    prepare_levels(mat, sizeof(T) == 4);
    const int nl = int(mat->mesh->dev.size());
    if ((int)mat->lv64.size() < nl) mat->lv64.resize(nl);
    if ((int)mat->lv32.size() < nl) mat->lv32.resize(nl);
    set_state(ctx, PC_SLOT, P->ctl, P->ctl.tolerance, P->ctl.relTol, 1, 0);
    setup_cycle<T>(pc_cycle<T>(P), mat, &P->ctl, work_of<T>(mat), ctx->d_state + PC_SLOT);
    // the finest residual and A wA: allocated here, outside graph capture
    work_of<T>(mat).get(G0 + 600, mat->mesh->dev[0].n);
    work_of<T>(mat).get(G0 + 601, mat->mesh->dev[0].n);
}

// wA = 0; nVcycles V-cycles of A wA = rA, the finest residual rA - A wA
// recomputed between them (GAMGPreconditioner.C:81-148).  The dot product
// w.r (PCG's wArA), when asked, lands in chunkPartials[0] (one partial).
template <class T>
int pc_gamg_apply(cfx_matrix* mat, const T* r, T* w, const int* done, bool dot) {
    PcGamg* P = mat->pcGamg;
    GamgCycle<T>& cy = pc_cycle<T>(P);
    cfx_ctx* ctx = mat->mesh->ctx;
    cudaStream_t s = ctx->stream;
    const LevelMesh& m0 = mat->mesh->dev[0];
    LevelCoeffs<T>& c0 = coeffs<T>(mat, 0);
    const int n = m0.n;
    Work<T>& W = work_of<T>(mat);
    T* fres = W.get(G0 + 600, n);
    T* Aw = W.get(G0 + 601, n);
    Kern<T>::fill(s, n, T(0), w, done);
    Kern<T>::copy(s, n, r, fres, done);
    for (int cyc = 0; cyc < P->ctl.nVcycles; ++cyc) {
        cy.enqueue(w, r, fres);
        Kern<T>::axpy(s, n, T(1), cy.fcorr, w, done);
        smooth<T>(ctx, mat, 0, P->ctl.smoother, w, r, P->ctl.nFinestSweeps, cy.workFor(0));
        if (cyc < P->ctl.nVcycles - 1) {
            // finestResidual = rA; finestResidual -= AwA
            Ops<T>::amul(s, m0, c0, w, Aw);
            Kern<T>::copy(s, n, r, fres, done);
            Kern<T>::axpy(s, n, T(-1), Aw, fres, done);
        }
    }
    if (!dot) return 0;
    launch_reduce<T>(s, ctx->sc, 3, n, w, r, ctx->sc.chunkPartials);
    count_launch();
    return 1;
}

cfx_status gamg_solve(cfx_matrix* mat, const cfx_controls& ctl, double* psi, const double* b, cfx_perf* perf) {
    cfx_mesh* mesh = mat->mesh;
    cfx_ctx* ctx = mesh->ctx;
    cudaStream_t s = ctx->stream;
    if (mesh->nCoarseLevels < 1) {
        set_error("No coarse levels created, either matrix too small for GAMG or nCellsInCoarsestLevel too large");
        return CFX_ERR_STATE;
    }
    const bool mixed = ctl.precision == CFX_MIXED;
    prepare_levels(mat, mixed);
    const int nl = int(mesh->dev.size());
    if ((int)mat->lv64.size() < nl) mat->lv64.resize(nl);
    if ((int)mat->lv32.size() < nl) mat->lv32.resize(nl);
    const LevelMesh& m0 = mesh->dev[0];
    const int n = m0.n;
    SolveState* st = ctx->d_state;
    set_state(ctx, 0, ctl, ctl.tolerance, ctl.relTol, ctl.maxIter, ctl.minIter);
    Work<double>& W = mat->w64;
    W.n = std::max(W.n, n);
    double* Apsi = W.get(200, n);
    double* fres = W.get(201, n);
    launch_reduce<double>(s, ctx->sc, 0, n, psi, nullptr, &st->red0);
    count_launch();
    Ops<double>::amul(s, m0, mat->c64[0], psi, Apsi);
    Kern<double>::norm_init(s, ctx->sc, m0, mat->c64[0], Apsi, b, fres, nullptr, st);
    uint64_t key = hkey({mesh->version, uint64_t(small_sweep_threshold()), uint64_t(cluster_global_cells()), uint64_t(sweep_cluster_size()), uint64_t(sweep_cluster_pre()), uint64_t(sweep_flow()), uint64_t(sweep_flow_ahead()), uint64_t(amul_sell()), uint64_t(sweep_grid_stride()), uint64_t(sweep_grid_poll_ns()), uint64_t(sweep_cta_xl()), uint64_t(colored_gs()), uint64_t(colored_pre()), uint64_t(sweep_level_launch()), uint64_t(sweep_smem_cap()), uint64_t(sweep_wave()), uint64_t(sched_chunk_groups()), uint64_t(nl), uint64_t(ctl.smoother), uint64_t(ctl.nPreSweeps), uint64_t(ctl.nPostSweeps),
                         uint64_t(ctl.nFinestSweeps), uint64_t(ctl.maxPreSweeps), uint64_t(ctl.maxPostSweeps),
                         uint64_t(ctl.preSweepsLevelMultiplier), uint64_t(ctl.postSweepsLevelMultiplier),
                         uint64_t(ctl.scaleCorrection + 7), uint64_t(ctl.interpolateCorrection),
                         uint64_t(ctl.directSolveCoarsest), uint64_t(mixed),
                         reinterpret_cast<uint64_t>(psi),
                         reinterpret_cast<uint64_t>(b)});
    SolveState h = read_state(ctx, 0);
    if (!mixed) {
        GamgCycle<double> cy;
        setup_cycle<double>(cy, mat, &ctl, mat->w64, st);
        auto body = [&]() {
            cy.enqueue(psi, b, fres);
            // psi += finestCorrection; smoothers[0].smooth(nFinestSweeps)
            Kern<double>::axpy(s, n, 1.0, cy.fcorr, psi, nullptr);
            smooth<double>(ctx, mat, 0, ctl.smoother, psi, b, ctl.nFinestSweeps, mat->lv64[0]);
            Kern<double>::gamg_residual_check(s, ctx->sc, m0, mat->c64[0], psi, b, fres, st);
        };
        while (!h.done) {
            graph_launch(mat->gGAMG, key, s, body);
            h = read_state(ctx, 0);
            const int stc = read_status(ctx);
            if (stc != 0) return cfx_status(stc);
            if (ctx->yield && !h.done) ctx->yield(ctx->yieldArg);
        }
    } else {
        // FP32 V-cycle on the residual equation A e = r inside an FP64
        // refinement loop: e = S(0 + C(r)) equals the FP64 cycle's
        // psi_new - psi in exact arithmetic (Gauss-Seidel is affine).
        GamgCycle<float> cy;
        setup_cycle<float>(cy, mat, &ctl, mat->w32, st);
        Work<float>& W32 = mat->w32;
        float* r32 = W32.get(201, n);
        float* e32 = cy.fcorr;
        auto body = [&]() {
            launch_cast_pred(s, n, fres, r32, nullptr);
            cy.enqueue(nullptr, nullptr, r32);
            smooth<float>(ctx, mat, 0, ctl.smoother, e32, r32, ctl.nFinestSweeps, mat->lv32[0]);
            launch_add_f2d(s, n, e32, psi, nullptr);
            Kern<double>::gamg_residual_check(s, ctx->sc, m0, mat->c64[0], psi, b, fres, st);
        };
        while (!h.done) {
            graph_launch(mat->gMixed, key, s, body);
            h = read_state(ctx, 0);
            const int stc = read_status(ctx);
            if (stc != 0) return cfx_status(stc);
            if (ctx->yield && !h.done) ctx->yield(ctx->yieldArg);
        }
    }
    std::snprintf(perf->solverName, sizeof(perf->solverName), "GAMG");
    perf->initialResidual = h.initialResidual;
    perf->finalResidual = h.finalResidual;
    perf->nIterations = h.nIterations;
    perf->converged = h.converged;
    perf->singular = h.singular;
    perf->nOuter = mixed ? h.nIterations : 0;
    return CFX_OK;
}

const char* pre_name(int p) {
    switch (p) {
        case CFX_PRE_NONE: return "none";
        case CFX_PRE_DIAGONAL: return "diagonal";
        case CFX_PRE_DIC: return "DIC";
        case CFX_PRE_GAMG: return "GAMG";
        default: return "DILU";
    }
}

cfx_status krylov_solve(cfx_matrix* mat, const cfx_controls& ctl, double* psi, const double* b, cfx_perf* perf) {
    cfx_ctx* ctx = mat->mesh->ctx;
    cudaStream_t s = ctx->stream;
    const int n = mat->mesh->dev[0].n;
    SolveState h{};
    if (ctl.preconditioner == CFX_PRE_GAMG) {
        if (mat->mesh->nCoarseLevels < 1) {
            set_error("GAMG preconditioner: no coarse levels (agglomerate the mesh first)");
            return CFX_ERR_STATE;
        }
        if (!mat->pcGamg) mat->pcGamg = new PcGamg();
        // coarse coefficients and level work lists before krylov() takes
        // references into them (prepare_levels grows mat->c64 / c32)
        prepare_levels(mat, ctl.precision == CFX_MIXED);
        const int nl = int(mat->mesh->dev.size());
        if ((int)mat->lv64.size() < nl) mat->lv64.resize(nl);
        if ((int)mat->lv32.size() < nl) mat->lv32.resize(nl);
        cfx_controls pc = ctl;
        pc.solver = CFX_SOLVER_GAMG;
        pc.tolerance = ctl.pcTolerance;
        pc.relTol = ctl.pcRelTol;
        pc.maxIter = 1000;
        pc.minIter = 0;
        mat->pcGamg->ctl = pc;
    }
    if (ctl.precision != CFX_MIXED) {
        CFX_TRY(krylov<double>(mat, mat->w64, ctl.solver == CFX_SOLVER_PCG ? mat->gPCG : mat->gBiCG, 0, ctl.solver,
                               ctl.preconditioner, psi, b, 0, ctl.tolerance, ctl.relTol, ctl.maxIter, ctl.minIter,
                               ctl, &h));
        perf->nOuter = 0;
    } else {
        // FP64 iterative refinement around an FP32 Krylov solve of A e = r:
        // the outer residual, solution, normFactor and convergence test are
        // FP64 (the reference's definitions); the inner solve reduces the
        // residual by innerRelTol.
        prepare_levels(mat, true);
        const LevelMesh& m = mat->mesh->dev[0];
        Work<double>& W = mat->w64;
        W.n = std::max(W.n, n);
        double* Apsi = W.get(300, n);
        double* r64 = W.get(301, n);
        float* r32 = mat->w32.get(300, n);
        float* e32 = mat->w32.get(301, n);
        SolveState* st = ctx->d_state;
        set_state(ctx, 0, ctl, ctl.tolerance, ctl.relTol, ctl.maxIter, ctl.minIter);
        launch_reduce<double>(s, ctx->sc, 0, n, psi, nullptr, &st->red0);
        count_launch();
        Ops<double>::amul(s, m, mat->c64[0], psi, Apsi);
        Kern<double>::norm_init(s, ctx->sc, m, mat->c64[0], Apsi, b, r64, nullptr, st);
        h = read_state(ctx, 0);
        int inner = 0, outer = 0;
        const double innerRelTol = 1e-3;
        // An FP32 inner solve that has not reduced its residual by
        // innerRelTol within innerCap iterations has stalled (FP32 rounding
        // on an ill-conditioned system): the solve then finishes in FP64 from
        // the current psi.
        const int innerCap = std::max(100, ctl.maxIter / 10);
        bool stalled = false;
        while (!h.done) {
            launch_cast_d2f(s, n, r64, r32);
            Kern<float>::fill(s, n, 0.0f, e32, nullptr);
            SolveState hi{};
            CFX_TRY(krylov<float>(mat, mat->w32, ctl.solver == CFX_SOLVER_PCG ? mat->gPCG : mat->gBiCG, 0, ctl.solver,
                                  ctl.preconditioner, e32, r32, 1, 0.0, innerRelTol, innerCap, 0, ctl, &hi));
            inner += hi.nIterations;
            launch_add_f2d(s, n, e32, psi, nullptr);
            // outer: r = b - A psi, |r|/normFactor, one refinement step
            Kern<double>::gamg_residual_check(s, ctx->sc, m, mat->c64[0], psi, b, r64, st);
            h = read_state(ctx, 0);
            ++outer;
            if (hi.singular || hi.nIterations == 0) break;
            if (!hi.converged) {
                stalled = true;
                break;
            }
        }
        if (stalled && !h.done) {
            // the FP64 Krylov solve from here; its test keeps the original
            // initial residual: final < max(tolerance, relTol * initial)
            SolveState h64{};
            const double tol = std::max(ctl.tolerance, ctl.relTol * h.initialResidual);
            CFX_TRY(krylov<double>(mat, mat->w64, ctl.solver == CFX_SOLVER_PCG ? mat->gPCG : mat->gBiCG, 0,
                                   ctl.solver, ctl.preconditioner, psi, b, 0, tol, 0.0, ctl.maxIter, 0, ctl, &h64));
            inner += h64.nIterations;
            h.finalResidual = h64.finalResidual;
            h.converged = h64.converged;
            h.singular = h64.singular;
        }
        h.nIterations = inner;
        perf->nOuter = outer;
    }
    const char* base = ctl.solver == CFX_SOLVER_PCG ? "PCG" : ctl.solver == CFX_SOLVER_PBICG ? "PBiCG" : "PBiCGStab";
    std::snprintf(perf->solverName, sizeof(perf->solverName), "%s%s", pre_name(ctl.preconditioner), base);
    perf->initialResidual = h.initialResidual;
    perf->finalResidual = h.finalResidual;
    perf->nIterations = h.nIterations;
    perf->converged = h.converged;
    perf->singular = h.singular;
    if (ctl.solver == CFX_SOLVER_PBICG && h.nIterations > std::max(1000, ctl.maxIter)) {
        set_error("PBiCG has failed to converge within the maximum number of iterations " +
                  std::to_string(std::max(1000, ctl.maxIter)) + "\n    Please try the more robust PBiCGStab solver.");
        return CFX_ERR_FATAL;
    }
    return CFX_OK;
}

// smoothSolver::solve (smoothSolver.C:77-196) in FP64: normFactor and the
// initial residual |source - A psi|, then sweeps of the smoother with the
// residual (lduMatrix::residual) checked every nSweeps; nIterations counts
// sweeps.  The scalar loop test runs on the device (gamg_residual_check with
// an increment of nSweeps); the host reads the state once per check.
cfx_status smooth_solve(cfx_matrix* mat, const cfx_controls& ctl, double* psi, const double* b, cfx_perf* perf) {
    cfx_ctx* ctx = mat->mesh->ctx;
    cudaStream_t s = ctx->stream;
    const LevelMesh& m = mat->mesh->dev[0];
    LevelCoeffs<double>& c = mat->c64[0];
    const int n = m.n;
    if ((int)mat->lv64.size() < 1) mat->lv64.resize(1);
    Work<double>& LW = mat->lv64[0];
    std::snprintf(perf->solverName, sizeof(perf->solverName), "smoothSolver");
    const bool fact = ctl.smoother != CFX_SMOOTH_GS && ctl.smoother != CFX_SMOOTH_SYMGS;
    if (ctl.nSweeps < 0) {
        if (fact) compute_rD<double>(mat, 0);
        prepare_smooth<double>(mat, 0, ctl.smoother, -ctl.nSweeps, LW);
        smooth<double>(ctx, mat, 0, ctl.smoother, psi, b, -ctl.nSweeps, LW);
        CK(cudaStreamSynchronize(s));
        const int stc = read_status(ctx);
        if (stc) return cfx_status(stc);
        perf->nIterations = -ctl.nSweeps;
        return CFX_OK;
    }
    const int slot = 0;
    set_state(ctx, slot, ctl, ctl.tolerance, ctl.relTol, ctl.maxIter, ctl.minIter);
    SolveState* st = ctx->d_state + slot;
    double* Apsi = mat->w64.get(0, n);
    double* r = mat->w64.get(1, n);
    launch_reduce<double>(s, ctx->sc, 0, n, psi, nullptr, &st->red0);
    count_launch();
    Ops<double>::amul(s, m, c, psi, Apsi);
    Kern<double>::norm_init(s, ctx->sc, m, c, Apsi, b, r, nullptr, st);
    SolveState h = read_state(ctx, slot);
    if (!h.done) {
        if (fact) compute_rD<double>(mat, 0);
        const int ns = std::max(ctl.nSweeps, 1);
        prepare_smooth<double>(mat, 0, ctl.smoother, ns, LW);
        int checks = 0;
        while (!h.done) {
            smooth<double>(ctx, mat, 0, ctl.smoother, psi, b, ns, LW);
            Kern<double>::gamg_residual_check(s, ctx->sc, m, c, psi, b, r, st, ns);
            h = read_state(ctx, slot);
            const int stc = read_status(ctx);
            if (stc) return cfx_status(stc);
            if (++checks > ctl.maxIter + ctl.minIter + 16) {
                set_error("smoothing loop did not terminate");
                return CFX_ERR_STATE;
            }
        }
    }
    perf->initialResidual = h.initialResidual;
    perf->finalResidual = h.finalResidual;
    perf->nIterations = h.nIterations;
    perf->converged = h.converged;
    perf->singular = 0;
    return CFX_OK;
}

cfx_status check_controls(const cfx_matrix* mat, const cfx_controls* c) {
    if (!c) {
        set_error("null controls");
        return CFX_ERR_ARG;
    }
    if (c->solver < 0 || c->solver > 4 || c->preconditioner < 0 || c->preconditioner > 5 || c->smoother < 0 ||
        c->smoother > 7 || (c->precision != CFX_FP64 && c->precision != CFX_MIXED)) {
        set_error("unknown solver, preconditioner, smoother or precision");
        return CFX_ERR_CONFIG;
    }
    // lduMatrix::solver::New (lduMatrixSolver.C:67-120): PCG is registered
    // for symmetric matrices only; DIC only for symmetric, DILU for asymmetric.
    if (c->solver == CFX_SOLVER_PCG && !mat->sym) {
        set_error("Unknown asymmetric matrix solver cudaPCG");
        return CFX_ERR_CONFIG;
    }
    if (mat->mesh->nIf) {
        // coupled interfaces: the lduMatrix operations, the Krylov solvers,
        // smoothSolver and GAMG (cyclicGAMGInterface levels); the direct
        // coarsest-level solve's dense matrix does not take them
        if ((c->solver == CFX_SOLVER_GAMG || c->preconditioner == CFX_PRE_GAMG) && c->directSolveCoarsest &&
            mat->mesh->ifNbrPatch.empty()) {
            set_error("directSolveCoarsest with coupled interfaces needs the interfaces' partner patches "
                      "(cfx_mesh_set_interface_partners)");
            return CFX_ERR_CONFIG;
        }
        if ((c->solver == CFX_SOLVER_GAMG || c->preconditioner == CFX_PRE_GAMG) && c->smoother == CFX_SMOOTH_NBGS) {
            set_error("nonBlockingGaussSeidel with coupled interfaces is not supported");
            return CFX_ERR_CONFIG;
        }
        // nonBlockingGaussSeidel splits its sweep at the first interface cell
        // (nonBlockingGaussSeidelSmoother.C:56-78); only GaussSeidel's
        // arithmetic (no interfaces) is built
        if ((c->solver == CFX_SOLVER_SMOOTH) && c->smoother == CFX_SMOOTH_NBGS) {
            set_error("nonBlockingGaussSeidel with coupled interfaces is not supported");
            return CFX_ERR_CONFIG;
        }
        if (mat->ifN != mat->mesh->nIf) {
            set_error("the interface coefficients are not set (cfx_matrix_set_interface_coeffs)");
            return CFX_ERR_STATE;
        }
    }
    if (c->solver == CFX_SOLVER_PBICG && mat->sym) {
        set_error("Unknown symmetric matrix solver cudaPBiCG");  // PBiCG.C:34-35: asymmetric only
        return CFX_ERR_CONFIG;
    }
    if (c->solver == CFX_SOLVER_PBICG && c->preconditioner == CFX_PRE_GAMG) {
        // lduMatrix::preconditioner::preconditionT (lduMatrix.H:500-508)
        set_error("Not implemented: GAMGPreconditioner::preconditionT");
        return CFX_ERR_FATAL;
    }
    if (c->solver == CFX_SOLVER_SMOOTH && c->precision == CFX_MIXED) {
        set_error("precision mixed is not available for cudaSmoothSolver");
        return CFX_ERR_CONFIG;
    }
    const bool pcGamg = (c->solver == CFX_SOLVER_PCG || c->solver == CFX_SOLVER_PBICGSTAB) &&
                        c->preconditioner == CFX_PRE_GAMG;
    if (c->solver == CFX_SOLVER_PBICG && c->precision == CFX_MIXED) {
        set_error("precision mixed is not available for cudaPBiCG");
        return CFX_ERR_CONFIG;
    }
    if (pcGamg && c->nVcycles < 1) {
        set_error("GAMG preconditioner: nVcycles must be at least 1");
        return CFX_ERR_CONFIG;
    }
    if (c->solver == CFX_SOLVER_GAMG || c->solver == CFX_SOLVER_SMOOTH || pcGamg) {
        // smoother tables (the smoothers' *ConstructorToTable registrations)
        const bool symOnly =
            c->smoother == CFX_SMOOTH_DIC || c->smoother == CFX_SMOOTH_DICGS || c->smoother == CFX_SMOOTH_FDIC;
        const bool asymOnly = c->smoother == CFX_SMOOTH_DILU || c->smoother == CFX_SMOOTH_DILUGS;
        static const char* names[] = {"GaussSeidel",     "DIC",  "symGaussSeidel",        "DILU", "DICGaussSeidel",
                                      "DILUGaussSeidel", "FDIC", "nonBlockingGaussSeidel"};
        if ((symOnly && !mat->sym) || (asymOnly && mat->sym)) {
            set_error(std::string("Unknown ") + (mat->sym ? "symmetric" : "asymmetric") + " matrix smoother " +
                      names[c->smoother]);
            return CFX_ERR_CONFIG;
        }
    }
    if (c->solver != CFX_SOLVER_GAMG && c->solver != CFX_SOLVER_SMOOTH) {
        if ((c->preconditioner == CFX_PRE_DIC || c->preconditioner == CFX_PRE_FDIC) && !mat->sym) {
            set_error(std::string("Unknown asymmetric matrix preconditioner ") +
                      (c->preconditioner == CFX_PRE_DIC ? "DIC" : "FDIC"));
            return CFX_ERR_CONFIG;
        }
        if (c->preconditioner == CFX_PRE_DILU && mat->sym) {
            set_error("Unknown symmetric matrix preconditioner DILU");
            return CFX_ERR_CONFIG;
        }
    }
    return CFX_OK;
}

}  // namespace

// ===================================================================== C ABI
namespace cfx {
void ctx_retain(cfx_ctx* ctx) { ctx->refs.fetch_add(1, std::memory_order_relaxed); }

void ctx_release(cfx_ctx* ctx) {
    if (ctx->refs.fetch_sub(1, std::memory_order_acq_rel) != 1) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    cudaFreeHost(ctx->h_state);
    cudaFreeHost(ctx->h_red);
    ctx->arena.release();
    if (ctx->evIn) cudaEventDestroy(ctx->evIn);
    if (ctx->evOut) cudaEventDestroy(ctx->evOut);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
}

void mesh_retain(cfx_mesh* mesh) { mesh->refs.fetch_add(1, std::memory_order_relaxed); }

void mesh_release(cfx_mesh* mesh) {
    if (mesh->refs.fetch_sub(1, std::memory_order_acq_rel) != 1) return;
    cfx_ctx* ctx = mesh->ctx;
    cudaStreamSynchronize(ctx->stream);
    delete mesh;
    ctx_release(ctx);
}
}  // namespace cfx

extern "C" {

void cfx_default_controls(cfx_controls* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->solver = CFX_SOLVER_PCG;
    c->preconditioner = CFX_PRE_DIC;
    c->tolerance = 1e-6;
    c->relTol = 0.0;
    c->maxIter = 1000;
    c->minIter = 0;
    c->smoother = CFX_SMOOTH_GS;
    c->nPreSweeps = 0;
    c->preSweepsLevelMultiplier = 1;
    c->maxPreSweeps = 4;
    c->nPostSweeps = 2;
    c->postSweepsLevelMultiplier = 1;
    c->maxPostSweeps = 4;
    c->nFinestSweeps = 2;
    c->scaleCorrection = -1;
    c->nCellsInCoarsestLevel = 10;
    c->precision = CFX_FP64;
    c->nSweeps = 1;
    c->nVcycles = 2;
    c->pcTolerance = 1e-6;
    c->pcRelTol = 0.0;
}

const char* cfx_last_error(void) { return cfx::last_error(); }
int cfx_version(void) { return 100; }

cfx_status cfx_ctx_create(int device, cfx_ctx** out) {
    if (!out) return CFX_ERR_ARG;
    return guard([&]() -> cfx_status {
        auto ctx = std::make_unique<cfx_ctx>();
        ctx->device = device;
        CK(cudaSetDevice(device));
        CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&ctx->evIn, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&ctx->evOut, cudaEventDisableTiming));
        int sms = 0;
        CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        sweeps_init(sms);
        ctx->sc.partials = ctx->arena.get<double>(RED_MAXB * 4);
        ctx->sc.counters = ctx->arena.get<unsigned>(16);
        ctx->sc.result = ctx->arena.get<double>(16);
        CK(cudaMemset(ctx->sc.counters, 0, 16 * sizeof(unsigned)));
        ctx->d_state = ctx->arena.get<SolveState>(4);
        ctx->d_status = ctx->arena.get<int>(1);
        CK(cudaMemset(ctx->d_status, 0, sizeof(int)));
        ctx->d_red = ctx->arena.get<double>(8);
        CK(cudaMallocHost(&ctx->h_state, 4 * sizeof(SolveState)));
        CK(cudaMallocHost(&ctx->h_red, 8 * sizeof(double)));
        *out = ctx.release();
        return CFX_OK;
    });
}


cfx_status cfx_ctx_destroy(cfx_ctx* ctx) {
    if (!ctx) return CFX_ERR_ARG;
    ctx_release(ctx);
    return CFX_OK;
}

cfx_status cfx_ctx_stream(cfx_ctx* ctx, void** stream) {
    if (!ctx || !stream) return CFX_ERR_ARG;
    *stream = ctx->stream;
    return CFX_OK;
}

cfx_status cfx_ctx_synchronize(cfx_ctx* ctx) {
    if (!ctx) return CFX_ERR_ARG;
    return guard([&]() -> cfx_status {
        CK(cudaStreamSynchronize(ctx->stream));
        return CFX_OK;
    });
}

cfx_status cfx_ctx_launch_count(cfx_ctx* ctx, int64_t* count) {
    if (!ctx || !count) return CFX_ERR_ARG;
    *count = launch_count();
    return CFX_OK;
}

cfx_status cfx_mesh_create(cfx_ctx* ctx, int nCells, int nFaces, const int32_t* l, const int32_t* u,
                           cfx_mesh** out) {
    if (!ctx || !out || nCells < 1) {
        set_error("cfx_mesh_create: bad argument");
        return CFX_ERR_ARG;
    }
    return guard([&]() -> cfx_status {
        auto mesh = std::make_unique<cfx_mesh>();
        mesh->ctx = ctx;
        HostLevel h;
        CFX_TRY(build_host_level(nCells, nFaces, l, u, h, true));
        mesh->host.push_back(std::move(h));
        LevelMesh m;
        upload_level(mesh->arena, ctx->stream, mesh->host[0], m);
        mesh->dev.push_back(m);
        CK(cudaStreamSynchronize(ctx->stream));
        ctx_retain(ctx);
        *out = mesh.release();
        return CFX_OK;
    });
}

cfx_status cfx_mesh_destroy(cfx_mesh* mesh) {
    if (!mesh) return CFX_ERR_ARG;
    mesh_release(mesh);
    return CFX_OK;
}

cfx_status cfx_mesh_info(cfx_mesh* mesh, int* nFwd, int* nBwd) {
    if (!mesh) return CFX_ERR_ARG;
    if (nFwd) *nFwd = mesh->dev[0].fwd.nLevels;
    if (nBwd) *nBwd = mesh->dev[0].bwd.nLevels;
    return CFX_OK;
}

cfx_status cfx_mesh_sell_info(cfx_mesh* mesh, int* slices, int* patternSlices, int64_t* entries) {
    if (!mesh) return CFX_ERR_ARG;
    const LevelMesh& m = mesh->dev[0];
    if (slices) *slices = m.sellCol ? (m.n + 31) / 32 : 0;
    if (patternSlices) *patternSlices = m.sellCol ? m.sellPatternSlices : 0;
    if (entries) *entries = m.sellCol ? m.sellEntries : 0;
    return CFX_OK;
}

cfx_status cfx_face_area_pair_weights(int nFaces, const double* Sf, double* w) {
    if (nFaces < 0 || (nFaces && (!Sf || !w))) return CFX_ERR_ARG;
    face_area_pair_weights(nFaces, Sf, w);
    return CFX_OK;
}

cfx_status cfx_gamg_agglomerate(cfx_mesh* mesh, const double* weights, int nCellsInCoarsestLevel, int forwardStart) {
    if (!mesh || (!weights && mesh->host[0].nf)) return CFX_ERR_ARG;
    return guard([&]() -> cfx_status {
        // pairGAMGAgglomeration::agglomerate (pairGAMGAgglomerate.C:31-118),
        // mergeLevels 1, maxLevels 50, continueAgglomerating (GAMGAgglomeration.C:205-230)
        std::vector<std::vector<int>> maps;
        std::vector<int> nCoarse;
        bool forward = forwardStart != 0;
        std::vector<double> w(weights, weights + mesh->host[0].nf);
        int fn = mesh->host[0].n;
        std::vector<int> fl = mesh->host[0].l, fu = mesh->host[0].u;
        while (int(maps.size()) < MAX_LEVELS - 1) {
            std::vector<int> map;
            const int nc = pair_agglomerate(fn, int(fl.size()), fl.data(), fu.data(), w.data(), forward, map);
            if (!(nc >= nCellsInCoarsestLevel && nc < fn)) break;
            std::vector<int> cl, cu, fra, flip;
            const int ncf = agglomerate_addressing(int(fl.size()), fl.data(), fu.data(), map, nc, cl, cu, fra, flip);
            std::vector<double> cw(ncf, 0.0);
            for (size_t f = 0; f < fra.size(); ++f)
                if (fra[f] >= 0) cw[fra[f]] += w[f];
            maps.push_back(std::move(map));
            nCoarse.push_back(nc);
            w.swap(cw);
            fl.swap(cl);
            fu.swap(cu);
            fn = nc;
        }
        if (maps.empty()) {
            set_error("No coarse levels created, either matrix too small for GAMG or nCellsInCoarsestLevel too large");
            return CFX_ERR_STATE;
        }
        CFX_TRY(build_hierarchy(mesh, maps, nCoarse));
        CK(cudaStreamSynchronize(mesh->ctx->stream));
        return CFX_OK;
    });
}

cfx_status cfx_gamg_set_levels(cfx_mesh* mesh, int nLevels, const int32_t* const* restrictAddr,
                               const int32_t* nCoarseCells) {
    if (!mesh || nLevels < 1 || nLevels >= MAX_LEVELS || !restrictAddr || !nCoarseCells) return CFX_ERR_ARG;
    return guard([&]() -> cfx_status {
        std::vector<std::vector<int>> maps;
        std::vector<int> nCoarse;
        int fn = mesh->host[0].n;
        for (int i = 0; i < nLevels; ++i) {
            maps.emplace_back(restrictAddr[i], restrictAddr[i] + fn);
            nCoarse.push_back(nCoarseCells[i]);
            fn = nCoarseCells[i];
        }
        CFX_TRY(build_hierarchy(mesh, maps, nCoarse));
        CK(cudaStreamSynchronize(mesh->ctx->stream));
        return CFX_OK;
    });
}

cfx_status cfx_gamg_coarse_interfaces(int32_t nFineCells, const int32_t* restrictAddr, int32_t nPatches,
                                      const int32_t* patchSize, const int32_t* faceCells,
                                      const int32_t* nbrCells, int32_t* coarsePatchSize,
                                      int32_t* coarseFaceCells, int32_t* coarseNbrCells,
                                      int32_t* fineToCoarse, int32_t* nCoarseFaces) {
    if (nFineCells < 0 || nPatches < 0 || !nCoarseFaces || (nPatches && (!patchSize || !coarsePatchSize)) ||
        (nFineCells && !restrictAddr))
        return CFX_ERR_ARG;
    int64_t nIf = 0;
    for (int p = 0; p < nPatches; ++p) {
        if (patchSize[p] < 0) return CFX_ERR_ARG;
        nIf += patchSize[p];
    }
    if (nIf > (int64_t(1) << 30)) return CFX_ERR_ARG;
    if (nIf && (!faceCells || !nbrCells || !coarseFaceCells || !coarseNbrCells || !fineToCoarse)) return CFX_ERR_ARG;
    for (int64_t k = 0; k < nIf; ++k)
        if (faceCells[k] < 0 || faceCells[k] >= nFineCells || nbrCells[k] < 0 || nbrCells[k] >= nFineCells) {
            set_error("cfx_gamg_coarse_interfaces: a face cell is out of range");
            return CFX_ERR_ADDRESSING;
        }
    return guard([&]() -> cfx_status {
        std::vector<int> size(patchSize, patchSize + nPatches), cell(faceCells, faceCells + nIf),
            nbr(nbrCells, nbrCells + nIf), cSize, cCell, cNbr, toCoarse;
        coarse_interface_faces(restrictAddr, size, cell, nbr, cSize, cCell, cNbr, toCoarse);
        std::copy(cSize.begin(), cSize.end(), coarsePatchSize);
        std::copy(cCell.begin(), cCell.end(), coarseFaceCells);
        std::copy(cNbr.begin(), cNbr.end(), coarseNbrCells);
        std::copy(toCoarse.begin(), toCoarse.end(), fineToCoarse);
        *nCoarseFaces = int32_t(cCell.size());
        return CFX_OK;
    });
}

cfx_status cfx_gamg_n_levels(cfx_mesh* mesh, int* n) {
    if (!mesh || !n) return CFX_ERR_ARG;
    *n = mesh->nCoarseLevels;
    return CFX_OK;
}

cfx_status cfx_gamg_level_info(cfx_mesh* mesh, int level, int* nCells, int* nFaces, int32_t* restrictAddr,
                               int32_t* faceRestrict, int32_t* faceFlip, int32_t* coarseL, int32_t* coarseU) {
    if (!mesh || level < 0 || level >= mesh->nCoarseLevels) return CFX_ERR_ARG;
    const HostLevel& f = mesh->host[level];
    const HostLevel& c = mesh->host[level + 1];
    if (nCells) *nCells = c.n;
    if (nFaces) *nFaces = c.nf;
    if (restrictAddr) std::copy(f.restrictAddr.begin(), f.restrictAddr.end(), restrictAddr);
    if (faceRestrict) std::copy(f.faceRestrict.begin(), f.faceRestrict.end(), faceRestrict);
    if (faceFlip) std::copy(f.faceFlip.begin(), f.faceFlip.end(), faceFlip);
    if (coarseL) std::copy(c.l.begin(), c.l.end(), coarseL);
    if (coarseU) std::copy(c.u.begin(), c.u.end(), coarseU);
    return CFX_OK;
}

cfx_status cfx_matrix_create(cfx_mesh* mesh, const double* diag, const double* upper, const double* lower,
                             cfx_matrix** out) {
    if (!mesh || !out || !diag || (!upper && lower)) return CFX_ERR_ARG;
    return guard([&]() -> cfx_status {
        auto mat = std::make_unique<cfx_matrix>();
        mat->mesh = mesh;
        mat->sym = lower == nullptr;
        mat->diagonal = upper == nullptr;
        LevelCoeffs<double> c;
        alloc_coeffs(mat->arena, mesh->dev[0], mat->sym, c);
        mat->c64.push_back(c);
        const int n = mesh->dev[0].n;
        mat->d_psi = mat->arena.get<double>(n);
        mat->d_src = mat->arena.get<double>(n);
        set_coefficients(mat.get(), diag, upper, lower, cudaMemcpyHostToDevice);
        CK(cudaStreamSynchronize(mesh->ctx->stream));
        mesh_retain(mesh);
        *out = mat.release();
        return CFX_OK;
    });
}

cfx_status cfx_mesh_set_interfaces(cfx_mesh* mesh, int32_t nPatches, const int32_t* patchSize,
                                   const int32_t* faceCells, const int32_t* nbrCells) {
    if (!mesh || nPatches < 0 || (nPatches && (!patchSize || !faceCells || !nbrCells))) return CFX_ERR_ARG;
    const int n = mesh->host[0].n;
    int64_t nIf = 0;
    for (int p = 0; p < nPatches; ++p) {
        if (patchSize[p] < 0) return CFX_ERR_ARG;
        nIf += patchSize[p];
    }
    if (nIf > (int64_t(1) << 30)) return CFX_ERR_ARG;
    for (int64_t k = 0; k < nIf; ++k)
        if (faceCells[k] < 0 || faceCells[k] >= n || nbrCells[k] < 0 || nbrCells[k] >= n) {
            set_error("cfx_mesh_set_interfaces: a face cell is out of range");
            return CFX_ERR_ADDRESSING;
        }
    return guard([&]() -> cfx_status {
        cudaStream_t s = mesh->ctx->stream;
        CK(cudaStreamSynchronize(s));
        mesh->ifArena.release();
        LevelMesh& m = mesh->dev[0];
        m.nIf = int(nIf);
        m.ifStart = m.ifNbr = m.ifCells = nullptr;
        mesh->ifPos.assign(size_t(nIf), 0);
        mesh->d_ifPos = nullptr;
        mesh->nIf = int(nIf);
        if (nIf) {
            // CSR over cells, each cell's faces in patch-then-face order (a
            // stable counting sort): the order updateMatrixInterfaces adds them
            std::vector<int> start(n + 1, 0);
            std::vector<int> nbr(static_cast<size_t>(nIf), 0);
            for (int64_t k = 0; k < nIf; ++k) start[faceCells[k] + 1]++;
            for (int c = 0; c < n; ++c) start[c + 1] += start[c];
            std::vector<int> fill(start.begin(), start.end() - 1);
            for (int64_t k = 0; k < nIf; ++k) {
                const int j = fill[faceCells[k]]++;
                nbr[j] = nbrCells[k];
                mesh->ifPos[size_t(k)] = j;
            }
            m.ifStart = mesh->ifArena.upload(start, s);
            mesh->d_ifPos = mesh->ifArena.upload(mesh->ifPos, s);
            m.ifNbr = mesh->ifArena.upload(nbr, s);
        }
        mesh->ifPatchSize.assign(patchSize, patchSize + nPatches);
        mesh->ifFaceCell.assign(faceCells, faceCells + nIf);
        mesh->ifNbrCell.assign(nbrCells, nbrCells + nIf);
        mesh->ifNbrPatch.clear();
        build_coarse_interfaces(mesh);
        mesh->version++;  // captured graphs hold the interface pointers
        CK(cudaStreamSynchronize(s));
        return CFX_OK;
    });
}

cfx_status cfx_mesh_set_interface_partners(cfx_mesh* mesh, const int32_t* nbrPatch) {
    if (!mesh || !nbrPatch) return CFX_ERR_ARG;
    const int nP = int(mesh->ifPatchSize.size());
    for (int p = 0; p < nP; ++p)
        if (nbrPatch[p] < 0 || nbrPatch[p] >= nP || mesh->ifPatchSize[nbrPatch[p]] != mesh->ifPatchSize[p]) {
            set_error("cfx_mesh_set_interface_partners: patch " + std::to_string(p) +
                      ": the partner patch is out of range or of another size");
            return CFX_ERR_ARG;
        }
    return guard([&]() -> cfx_status {
        mesh->ifNbrPatch.assign(nbrPatch, nbrPatch + nP);
        build_coarse_interfaces(mesh);
        mesh->version++;
        return CFX_OK;
    });
}

cfx_status cfx_matrix_set_interface_coeffs(cfx_matrix* mat, const double* bouCoeffs, const double* intCoeffs) {
    if (!mat) return CFX_ERR_ARG;
    cfx_mesh* mesh = mat->mesh;
    const int nIf = mesh->nIf;
    if (nIf && !bouCoeffs) return CFX_ERR_ARG;
    return guard([&]() -> cfx_status {
        cudaStream_t s = mesh->ctx->stream;
        LevelCoeffs<double>& c = mat->c64[0];
        if (!nIf) {
            c.ifBou = c.ifInt = nullptr;
            mat->ifN = 0;
            return CFX_OK;
        }
        if (mat->ifN != nIf || !c.ifBou) {
            c.ifBou = mat->arena.get<double>(nIf);
            c.ifInt = mat->arena.get<double>(nIf);
        }
        std::vector<double> b(nIf), ic(nIf);
        for (int k = 0; k < nIf; ++k) {
            b[mesh->ifPos[k]] = bouCoeffs[k];
            ic[mesh->ifPos[k]] = intCoeffs ? intCoeffs[k] : bouCoeffs[k];
        }
        CK(cudaMemcpyAsync(c.ifBou, b.data(), sizeof(double) * nIf, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(c.ifInt, ic.data(), sizeof(double) * nIf, cudaMemcpyHostToDevice, s));
        CK(cudaStreamSynchronize(s));  // b and ic are host temporaries
        mat->ifN = nIf;
        mat->coarse64 = mat->coarse32 = false;  // the GAMG levels' interface sums
        return CFX_OK;
    });
}

cfx_status cfx_matrix_create_empty(cfx_mesh* mesh, int symmetric, cfx_matrix** out) {
    if (!mesh || !out) return CFX_ERR_ARG;
    return guard([&]() -> cfx_status {
        auto mat = std::make_unique<cfx_matrix>();
        mat->mesh = mesh;
        mat->sym = symmetric != 0;
        LevelCoeffs<double> c;
        alloc_coeffs(mat->arena, mesh->dev[0], mat->sym, c);
        mat->c64.push_back(c);
        const LevelMesh& m = mesh->dev[0];
        mat->d_psi = mat->arena.get<double>(m.n);
        mat->d_src = mat->arena.get<double>(m.n);
        cudaStream_t s = mesh->ctx->stream;
        CK(cudaMemsetAsync(c.diag, 0, sizeof(double) * m.n, s));
        if (m.nf) CK(cudaMemsetAsync(c.upper, 0, sizeof(double) * m.nf, s));
        if (m.nf && !mat->sym) CK(cudaMemsetAsync(c.lower, 0, sizeof(double) * m.nf, s));
        coefficients_changed(mat.get());
        CK(cudaStreamSynchronize(s));
        mesh_retain(mesh);
        *out = mat.release();
        return CFX_OK;
    });
}

cfx_status cfx_fv_geometry(cfx_mesh* mesh, const double* magSf, const double* deltaCoeffs, const double* weights,
                           const double* V, int32_t nB, const int32_t* bCell, const double* magSfB,
                           const double* deltaCoeffsB) {
    if (!mesh || !V || nB < 0) return CFX_ERR_ARG;
    const HostLevel& h = mesh->host[0];
    if (h.nf && (!magSf || !deltaCoeffs)) return CFX_ERR_ARG;
    if (nB && (!bCell || !magSfB || !deltaCoeffsB)) return CFX_ERR_ARG;
    for (int b = 0; b < nB; ++b)
        if (bCell[b] < 0 || bCell[b] >= h.n) {
            set_error("cfx_fv_geometry: boundary face cell out of range");
            return CFX_ERR_ADDRESSING;
        }
    return guard([&]() -> cfx_status {
        cudaStream_t s = mesh->ctx->stream;
        CK(cudaStreamSynchronize(s));
        mesh->fvArena.release();
        FvGeom g;
        auto up = [&](const double* p, int n) -> double* {
            if (!p) return nullptr;
            double* d = mesh->fvArena.get<double>(n);
            if (n) CK(cudaMemcpyAsync(d, p, sizeof(double) * n, cudaMemcpyHostToDevice, s));
            return d;
        };
        g.nBoundary = nB;
        g.magSf = up(magSf, h.nf);
        g.deltaCoeffs = up(deltaCoeffs, h.nf);
        g.weights = up(weights, h.nf);
        g.V = up(V, h.n);
        g.magSfB = up(magSfB, nB);
        g.deltaCoeffsB = up(deltaCoeffsB, nB);
        // cell -> boundary faces, ascending (a stable counting sort)
        std::vector<int> start(h.n + 1, 0), face(nB), cell(bCell, bCell + nB);
        for (int b = 0; b < nB; ++b) start[bCell[b] + 1]++;
        for (int c = 0; c < h.n; ++c) start[c + 1] += start[c];
        std::vector<int> fill(start.begin(), start.end() - 1);
        for (int b = 0; b < nB; ++b) face[fill[bCell[b]]++] = b;
        g.bCell = mesh->fvArena.upload(cell, s);
        g.bStart = mesh->fvArena.upload(start, s);
        g.bFace = mesh->fvArena.upload(face, s);
        CK(cudaStreamSynchronize(s));
        mesh->fv = g;
        mesh->hasFv = true;
        return CFX_OK;
    });
}

cfx_status cfx_fvm_assemble(cfx_matrix* mat, const cfx_fvm_terms* t, double* d_source) {
    if (!mat || !t || !d_source) return CFX_ERR_ARG;
    cfx_mesh* mesh = mat->mesh;
    if (!mesh->hasFv) {
        set_error("cfx_fvm_assemble: no face geometry (cfx_fv_geometry)");
        return CFX_ERR_STATE;
    }
    const FvGeom& g = mesh->fv;
    const bool ddt = t->rDeltaT > 0, div = t->phi != nullptr, lap = t->lapSign != 0;
    const int nB = g.nBoundary;
    std::string why;
    if (!ddt && !div && !lap) why = "no term";
    else if (ddt && !t->psi0) why = "ddt without psi0";
    else if (div && nB && !t->phiB) why = "div without boundary fluxes";
    else if (div && t->divScheme != CFX_DIV_UPWIND && t->divScheme != CFX_DIV_LINEAR) why = "unknown div scheme";
    else if (div && t->divScheme == CFX_DIV_LINEAR && !g.weights) why = "linear div without weights";
    else if (lap && t->lapSign != 1 && t->lapSign != -1) why = "lapSign must be +1, -1 or 0";
    else if (lap && t->gamma && nB && !t->gammaB) why = "laplacian gamma without boundary values";
    else if (nB && (!t->bcType || !t->bcValue)) why = "boundary conditions missing";
    else if (div == mat->sym) why = div ? "a div term needs an asymmetric matrix" : "an asymmetric matrix without a div term";
    if (!why.empty()) {
        set_error("cfx_fvm_assemble: " + why);
        return CFX_ERR_ARG;
    }
    return guard([&]() -> cfx_status {
        FvmArgs a{};
        a.rDeltaT = t->rDeltaT;
        a.psi0 = t->psi0;
        a.phi = t->phi;
        a.phiB = t->phiB;
        a.divScheme = t->divScheme;
        a.lapSign = t->lapSign;
        a.gammaUniform = t->gammaUniform;
        a.gamma = t->gamma;
        a.gammaB = t->gammaB;
        a.bcType = t->bcType;
        a.bcValue = t->bcValue;
        a.su = t->su;
        a.hasDdt = ddt;
        a.hasDiv = div;
        LevelCoeffs<double>& c = mat->c64[0];
        cfx_ctx* ctx = mesh->ctx;
        const int nIf = mesh->nIf;
        if (nIf && (mat->ifN != nIf || !c.ifBou)) {
            c.ifBou = mat->arena.get<double>(nIf);
            c.ifInt = mat->arena.get<double>(nIf);
        }
        after_caller(ctx);
        launch_fvm_assemble(ctx->stream, mesh->dev[0], g, a, c.diag, c.upper, mat->sym ? nullptr : c.lower,
                            d_source);
        CK(cudaGetLastError());
        if (nIf) {
            // the cyclic faces' coefficients become the interface coefficients
            CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
            launch_fvm_interfaces(ctx->stream, g, a, nIf, mesh->d_ifPos, c.ifBou, c.ifInt, ctx->d_status);
            CK(cudaGetLastError());
            if (read_status(ctx) != 0) {
                CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
                set_error("cfx_fvm_assemble: the cyclic boundary faces (bcType CFX_BC_CYCLIC) are not the "
                          "interfaces' faces, or a linear div term meets them");
                return CFX_ERR_ARG;
            }
            mat->ifN = nIf;
            mat->coarse64 = mat->coarse32 = false;  // the GAMG levels' interface sums
        }
        to_caller(ctx);
        mat->diagonal = false;
        coefficients_changed(mat);
        return CFX_OK;
    });
}

cfx_status cfx_matrix_update(cfx_matrix* mat, const double* diag, const double* upper, const double* lower) {
    if (!mat || !diag || (mat->sym != (lower == nullptr)) || (mat->diagonal != (upper == nullptr))) {
        set_error("cfx_matrix_update: symmetry of the coefficients changed or null diag");
        return CFX_ERR_ARG;
    }
    return guard([&]() -> cfx_status {
        set_coefficients(mat, diag, upper, lower, cudaMemcpyHostToDevice);
        return CFX_OK;
    });
}

cfx_status cfx_matrix_update_device(cfx_matrix* mat, const double* diag, const double* upper, const double* lower) {
    if (!mat || !diag || (mat->sym != (lower == nullptr)) || (mat->diagonal != (upper == nullptr)))
        return CFX_ERR_ARG;
    return guard([&]() -> cfx_status {
        after_caller(mat->mesh->ctx);
        set_coefficients(mat, diag, upper, lower, cudaMemcpyDeviceToDevice);
        to_caller(mat->mesh->ctx);
        return CFX_OK;
    });
}

cfx_status cfx_matrix_destroy(cfx_matrix* mat) {
    if (!mat) return CFX_ERR_ARG;
    cfx_mesh* mesh = mat->mesh;  // alive: the matrix holds a reference
    cudaStreamSynchronize(mesh->ctx->stream);
    pc_gamg_free(mat->pcGamg);
    delete mat;
    mesh_release(mesh);
    return CFX_OK;
}

cfx_status cfx_matrix_coarse(cfx_matrix* mat, int level, double* diag, double* upper, double* lower) {
    if (!mat || level < 0 || level > mat->mesh->nCoarseLevels) return CFX_ERR_ARG;
    return guard([&]() -> cfx_status {
        if (level > 0) prepare_levels(mat, false);
        const LevelMesh& m = mat->mesh->dev[level];
        cudaStream_t s = mat->mesh->ctx->stream;
        const LevelCoeffs<double>& c = mat->c64[level];
        if (diag) CK(cudaMemcpyAsync(diag, c.diag, sizeof(double) * m.n, cudaMemcpyDeviceToHost, s));
        if (upper && m.nf) CK(cudaMemcpyAsync(upper, c.upper, sizeof(double) * m.nf, cudaMemcpyDeviceToHost, s));
        if (lower && !mat->sym && m.nf)
            CK(cudaMemcpyAsync(lower, c.lower, sizeof(double) * m.nf, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        return CFX_OK;
    });
}

cfx_status cfx_solve_device(cfx_matrix* mat, const cfx_controls* ctl, double* d_psi, const double* d_source,
                            cfx_perf* perf) {
    if (!mat || !d_psi || !d_source || !perf) return CFX_ERR_ARG;
    if (mat->diagonal) {
        // lduMatrix::solver::New picks diagonalSolver for a diagonal matrix
        // before it looks at the solver name (lduMatrixSolver.C:52-66)
        if (!ctl) return CFX_ERR_ARG;
        std::memset(perf, 0, sizeof(*perf));
        const cfx_status st = guard([&]() -> cfx_status {
            after_caller(mat->mesh->ctx);
            Ops<double>::diag_solve(mat->mesh->ctx->stream, mat->mesh->dev[0].n, mat->c64[0].diag, d_source, d_psi);
            to_caller(mat->mesh->ctx);
            return CFX_OK;
        });
        std::snprintf(perf->solverName, sizeof(perf->solverName), "diagonal");
        perf->converged = 1;
        perf->status = st;
        return st;
    }
    CFX_TRY(check_controls(mat, ctl));
    std::memset(perf, 0, sizeof(*perf));
    // FDIC (preconditioner and smoother) forms DIC's products in DIC's order
    // (sqr(upper) = upper*upper; rDuUpper = rD[u]*upper is the left factor
    // DIC multiplies first) and nonBlockingGaussSeidel without coupled
    // interfaces is GaussSeidel: they run those kernels under their names
    cfx_controls c = *ctl;
    if (c.preconditioner == CFX_PRE_FDIC) c.preconditioner = CFX_PRE_DIC;
    if (c.smoother == CFX_SMOOTH_FDIC) c.smoother = CFX_SMOOTH_DIC;
    if (c.smoother == CFX_SMOOTH_NBGS) c.smoother = CFX_SMOOTH_GS;
    const cfx_status st = guard([&]() -> cfx_status {
        after_caller(mat->mesh->ctx);
        CK(cudaMemsetAsync(mat->mesh->ctx->d_status, 0, sizeof(int), mat->mesh->ctx->stream));
        if (c.solver == CFX_SOLVER_GAMG) return gamg_solve(mat, c, d_psi, d_source, perf);
        if (c.solver == CFX_SOLVER_SMOOTH) return smooth_solve(mat, c, d_psi, d_source, perf);
        return krylov_solve(mat, c, d_psi, d_source, perf);
    });
    if (ctl->preconditioner == CFX_PRE_FDIC && (c.solver == CFX_SOLVER_PCG || c.solver == CFX_SOLVER_PBICGSTAB))
        std::snprintf(perf->solverName, sizeof(perf->solverName), "FDIC%s",
                      c.solver == CFX_SOLVER_PCG ? "PCG" : "PBiCGStab");
    perf->status = st;
    return st;
}

cfx_status cfx_solve(cfx_matrix* mat, const cfx_controls* ctl, double* psi, const double* source, cfx_perf* perf) {
    if (!mat || !psi || !source || !perf) return CFX_ERR_ARG;
    const int n = mat->mesh->dev[0].n;
    cudaStream_t s = mat->mesh->ctx->stream;
    cfx_status st = guard([&]() -> cfx_status {
        CK(cudaMemcpyAsync(mat->d_psi, psi, sizeof(double) * n, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(mat->d_src, source, sizeof(double) * n, cudaMemcpyHostToDevice, s));
        return CFX_OK;
    });
    if (st != CFX_OK) return st;
    st = cfx_solve_device(mat, ctl, mat->d_psi, mat->d_src, perf);
    const cfx_status st2 = guard([&]() -> cfx_status {
        CK(cudaMemcpyAsync(psi, mat->d_psi, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        return CFX_OK;
    });
    return st != CFX_OK ? st : st2;
}

cfx_status cfx_tune_set(int key, int value) {
    if (value < 0) return CFX_ERR_ARG;
    switch (key) {
        case CFX_TUNE_SMALL_SWEEP: set_small_sweep_threshold(value); return CFX_OK;
        case CFX_TUNE_CLUSTER_GLOBAL: set_cluster_global_cells(value); return CFX_OK;
        case CFX_TUNE_CLUSTER_SIZE:
            if (value != 0 && value != 8 && value != 16 && value != 4 && value != 2) return CFX_ERR_ARG;
            set_sweep_cluster_size(value);
            return CFX_OK;
        case CFX_TUNE_BATCH_INNER_DIGITS:
            if (value < 1 || value > 7) return CFX_ERR_ARG;
            batch_set_inner_digits(value);
            return CFX_OK;
        case CFX_TUNE_SMEM_BYTES:
            if (size_t(value) > sweep_smem_cap_max()) return CFX_ERR_ARG;
            set_sweep_smem_cap(size_t(value));
            return CFX_OK;
        case CFX_TUNE_GRID_WAVE:
            if (value > 1) return CFX_ERR_ARG;
            set_sweep_wave(value);
            return CFX_OK;
        case CFX_TUNE_CLUSTER_PRE:
            if (value != 0 && value != 2 && value != 4 && value != 8 && value != 16) return CFX_ERR_ARG;
            set_sweep_cluster_pre(value);
            return CFX_OK;
        case CFX_TUNE_FLOW:
            if (value > 2) return CFX_ERR_ARG;
            set_sweep_flow(value);
            return CFX_OK;
        case CFX_TUNE_FLOW_AHEAD:
            if (value < 1 || value > 64) return CFX_ERR_ARG;
            set_sweep_flow_ahead(value);
            return CFX_OK;
        case CFX_TUNE_AMUL_SELL:
            if (value < 0 || value > 2) return CFX_ERR_ARG;
            set_amul_sell(value);
            return CFX_OK;
        case CFX_TUNE_GRID_STRIDE:
            if (value < 1 || value > LVL_STRIDE_MAX) return CFX_ERR_ARG;
            set_sweep_grid_stride(value);
            return CFX_OK;
        case CFX_TUNE_GRID_POLL_NS:
            if (value < 0 || value > 1000) return CFX_ERR_ARG;
            set_sweep_grid_poll_ns(value);
            return CFX_OK;
        case CFX_TUNE_CHUNK_GROUPS:
            if (value < 1 || value > SCHED_CHUNK_GROUPS) return CFX_ERR_ARG;
            set_sched_chunk_groups(value);
            return CFX_OK;
        case CFX_TUNE_CTA_XL:
            if (value < 0 || value > 1) return CFX_ERR_ARG;
            set_sweep_cta_xl(value);
            return CFX_OK;
        case CFX_TUNE_COLORED_GS:
            if (value < 0 || value > 2) return CFX_ERR_ARG;
            set_colored_gs(value);
            return CFX_OK;
        case CFX_TUNE_COLORED_PRE:
            if (value < 0 || value > 3) return CFX_ERR_ARG;
            set_colored_pre(value);
            return CFX_OK;
        case CFX_TUNE_LEVEL_LAUNCH:
            if (value < 0 || value > LVL_LAUNCH_MAX) return CFX_ERR_ARG;
            set_sweep_level_launch(value);
            return CFX_OK;
        default: return CFX_ERR_ARG;
    }
}

cfx_status cfx_tune_get(int key, int* value) {
    if (!value) return CFX_ERR_ARG;
    switch (key) {
        case CFX_TUNE_SMALL_SWEEP: *value = small_sweep_threshold(); return CFX_OK;
        case CFX_TUNE_CLUSTER_GLOBAL: *value = cluster_global_cells(); return CFX_OK;
        case CFX_TUNE_CLUSTER_SIZE: *value = sweep_cluster_size(); return CFX_OK;
        case CFX_TUNE_CLUSTER_PRE: *value = sweep_cluster_pre(); return CFX_OK;
        case CFX_TUNE_BATCH_INNER_DIGITS: *value = batch_inner_digits(); return CFX_OK;
        case CFX_TUNE_SMEM_BYTES: *value = int(sweep_smem_cap()); return CFX_OK;
        case CFX_TUNE_GRID_WAVE: *value = sweep_wave(); return CFX_OK;
        case CFX_TUNE_FLOW: *value = sweep_flow(); return CFX_OK;
        case CFX_TUNE_FLOW_AHEAD: *value = sweep_flow_ahead(); return CFX_OK;
        case CFX_TUNE_AMUL_SELL: *value = amul_sell(); return CFX_OK;
        case CFX_TUNE_GRID_STRIDE: *value = sweep_grid_stride(); return CFX_OK;
        case CFX_TUNE_GRID_POLL_NS: *value = sweep_grid_poll_ns(); return CFX_OK;
        case CFX_TUNE_CHUNK_GROUPS: *value = sched_chunk_groups(); return CFX_OK;
        case CFX_TUNE_CTA_XL: *value = sweep_cta_xl(); return CFX_OK;
        case CFX_TUNE_COLORED_GS: *value = colored_gs(); return CFX_OK;
        case CFX_TUNE_COLORED_PRE: *value = colored_pre(); return CFX_OK;
        case CFX_TUNE_LEVEL_LAUNCH: *value = sweep_level_launch(); return CFX_OK;
        default: return CFX_ERR_ARG;
    }
}

// ---------------------------------------------------------- single operations
cfx_status cfx_amul(cfx_matrix* mat, const double* x, double* y) {
    if (!mat || !x || !y) return CFX_ERR_ARG;
    return guard([&]() -> cfx_status {
        after_caller(mat->mesh->ctx);
        Ops<double>::amul(mat->mesh->ctx->stream, mat->mesh->dev[0], mat->c64[0], x, y);
        CK(cudaStreamSynchronize(mat->mesh->ctx->stream));
        return CFX_OK;
    });
}

cfx_status cfx_tmul(cfx_matrix* mat, const double* x, double* y) {
    if (!mat || !x || !y) return CFX_ERR_ARG;
    return guard([&]() -> cfx_status {
        after_caller(mat->mesh->ctx);
        Ops<double>::tmul(mat->mesh->ctx->stream, mat->mesh->dev[0], mat->c64[0], x, y);
        CK(cudaStreamSynchronize(mat->mesh->ctx->stream));
        return CFX_OK;
    });
}

cfx_status cfx_residual(cfx_matrix* mat, const double* x, const double* b, double* r) {
    if (!mat || !x || !b || !r) return CFX_ERR_ARG;
    return guard([&]() -> cfx_status {
        after_caller(mat->mesh->ctx);
        Ops<double>::residual(mat->mesh->ctx->stream, mat->mesh->dev[0], mat->c64[0], x, b, r);
        CK(cudaStreamSynchronize(mat->mesh->ctx->stream));
        return CFX_OK;
    });
}

cfx_status cfx_sumA(cfx_matrix* mat, double* s) {
    if (!mat || !s) return CFX_ERR_ARG;
    return guard([&]() -> cfx_status {
        after_caller(mat->mesh->ctx);
        Ops<double>::sumA(mat->mesh->ctx->stream, mat->mesh->dev[0], mat->c64[0], s);
        CK(cudaStreamSynchronize(mat->mesh->ctx->stream));
        return CFX_OK;
    });
}

cfx_status cfx_reduce(cfx_ctx* ctx, int which, int n, const double* a, const double* b, double* out) {
    if (!ctx || !a || !out || which < 0 || which > 3 || (which == 3 && !b) || n < 0) return CFX_ERR_ARG;
    return guard([&]() -> cfx_status {
        after_caller(ctx);
        launch_reduce<double>(ctx->stream, ctx->sc, which, n, a, b, ctx->d_red);
        count_launch();
        CK(cudaMemcpyAsync(ctx->h_red, ctx->d_red, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        *out = ctx->h_red[0];
        return CFX_OK;
    });
}

cfx_status cfx_norm_factor(cfx_matrix* mat, const double* psi, const double* b, double* out) {
    if (!mat || !psi || !b || !out) return CFX_ERR_ARG;
    return guard([&]() -> cfx_status {
        cfx_ctx* ctx = mat->mesh->ctx;
        after_caller(ctx);
        cudaStream_t s = ctx->stream;
        const LevelMesh& m = mat->mesh->dev[0];
        Work<double>& W = mat->w64;
        W.n = std::max(W.n, m.n);
        double* Apsi = W.get(400, m.n);
        double* r = W.get(401, m.n);
        cfx_controls c;
        cfx_default_controls(&c);
        set_state(ctx, 2, c, 0.0, 0.0, 1, 0);
        SolveState* st = ctx->d_state + 2;
        launch_reduce<double>(s, ctx->sc, 0, m.n, psi, nullptr, &st->red0);
        count_launch();
        Ops<double>::amul(s, m, mat->c64[0], psi, Apsi);
        Kern<double>::norm_init(s, ctx->sc, m, mat->c64[0], Apsi, b, r, nullptr, st);
        *out = read_state(ctx, 2).normFactor;
        return CFX_OK;
    });
}

cfx_status cfx_reciprocal_d(cfx_matrix* mat, int kind, double* rD) {
    if (!mat || !rD) return CFX_ERR_ARG;
    if ((kind == CFX_PRE_DIC && !mat->sym) || (kind == CFX_PRE_DILU && mat->sym) ||
        (kind != CFX_PRE_DIC && kind != CFX_PRE_DILU && kind != CFX_PRE_DIAGONAL))
        return CFX_ERR_CONFIG;
    return guard([&]() -> cfx_status {
        cfx_ctx* ctx = mat->mesh->ctx;
        after_caller(ctx);
        const LevelMesh& m = mat->mesh->dev[0];
        CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
        setup_preconditioner<double>(mat, 0, kind);
        CK(cudaMemcpyAsync(rD, mat->c64[0].rD, sizeof(double) * m.n, cudaMemcpyDeviceToDevice, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        const int stc = read_status(ctx);
        return stc ? cfx_status(stc) : CFX_OK;
    });
}

cfx_status cfx_precondition(cfx_matrix* mat, int kind, int transpose, const double* r, double* w) {
    if (!mat || !r || !w) return CFX_ERR_ARG;
    if (transpose) {
        set_error("preconditionT is used by PBiCG only, which this library does not provide");
        return CFX_ERR_CONFIG;
    }
    if ((kind == CFX_PRE_DIC && !mat->sym) || (kind == CFX_PRE_DILU && mat->sym) || kind < 0 || kind > 3)
        return CFX_ERR_CONFIG;
    return guard([&]() -> cfx_status {
        cfx_ctx* ctx = mat->mesh->ctx;
        after_caller(ctx);
        CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
        setup_preconditioner<double>(mat, 0, kind);
        precondition<double>(mat, 0, kind, r, w, nullptr, false);
        CK(cudaStreamSynchronize(ctx->stream));
        const int stc = read_status(ctx);
        return stc ? cfx_status(stc) : CFX_OK;
    });
}

cfx_status cfx_diag_sweep_stall(cfx_matrix* mat, int timeoutMs, int* status) {
    if (!mat || !status || timeoutMs < 1 || timeoutMs > 10000) return CFX_ERR_ARG;
    return guard([&]() -> cfx_status {
        cfx_ctx* ctx = mat->mesh->ctx;
        cudaStream_t s = ctx->stream;
        const int n = mat->mesh->dev[0].n;
        prepare_gs<double>(mat, 0, 1);
        const DevSched& g = sched(mat->mesh, 0, SCHED_GS, 1);
        Packed<double>& p = packed<double>(mat, 0, OP_GS, 1, g);
        double* b = mat->w64.get(990, n);
        double* x = mat->w64.get(991, n);
        CK(cudaMemsetAsync(b, 0, sizeof(double) * n, s));
        CK(cudaMemsetAsync(x, 0, sizeof(double) * n, s));
        CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), s));
        const cfx_status st = run_sweep_stalled<double>(s, g, p, b, x, 1000000ull * unsigned(timeoutMs),
                                                        ctx->d_status);
        if (st != CFX_OK) return st;
        CK(cudaStreamSynchronize(s));
        *status = read_status(ctx);
        // the context stays usable: clear the status for the next solve
        CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), s));
        CK(cudaStreamSynchronize(s));
        return CFX_OK;
    });
}

cfx_status cfx_diag_smooth_f32(cfx_matrix* mat, int kind, float* psi, const float* b, int nSweeps, int* form) {
    if (!mat || !psi || !b || nSweeps < 0) return CFX_ERR_ARG;
    if (kind != CFX_SMOOTH_GS && kind != CFX_SMOOTH_DIC && kind != CFX_SMOOTH_DILU && kind != CFX_SMOOTH_DICGS &&
        kind != CFX_SMOOTH_DILUGS)
        return CFX_ERR_CONFIG;
    if ((kind == CFX_SMOOTH_DIC || kind == CFX_SMOOTH_DICGS) && !mat->sym) return CFX_ERR_CONFIG;
    if ((kind == CFX_SMOOTH_DILU || kind == CFX_SMOOTH_DILUGS) && mat->sym) return CFX_ERR_CONFIG;
    return guard([&]() -> cfx_status {
        cfx_ctx* ctx = mat->mesh->ctx;
        after_caller(ctx);
        CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
        prepare_levels(mat, true);
        if ((int)mat->lv32.size() < 1) mat->lv32.resize(1);
        if (kind == CFX_SMOOTH_DIC || kind == CFX_SMOOTH_DICGS) setup_preconditioner<float>(mat, 0, CFX_PRE_DIC);
        if (kind == CFX_SMOOTH_DILU || kind == CFX_SMOOTH_DILUGS) setup_preconditioner<float>(mat, 0, CFX_PRE_DILU);
        prepare_smooth<float>(mat, 0, kind, nSweeps, mat->lv32[0]);
        // captured and replayed as a CUDA graph, as inside the V-cycle
        const uint64_t key =
            hkey({mat->mesh->version, uint64_t(kind), uint64_t(nSweeps), uint64_t(reinterpret_cast<uintptr_t>(psi)),
                  uint64_t(reinterpret_cast<uintptr_t>(b)), uint64_t(small_sweep_threshold()),
                  uint64_t(cluster_global_cells()), uint64_t(sweep_cluster_size()), uint64_t(sweep_cluster_pre()),
                  uint64_t(sweep_flow()), uint64_t(sweep_flow_ahead()), uint64_t(amul_sell()),
                  uint64_t(sweep_grid_stride()), uint64_t(sweep_grid_poll_ns()), uint64_t(sweep_cta_xl()),
                  uint64_t(colored_gs()), uint64_t(colored_pre()), uint64_t(sweep_level_launch()), uint64_t(sweep_smem_cap()), uint64_t(sweep_wave()), uint64_t(sched_chunk_groups())});
        graph_launch(mat->gDiag32, key, ctx->stream,
                     [&] { smooth<float>(ctx, mat, 0, kind, psi, b, nSweeps, mat->lv32[0]); });
        if (form) {
            const int S = std::max(nSweeps, 1);
            if (kind == CFX_SMOOTH_DIC || kind == CFX_SMOOTH_DILU)  // no Gauss-Seidel: the forward schedule's
                *form = sweep_mode<float>(sched_pre<float>(mat->mesh, 0, SCHED_FWD, pre_colored<float>(mat->sym)));
            else
                *form = sweep_mode<float>(gs_colored<float>() ? sched_colored(mat->mesh, 0, S)
                                                              : sched(mat->mesh, 0, SCHED_GS, S));
        }
        CK(cudaStreamSynchronize(ctx->stream));
        const int stc = read_status(ctx);
        return stc ? cfx_status(stc) : CFX_OK;
    });
}

cfx_status cfx_smooth(cfx_matrix* mat, int kind, double* psi, const double* b, int nSweeps) {
    if (!mat || !psi || !b || nSweeps < 0) return CFX_ERR_ARG;
    if (kind < CFX_SMOOTH_GS || kind > CFX_SMOOTH_NBGS) return CFX_ERR_CONFIG;
    if (kind == CFX_SMOOTH_FDIC && !mat->sym) return CFX_ERR_CONFIG;
    if (kind == CFX_SMOOTH_NBGS && mat->mesh->nIf) return CFX_ERR_CONFIG;  // its interface split is not built
    if (kind == CFX_SMOOTH_FDIC) kind = CFX_SMOOTH_DIC;  // the same arithmetic (FDICSmoother.C:40-160)
    if (kind == CFX_SMOOTH_NBGS) kind = CFX_SMOOTH_GS;   // no coupled interfaces
    if ((kind == CFX_SMOOTH_DIC || kind == CFX_SMOOTH_DICGS) && !mat->sym) return CFX_ERR_CONFIG;
    if ((kind == CFX_SMOOTH_DILU || kind == CFX_SMOOTH_DILUGS) && mat->sym) return CFX_ERR_CONFIG;
    return guard([&]() -> cfx_status {
        cfx_ctx* ctx = mat->mesh->ctx;
        after_caller(ctx);
        CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
        if ((int)mat->lv64.size() < 1) mat->lv64.resize(1);
        if (kind == CFX_SMOOTH_DIC || kind == CFX_SMOOTH_DICGS) setup_preconditioner<double>(mat, 0, CFX_PRE_DIC);
        if (kind == CFX_SMOOTH_DILU || kind == CFX_SMOOTH_DILUGS) setup_preconditioner<double>(mat, 0, CFX_PRE_DILU);
        prepare_smooth<double>(mat, 0, kind, nSweeps, mat->lv64[0]);
        smooth<double>(ctx, mat, 0, kind, psi, b, nSweeps, mat->lv64[0]);
        CK(cudaStreamSynchronize(ctx->stream));
        const int stc = read_status(ctx);
        return stc ? cfx_status(stc) : CFX_OK;
    });
}

}  // extern "C"
