// host.cpp - host-side addressing: validation, derived LDU addressing, level
// schedules, pairwise agglomeration and coarse-level addressing.
//
// The agglomeration is sequential by nature (each pairing decision depends on
// the previous ones) and runs once per mesh, as in the reference where the
// GAMGAgglomeration is cached in the mesh registry; everything per solve runs
// on the device.

#include <algorithm>
#include <cmath>
#include <limits>
#include <map>

#include "internal.h"

namespace cfx {

// Derived addressing of lduAddressing (lduAddressing.C:32-170) plus the
// lower-neighbour of each losort slot.  With validate, (l, u) must satisfy
// 0 <= l < u < n and l non-decreasing (the owner-sorted order that
// lduAddressing::calcOwnerStart and every face-order loop rely on).
cfx_status build_host_level(int n, int nf, const int* l, const int* u, HostLevel& h, bool validate) {
    if (n < 0 || nf < 0) {
        set_error("negative size");
        return CFX_ERR_ARG;
    }
    if (nf > 0 && (!l || !u)) {
        set_error("null addressing");
        return CFX_ERR_ARG;
    }
    if (validate) {
        for (int f = 0; f < nf; ++f) {
            if (l[f] < 0 || u[f] >= n || l[f] >= u[f]) {
                set_error("face " + std::to_string(f) + ": need 0 <= l < u < nCells (l=" +
                          std::to_string(l[f]) + " u=" + std::to_string(u[f]) + ")");
                return CFX_ERR_ADDRESSING;
            }
            if (f > 0 && l[f - 1] > l[f]) {
                set_error("lower not in incremental cell order at face " + std::to_string(f));
                return CFX_ERR_ADDRESSING;
            }
        }
    }
    h.n = n;
    h.nf = nf;
    h.l.assign(l, l + nf);
    h.u.assign(u, u + nf);
    h.ownerStart.assign(n + 1, 0);
    h.losortStart.assign(n + 1, 0);
    for (int f = 0; f < nf; ++f) {
        h.ownerStart[l[f] + 1]++;
        h.losortStart[u[f] + 1]++;
    }
    for (int c = 0; c < n; ++c) {
        h.ownerStart[c + 1] += h.ownerStart[c];
        h.losortStart[c + 1] += h.losortStart[c];
    }
    h.losort.resize(nf);
    h.losortL.resize(nf);
    std::vector<int> fill(h.losortStart.begin(), h.losortStart.end() - 1);
    for (int f = 0; f < nf; ++f) {
        const int k = fill[u[f]]++;
        h.losort[k] = f;
        h.losortL[k] = l[f];
    }
    build_schedules(h);
    return CFX_OK;
}

// Level schedules.  Forward: level(u) = 1 + max level(l) over the faces
// (l, u); a face's owner is final when the face is reached because faces are
// owner-sorted and l < u.  Backward: level(l) = 1 + max level(u), faces in
// reverse.  Cells are grouped by level, ascending index within a level.
static void group_by_level(const std::vector<int>& lev, int n, std::vector<int>& cells,
                           std::vector<int>& start) {
    int nl = 0;
    for (int c = 0; c < n; ++c) nl = std::max(nl, lev[c] + 1);
    start.assign(nl + 1, 0);
    for (int c = 0; c < n; ++c) start[lev[c] + 1]++;
    for (int i = 0; i < nl; ++i) start[i + 1] += start[i];
    cells.resize(n);
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (int c = 0; c < n; ++c) cells[fill[lev[c]]++] = c;
}

void build_schedules(HostLevel& h) {
    const int n = h.n, nf = h.nf;
    std::vector<int> lev(n, 0);
    for (int f = 0; f < nf; ++f) lev[h.u[f]] = std::max(lev[h.u[f]], lev[h.l[f]] + 1);
    group_by_level(lev, n, h.fwdCells, h.fwdLevelStart);
    std::fill(lev.begin(), lev.end(), 0);
    for (int f = nf - 1; f >= 0; --f) lev[h.l[f]] = std::max(lev[h.l[f]], lev[h.u[f]] + 1);
    group_by_level(lev, n, h.bwdCells, h.bwdLevelStart);
}

// pairGAMGAgglomeration::agglomerate, one level (pairGAMGAgglomerate.C:123-301).
// Cell faces list, per cell, the faces where it is the neighbour (upperAddr)
// then those where it is the owner, each in face order; ties in weight keep
// the first face (strict >).  forward is toggled on return.
int pair_agglomerate(int nFine, int nFaces, const int* l, const int* u, const double* w,
                     bool& forward, std::vector<int>& map) {
    const double great = 1.0 / std::numeric_limits<double>::epsilon();
    std::vector<int> off(nFine + 1, 0), cnt(nFine, 0), cellFaces(2 * size_t(nFaces));
    for (int f = 0; f < nFaces; ++f) {
        off[u[f] + 1]++;
        off[l[f] + 1]++;
    }
    for (int c = 0; c < nFine; ++c) off[c + 1] += off[c];
    for (int f = 0; f < nFaces; ++f) cellFaces[off[u[f]] + cnt[u[f]]++] = f;
    for (int f = 0; f < nFaces; ++f) cellFaces[off[l[f]] + cnt[l[f]]++] = f;
    map.assign(nFine, -1);
    int nCoarse = 0;
    const bool fwd = forward;
    for (int cf = 0; cf < nFine; ++cf) {
        const int c = fwd ? cf : nFine - cf - 1;
        if (map[c] >= 0) continue;
        int match = -1;
        double maxW = -great;
        for (int k = off[c]; k < off[c + 1]; ++k) {
            const int f = cellFaces[k];
            if (map[u[f]] < 0 && map[l[f]] < 0 && w[f] > maxW) {
                match = f;
                maxW = w[f];
            }
        }
        if (match >= 0) {
            map[u[match]] = nCoarse;
            map[l[match]] = nCoarse;
            nCoarse++;
        } else {
            int cmatch = -1;
            double cmax = -great;
            for (int k = off[c]; k < off[c + 1]; ++k) {
                const int f = cellFaces[k];
                if (w[f] > cmax) {
                    cmatch = f;
                    cmax = w[f];
                }
            }
            if (cmatch >= 0) map[c] = std::max(map[u[cmatch]], map[l[cmatch]]);
        }
    }
    for (int cf = 0; cf < nFine; ++cf) {
        const int c = fwd ? cf : nFine - cf - 1;
        if (map[c] < 0) map[c] = nCoarse++;
    }
    if (!fwd) {
        nCoarse--;
        for (int c = 0; c < nFine; ++c) map[c] = nCoarse - map[c];
        nCoarse++;
    }
    forward = !fwd;
    return nCoarse;
}

// GAMGAgglomeration::agglomerateLduAddressing (GAMGAgglomerateLduAddressing.C:32-222):
// coarse faces are created in fine-face order, then numbered by coarse owner
// (creation order within an owner); faceFlip marks fine faces whose coarse
// owner comes from the fine upper cell.
int agglomerate_addressing(int nFaces, const int* l, const int* u, const std::vector<int>& rm,
                           int nCoarse, std::vector<int>& cl, std::vector<int>& cu,
                           std::vector<int>& fra, std::vector<int>& flip) {
    std::vector<std::vector<int>> cCellFaces(nCoarse);
    std::vector<int> initNeighb;
    initNeighb.reserve(nFaces / 2 + 1);
    fra.assign(nFaces, 0);
    for (int f = 0; f < nFaces; ++f) {
        const int rU = rm[u[f]], rL = rm[l[f]];
        if (rU == rL) {
            fra[f] = -(rU + 1);
            continue;
        }
        const int cOwn = std::min(rU, rL), cNei = std::max(rU, rL);
        bool found = false;
        for (int cf : cCellFaces[cOwn]) {
            if (initNeighb[cf] == cNei) {
                fra[f] = cf;
                found = true;
                break;
            }
        }
        if (!found) {
            const int cf = int(initNeighb.size());
            cCellFaces[cOwn].push_back(cf);
            initNeighb.push_back(cNei);
            fra[f] = cf;
        }
    }
    const int ncf = int(initNeighb.size());
    cl.resize(ncf);
    cu.resize(ncf);
    std::vector<int> coarseFaceMap(ncf);
    int k = 0;
    for (int c = 0; c < nCoarse; ++c)
        for (int cf : cCellFaces[c]) {
            cl[k] = c;
            cu[k] = initNeighb[cf];
            coarseFaceMap[cf] = k++;
        }
    flip.assign(nFaces, 0);
    for (int f = 0; f < nFaces; ++f) {
        if (fra[f] >= 0) {
            fra[f] = coarseFaceMap[fra[f]];
            if (cl[fra[f]] == rm[u[f]] && cu[fra[f]] == rm[l[f]]) flip[f] = 1;
        }
    }
    return ncf;
}

// faceAreaPairGAMGAgglomeration.C:55-80 with magSf = max(|Sf|, rootVSmall)
// (primitiveMeshFaceCentresAndAreas.C:93).  Compiled without FMA contraction.
void face_area_pair_weights(int nFaces, const double* Sf, double* w) {
    const double rootVSmall = std::sqrt(std::numeric_limits<double>::min());
    for (int f = 0; f < nFaces; ++f) {
        const double x = Sf[3 * f], y = Sf[3 * f + 1], z = Sf[3 * f + 2];
        const double m = std::max(std::sqrt(x * x + y * y + z * z), rootVSmall);
        const double s = std::sqrt(m);
        const double a = (x / s) * 1.0, b = (y / s) * 1.01, c = (z / s) * 1.02;
        w[f] = std::sqrt(a * a + b * b + c * c);
    }
}

}  // namespace cfx

namespace cfx {

// Packed sweep schedules.  A slot is one cell update (for a combined
// Gauss-Seidel schedule: one cell in one sweep); slots are grouped by DAG
// level, levels padded to whole groups of 32 slots, entries of a group stored
// column-major (entry k of lane j at groupEntry[g] + 32*k + j) so a warp loads
// them coalesced.  src encodes where each entry's coefficient comes from:
// a losort slot k (lower side) or, with SRC_UPPER set, an owner face f.
namespace {

// DAG level of every (sweep, cell) slot, sweep-major.
void sched_levels(const HostLevel& h, int kind, int S, std::vector<int>& lev) {
    const int n = h.n;
    lev.assign(size_t(n) * S, 0);
    if (kind == SCHED_BWD || kind == SCHED_GSB) {
        for (int f = h.nf - 1; f >= 0; --f) lev[h.l[f]] = std::max(lev[h.l[f]], lev[h.u[f]] + 1);
    } else {
        for (int s = 0; s < S; ++s) {
            int* L = lev.data() + size_t(s) * n;
            const int* P = s > 0 ? lev.data() + size_t(s - 1) * n : nullptr;
            if (P) {
                for (int c = 0; c < n; ++c) L[c] = P[c] + 1;
                // c^(s) after the previous sweep of its upper neighbours
                for (int f = 0; f < h.nf; ++f) L[h.l[f]] = std::max(L[h.l[f]], P[h.u[f]] + 1);
            }
            for (int f = 0; f < h.nf; ++f) L[h.u[f]] = std::max(L[h.u[f]], L[h.l[f]] + 1);
        }
    }
}

// The entries of cell c in the reference's per-cell order: neighbour cell
// and coefficient source (a losort slot, or an owner face | SRC_UPPER).
void sched_entries(const HostLevel& h, int kind, int c, std::vector<int>& nbs, std::vector<int>& srcs) {
    nbs.clear();
    srcs.clear();
    if (kind == SCHED_FWD || kind == SCHED_GS || kind == SCHED_GSB) {
        for (int k = h.losortStart[c]; k < h.losortStart[c + 1]; ++k) {
            nbs.push_back(h.losortL[k]);
            srcs.push_back(k);
        }
    }
    if (kind == SCHED_GS || kind == SCHED_GSB) {
        for (int f = h.ownerStart[c]; f < h.ownerStart[c + 1]; ++f) {
            nbs.push_back(h.u[f]);
            srcs.push_back(f | SRC_UPPER);
        }
    }
    if (kind == SCHED_BWD) {
        for (int f = h.ownerStart[c + 1] - 1; f >= h.ownerStart[c]; --f) {
            nbs.push_back(h.u[f]);
            srcs.push_back(f | SRC_UPPER);
        }
    }
}

}  // namespace

namespace {
// 2 groups (64 slots) per chunk: a DAG level's arithmetic spread over about
// four times as many SMs as with full 8-group chunks; measured at 256^3
// (GAMG, GaussSeidel): FP64 solve 3.22 -> 2.76 s, mixed 1.91 -> 1.76 s
int g_chunk_groups = 2;
}
int sched_chunk_groups() { return g_chunk_groups; }
void set_sched_chunk_groups(int g) { g_chunk_groups = g < 1 ? 1 : g > SCHED_CHUNK_GROUPS ? SCHED_CHUNK_GROUPS : g; }

namespace {
int g_colored_gs = 1;
int g_colored_pre = 1;

// Colour of each neighbour entry relative to the cell: the multicolour
// schedule's levels.  Cells are taken colour by colour (ascending cells in a
// colour); (c, s) waits for its smaller-coloured neighbours in sweep s, its
// larger-coloured ones in sweep s-1, and itself in sweep s-1.
// The triangular sweeps (kind SCHED_FWD / SCHED_BWD) wait for every
// neighbour of a smaller (forward) or larger (backward) colour.
void colored_levels(const HostLevel& h, int kind, const std::vector<int>& color, int S, std::vector<int>& lev) {
    const int n = h.n;
    int nc = 0;
    for (int c = 0; c < n; ++c) nc = std::max(nc, color[c] + 1);
    std::vector<int> byColor(n), cstart(nc + 1, 0);
    for (int c = 0; c < n; ++c) cstart[color[c] + 1]++;
    for (int k = 0; k < nc; ++k) cstart[k + 1] += cstart[k];
    {
        std::vector<int> fill(cstart.begin(), cstart.end() - 1);
        for (int c = 0; c < n; ++c) byColor[fill[color[c]]++] = c;
    }
    lev.assign(size_t(n) * S, 0);
    std::vector<int> nbs, srcs;
    if (kind == SCHED_FWD || kind == SCHED_BWD) {
        const bool fwd = kind == SCHED_FWD;
        for (int i = 0; i < n; ++i) {
            const int c = byColor[fwd ? i : n - 1 - i];
            int v = 0;
            sched_entries(h, SCHED_GS, c, nbs, srcs);
            for (int nb : nbs)
                if (fwd ? color[nb] < color[c] : color[nb] > color[c]) v = std::max(v, lev[nb] + 1);
            lev[c] = v;
        }
        return;
    }
    for (int s = 0; s < S; ++s) {
        int* L = lev.data() + size_t(s) * n;
        const int* P = s > 0 ? lev.data() + size_t(s - 1) * n : nullptr;
        for (int c : byColor) {
            int v = P ? P[c] + 1 : 0;
            sched_entries(h, SCHED_GS, c, nbs, srcs);
            for (int nb : nbs) {
                if (color[nb] < color[c]) v = std::max(v, L[nb] + 1);
                else if (P) v = std::max(v, P[nb] + 1);
            }
            L[c] = v;
        }
    }
}
}  // namespace

int colored_gs() { return g_colored_gs; }
void set_colored_gs(int v) { g_colored_gs = v < 0 ? 0 : v > 2 ? 2 : v; }
int colored_pre() { return g_colored_pre; }
void set_colored_pre(int v) { g_colored_pre = v < 0 ? 0 : v > 3 ? 3 : v; }

int greedy_colors(const HostLevel& h, std::vector<int>& color) {
    const int n = h.n;
    color.assign(n, -1);
    std::vector<int> seen;  // seen[k] == c: colour k taken by a neighbour of c
    int nc = 0;
    for (int c = 0; c < n; ++c) {
        for (int q = h.losortStart[c]; q < h.losortStart[c + 1]; ++q) {
            const int k = color[h.losortL[q]];
            if (k >= int(seen.size())) seen.resize(k + 1, -1);
            seen[k] = c;
        }
        int k = 0;
        while (k < int(seen.size()) && seen[k] == c) ++k;
        color[c] = k;
        nc = std::max(nc, k + 1);
    }
    return nc;
}

void build_sched(const HostLevel& h, int kind, int nSweeps, HostSched& o, bool withDeps,
                 const std::vector<int>* color) {
    const int n = h.n;
    const int chunkGroups = g_chunk_groups;
    const int S = kind == SCHED_GS ? std::max(1, nSweeps) : 1;
    const bool colored = color != nullptr && (kind == SCHED_GS || kind == SCHED_FWD || kind == SCHED_BWD);
    if (colored) withDeps = false;
    // level of every (cell, sweep)
    std::vector<int> lev;
    if (colored)
        colored_levels(h, kind, *color, S, lev);
    else
        sched_levels(h, kind, S, lev);
    int nl = 0;
    for (int v : lev) nl = std::max(nl, v + 1);
    if (n == 0) nl = 0;
    // bucket (sweep-major, ascending cell) by level
    std::vector<int> cntL(nl + 1, 0);
    for (int v : lev) cntL[v + 1]++;
    std::vector<int> start(nl + 1, 0);
    for (int i = 0; i < nl; ++i) start[i + 1] = start[i] + cntL[i + 1];
    std::vector<int> order(lev.size());
    {
        std::vector<int> fill(start.begin(), start.end() - 1);
        for (size_t i = 0; i < lev.size(); ++i) order[fill[lev[i]]++] = int(i);
    }
    o.kind = kind;
    o.nSweeps = S;
    o.nLevels = nl;
    o.n = n;
    o.levelSlot.assign(nl + 1, 0);
    o.levelEntry.assign(nl + 1, 0);
    o.cell.clear();
    o.cnt.clear();
    o.nb.clear();
    o.src.clear();
    o.groupEntry.assign(1, 0);
    o.chunkGroup.assign(1, 0);
    o.chunkLevel.clear();
    o.levelChunks.assign(nl, 0);
    o.slotSweep.clear();
    o.slotLower.clear();
    o.maxK = 0;
    o.maxLevelBytes8 = 0;
    std::vector<int> cnb, csrc;
    int nLowerOf = 0;  // the colored form's lower-entry count of the last cell
    auto entries_of = [&](int c, std::vector<int>& nbs, std::vector<int>& srcs) {
        if (colored && kind != SCHED_GS) {
            // forward: the smaller-coloured neighbours in the Gauss-Seidel
            // entry order (losort slots, then owned faces); backward: the
            // larger-coloured ones in the reverse of that order
            sched_entries(h, SCHED_GS, c, cnb, csrc);
            nbs.clear();
            srcs.clear();
            const int m = int(cnb.size());
            for (int i = 0; i < m; ++i) {
                const int k = kind == SCHED_FWD ? i : m - 1 - i;
                if (kind == SCHED_FWD ? (*color)[cnb[k]] < (*color)[c] : (*color)[cnb[k]] > (*color)[c]) {
                    nbs.push_back(cnb[k]);
                    srcs.push_back(csrc[k]);
                }
            }
            return;
        }
        sched_entries(h, kind, c, nbs, srcs);
        if (!colored) return;
        // smaller-coloured neighbours first, then the larger-coloured ones,
        // each group in the reference's entry order
        cnb.clear();
        csrc.clear();
        for (int pass = 0; pass < 2; ++pass)
            for (size_t k = 0; k < nbs.size(); ++k)
                if (((*color)[nbs[k]] < (*color)[c]) == (pass == 0)) {
                    cnb.push_back(nbs[k]);
                    csrc.push_back(srcs[k]);
                }
        nLowerOf = 0;
        for (int nb : nbs) nLowerOf += (*color)[nb] < (*color)[c];
        nbs.swap(cnb);
        srcs.swap(csrc);
    };
    std::vector<int> nbs, srcs;
    std::vector<std::vector<int>> gnb(32), gsrc(32);
    for (int L = 0; L < nl; ++L) {
        o.levelSlot[L] = int(o.cell.size());
        o.levelEntry[L] = int(o.nb.size());
        const int b = start[L], e = start[L + 1];
        int groupsInChunk = 0;
        for (int g0 = b; g0 < e; g0 += 32) {
            int K = 0;
            for (int j = 0; j < 32; ++j) {
                const int i = g0 + j;
                if (i < e) {
                    const int c = order[i] % n;
                    entries_of(c, gnb[j], gsrc[j]);
                    o.cell.push_back(c);
                    o.cnt.push_back(int(gnb[j].size()));
                    o.slotSweep.push_back(order[i] / n);
                    o.slotLower.push_back(colored && kind == SCHED_GS ? nLowerOf
                                          : kind == SCHED_GS || kind == SCHED_GSB
                                              ? h.losortStart[c + 1] - h.losortStart[c] : 0);
                    K = std::max(K, int(gnb[j].size()));
                } else {
                    gnb[j].clear();
                    gsrc[j].clear();
                    o.cell.push_back(-1);
                    o.cnt.push_back(0);
                    o.slotSweep.push_back(0);
                    o.slotLower.push_back(0);
                }
            }
            for (int k = 0; k < K; ++k)
                for (int j = 0; j < 32; ++j) {
                    const bool has = k < int(gnb[j].size());
                    o.nb.push_back(has ? gnb[j][k] : 0);
                    o.src.push_back(has ? gsrc[j][k] : -1);
                }
            o.maxK = std::max(o.maxK, K);
            o.groupEntry.push_back(int(o.nb.size()));
            if (++groupsInChunk == chunkGroups || g0 + 32 >= e) {
                o.chunkGroup.push_back(int(o.groupEntry.size()) - 1);
                o.chunkLevel.push_back(L);
                o.levelChunks[L]++;
                groupsInChunk = 0;
            }
        }
        const int64_t slots = int64_t(o.cell.size()) - o.levelSlot[L];
        const int64_t ents = int64_t(o.nb.size()) - o.levelEntry[L];
        o.maxLevelBytes8 = std::max<int64_t>(o.maxLevelBytes8, slots * 16 + ents * 12);
    }
    o.levelSlot[nl] = int(o.cell.size());
    o.levelEntry[nl] = int(o.nb.size());
    // group dependencies (only for the wavefront form): the groups holding every (cell, sweep) a group's
    // slots read (lower neighbours in the same sweep; for Gauss-Seidel the
    // upper neighbours and the cell itself in the previous sweep)
    o.depStart.clear();
    o.dep.clear();
    o.waveOk = false;
    if (!withDeps) return;
    std::vector<int> slotOf(size_t(n) * S, -1);
    for (int L = 0; L < nl; ++L)
        for (int i = start[L]; i < start[L + 1]; ++i) slotOf[order[i]] = o.levelSlot[L] + (i - start[L]);
    const int nGroups = int(o.groupEntry.size()) - 1;
    o.depStart.assign(1, 0);
    o.dep.clear();
    o.waveOk = true;
    std::vector<int> ds;
    int L = 0;  // level of group g (groups are in level order)
    for (int g = 0; g < nGroups; ++g) {
        ds.clear();
        while (o.levelSlot[L + 1] <= g * 32) ++L;
        for (int j = 0; j < 32; ++j) {
            const int slot = g * 32 + j;
            const int c = o.cell[slot];
            if (c < 0) continue;
            // the sweep of this slot: its index in the (sweep, cell) order
            int sw = 0;
            if (S > 1) {
                sw = order[start[L] + (slot - o.levelSlot[L])] / n;
                if (sw > 0) ds.push_back(slotOf[size_t(sw - 1) * n + c] / 32);
            }
            for (int k = 0; k < o.cnt[slot]; ++k) {
                const int e = o.groupEntry[g] + 32 * k + j;
                const int nb = o.nb[e];
                // the backward pass reads its lower neighbours' values from
                // before the kernel: no dependency
                if (kind == SCHED_GSB && !(o.src[e] & SRC_UPPER)) continue;
                const bool prev = kind == SCHED_GS && (o.src[e] & SRC_UPPER);
                const int s2 = prev ? sw - 1 : sw;
                if (s2 < 0) continue;
                ds.push_back(slotOf[size_t(s2) * n + nb] / 32);
            }
        }
        std::sort(ds.begin(), ds.end());
        ds.erase(std::unique(ds.begin(), ds.end()), ds.end());
        // every source lies on an earlier level, hence in an earlier group:
        // the wavefront form's waits rely on it, so a violation disables it
        if (!ds.empty() && ds.back() >= g) o.waveOk = false;
        for (int d : ds) o.dep.push_back(d);
        o.depStart.push_back(int(o.dep.size()));
    }
}

// The level's rows in sliced ELL form (Sell in device.cuh): slices of 32
// rows, each row's entries in the reference's order (losort slots, then
// owner faces), stored in pairs: entry k of row c at
// start[c/32] + 64*(k/2) + 2*(c%32) + k%2.  With patterns, a slice whose
// rows' neighbour offsets are each ascending and together take at most 8
// values becomes a pattern slice: its entries sit at the offsets' positions
// in the slice's sorted offset list, cnt[c] is the row's offset mask, and no
// column is read.  False (nothing built) when a row has more than 255
// entries or the entries overflow 32-bit indices.
bool build_sell(const HostLevel& h, bool patterns, HostSell& out) {
    const int n = h.n;
    const int ns = (n + 31) / 32;
    out = HostSell();
    std::vector<unsigned char>& cnt = out.cnt;
    cnt.assign(n, 0);
    for (int c = 0; c < n; ++c) {
        const int k = (h.losortStart[c + 1] - h.losortStart[c]) + (h.ownerStart[c + 1] - h.ownerStart[c]);
        if (k > 255) return false;
        cnt[c] = static_cast<unsigned char>(k);
    }
    // each row's neighbours in the product's order: (column, coefficient source)
    auto row = [&](int c, std::vector<std::pair<int, int>>& nb) {
        nb.clear();
        for (int q = h.losortStart[c]; q < h.losortStart[c + 1]; ++q) nb.emplace_back(h.losortL[q], q);
        for (int f = h.ownerStart[c]; f < h.ownerStart[c + 1]; ++f) nb.emplace_back(h.u[f], f | SRC_UPPER);
    };
    std::vector<int>& start = out.start;
    std::vector<int>& pat = out.pat;
    start.assign(ns + 1, 0);
    pat.assign(ns, -1);
    std::map<std::vector<int>, int> patIndex;
    std::vector<std::vector<int>> slicePat(ns);
    std::vector<std::pair<int, int>> nb;
    int64_t nE = 0;
    for (int sl = 0; sl < ns; ++sl) {
        const int c0 = 32 * sl, c1 = std::min(n, c0 + 32);
        int K = 0;
        for (int c = c0; c < c1; ++c) K = std::max(K, int(cnt[c]));
        std::vector<int> u;
        bool ok = patterns;
        for (int c = c0; c < c1 && ok; ++c) {
            row(c, nb);
            for (size_t k = 0; k < nb.size(); ++k) {
                if (k && nb[k].first <= nb[k - 1].first) ok = false;
                u.push_back(nb[k].first - c);
            }
        }
        if (ok) {
            std::sort(u.begin(), u.end());
            u.erase(std::unique(u.begin(), u.end()), u.end());
            ok = !u.empty() && u.size() <= 8;
        }
        if (ok) {
            if (u.size() & 1) u.push_back(u.back());  // pad to the pair width (sorted); its bit is never set
            auto it = patIndex.find(u);
            if (it == patIndex.end()) {
                const int idx = int(patIndex.size());
                it = patIndex.emplace(u, idx).first;
                std::vector<int> o(8, 0);
                std::copy(u.begin(), u.end(), o.begin());
                out.offs.insert(out.offs.end(), o.begin(), o.end());
            }
            pat[sl] = it->second;
            K = int(u.size());
            slicePat[sl] = u;
        }
        K = (K + 1) & ~1;
        nE += 32 * int64_t(K);
        if (nE > std::numeric_limits<int>::max()) return false;  // entry indices are 32-bit
        start[sl + 1] = int(nE);
    }
    out.col.assign(std::max<int64_t>(nE, 1), 0);
    out.src.assign(std::max<int64_t>(nE, 1), -1);
    int nPat = 0;
    for (int sl = 0; sl < ns; ++sl) {
        const int K = (start[sl + 1] - start[sl]) / 32;
        const bool isPat = pat[sl] >= 0;
        nPat += isPat;
        for (int c = 32 * sl; c < std::min(n, 32 * sl + 32); ++c) {
            const int j = c & 31;
            auto at = [&](int k) { return int64_t(start[sl]) + 64 * (k >> 1) + 2 * j + (k & 1); };
            for (int k = 0; k < K; ++k) out.col[at(k)] = c;  // padding: a valid column, never read
            row(c, nb);
            if (isPat) {
                const std::vector<int>& u = slicePat[sl];
                unsigned mask = 0;
                for (const auto& e : nb) {
                    const int k = int(std::lower_bound(u.begin(), u.end(), e.first - c) - u.begin());
                    out.col[at(k)] = e.first;
                    out.src[at(k)] = e.second;
                    mask |= 1u << k;
                }
                cnt[c] = static_cast<unsigned char>(mask);
            } else {
                for (size_t k = 0; k < nb.size(); ++k) {
                    out.col[at(int(k))] = nb[k].first;
                    out.src[at(int(k))] = nb[k].second;
                }
            }
        }
    }
    out.entries = nE;
    out.patterns = int(patIndex.size());
    out.patternSlices = nPat;
    return true;
}

}  // namespace cfx
