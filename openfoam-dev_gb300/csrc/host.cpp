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

// The (sweep, cell) slot whose value an entry reads, or -1 when it reads a
// value from before the launch: lower neighbours in the same sweep, upper
// neighbours in the previous sweep (Gauss-Seidel), upper neighbours in the
// same pass (backward sweeps; the backward Gauss-Seidel pass reads its lower
// neighbours' values from before it).
inline int64_t entry_producer(int kind, int n, int sweep, int nb, int src) {
    const bool upper = (src & SRC_UPPER) != 0;
    if (kind == SCHED_FWD) return nb;
    if (kind == SCHED_BWD) return nb;
    if (kind == SCHED_GSB) return upper ? nb : -1;
    if (!upper) return int64_t(sweep) * n + nb;  // SCHED_GS, same sweep
    return sweep > 0 ? int64_t(sweep - 1) * n + nb : -1;
}

}  // namespace

void build_sched(const HostLevel& h, int kind, int nSweeps, HostSched& o, bool withDeps) {
    const int n = h.n;
    const int S = kind == SCHED_GS ? std::max(1, nSweeps) : 1;
    // level of every (cell, sweep)
    std::vector<int> lev;
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
    o.maxK = 0;
    o.maxLevelBytes8 = 0;
    auto entries_of = [&](int c, std::vector<int>& nbs, std::vector<int>& srcs) {
        sched_entries(h, kind, c, nbs, srcs);
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
                    K = std::max(K, int(gnb[j].size()));
                } else {
                    gnb[j].clear();
                    gsrc[j].clear();
                    o.cell.push_back(-1);
                    o.cnt.push_back(0);
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
            if (++groupsInChunk == SCHED_CHUNK_GROUPS || g0 + 32 >= e) {
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

// Tiled schedule.  The levels are cut into bands of Lb consecutive levels;
// a band's slots, in (sweep, cell) order -- ascending cells, or descending
// for the backward sweeps, a topological order of the sweep's DAG -- are
// split into equal tiles of at most tileCells distinct cells.  Every
// dependency between tiles of one band then runs from a lower to a higher
// tile, and dependencies between bands from an earlier to a later band.  A
// tile runs on one CTA, level by level (a segment per level), with the
// values it produces kept in shared memory at tile-local indices; values
// from other tiles (or from before the launch) are read from global memory
// after waiting for the producing tile's published progress.  Tile j of a
// band goes to CTA j, so a CTA holds at most one tile per band and works
// through its tiles band by band: with every CTA resident, the tile holding
// the lowest unfinished level can always proceed.
bool build_sched_tiled(const HostLevel& h, int kind, int nSweeps, int tileCells, int maxCtas, int pubEvery,
                       HostSched& o) {
    const int n = h.n;
    const int S = kind == SCHED_GS ? std::max(1, nSweeps) : 1;
    if (n == 0 || tileCells < 32 || maxCtas < 1) return false;
    std::vector<int> lev;
    sched_levels(h, kind, S, lev);
    const int64_t nSlot = int64_t(n) * S;
    int nl = 0;
    for (int v : lev) nl = std::max(nl, v + 1);
    std::vector<int64_t> width(nl, 0);
    for (int v : lev) width[v]++;
    // band height: the largest of 32, 16, ... whose bands need at most
    // maxCtas tiles each (by slots, which bound the distinct cells)
    int Lb = 32;
    for (;;) {
        bool ok = true;
        for (int b0 = 0; b0 < nl && ok; b0 += Lb) {
            int64_t m = 0;
            for (int L = b0; L < std::min(nl, b0 + Lb); ++L) m += width[L];
            if ((m + tileCells - 1) / tileCells > maxCtas) ok = false;
        }
        if (ok) break;
        if (Lb == 1) return false;
        Lb /= 2;
    }
    const int nb = (nl + Lb - 1) / Lb;
    const bool desc = kind == SCHED_BWD || kind == SCHED_GSB;
    // slots of each band in (sweep, cell) order
    std::vector<int64_t> bandStart(nb + 1, 0);
    for (int v : lev) bandStart[v / Lb + 1]++;
    for (int b = 0; b < nb; ++b) bandStart[b + 1] += bandStart[b];
    std::vector<int64_t> bandSlots(nSlot);
    {
        std::vector<int64_t> fill(bandStart.begin(), bandStart.end() - 1);
        for (int sw = 0; sw < S; ++sw)
            for (int i = 0; i < n; ++i) {
                const int c = desc ? n - 1 - i : i;
                const int64_t sl = int64_t(sw) * n + c;
                bandSlots[fill[lev[sl] / Lb]++] = sl;
            }
    }
    // tiles: equal slot counts within a band
    std::vector<int> tileOf(nSlot), tileBand, tileFirst;  // tileFirst: position of the tile in its band
    std::vector<int> bandTiles(nb), bandTile0(nb + 1, 0);
    int nTiles = 0;
    for (int b = 0; b < nb; ++b) {
        const int64_t m = bandStart[b + 1] - bandStart[b];
        const int R = int(std::max<int64_t>(1, (m + tileCells - 1) / tileCells));
        const int64_t per = (m + R - 1) / R;
        for (int64_t i = 0; i < m; ++i) tileOf[bandSlots[bandStart[b] + i]] = nTiles + int(i / per);
        const int R2 = m ? int((m - 1) / per) + 1 : 1;  // tiles actually filled
        for (int j = 0; j < R2; ++j) {
            tileBand.push_back(b);
            tileFirst.push_back(j);
        }
        bandTiles[b] = R2;
        nTiles += R2;
        bandTile0[b + 1] = nTiles;
    }
    // each tile's slots by level (segments), each level in band order
    std::vector<int64_t> tileStart(nTiles + 1, 0);
    for (int64_t i = 0; i < nSlot; ++i) tileStart[tileOf[i] + 1]++;
    for (int t = 0; t < nTiles; ++t) tileStart[t + 1] += tileStart[t];
    std::vector<int64_t> tileSlots(nSlot);
    {
        std::vector<int64_t> fill(tileStart.begin(), tileStart.end() - 1);
        for (int b = 0; b < nb; ++b)
            for (int64_t i = bandStart[b]; i < bandStart[b + 1]; ++i) {
                const int64_t sl = bandSlots[i];
                tileSlots[fill[tileOf[sl]]++] = sl;
            }
    }
    std::vector<int64_t>().swap(bandSlots);
    // segment of each slot within its tile; tile-local cell indices
    std::vector<int> segOf(nSlot), localOf(n, -1), stamp(n, -1), nSegOf(nTiles, 0);
    o.kind = kind;
    o.nSweeps = S;
    o.nLevels = nl;
    o.n = n;
    o.levelSlot.clear();
    o.levelEntry.clear();
    o.chunkGroup.clear();
    o.chunkLevel.clear();
    o.levelChunks.clear();
    o.depStart.clear();
    o.dep.clear();
    o.waveOk = false;
    o.cell.clear();
    o.cnt.clear();
    o.nb.clear();
    o.src.clear();
    o.slotLocal.clear();
    o.groupEntry.assign(1, 0);
    o.tileSeg.assign(1, 0);
    o.segGroup.assign(1, 0);
    o.maxK = 0;
    o.maxTileCells = 0;
    o.maxLevelBytes8 = 0;
    // first pass: segments and local indices (the waits need every slot's segment)
    std::vector<std::vector<int64_t>> segs;
    std::vector<int> segLevel;
    std::vector<int64_t> segBase(nTiles + 1, 0);
    for (int t = 0; t < nTiles; ++t) {
        // stable bucket of the tile's slots by level
        const int b = tileBand[t];
        const int L0 = b * Lb, L1 = std::min(nl, L0 + Lb);
        std::vector<std::vector<int64_t>> byL(L1 - L0);
        int nLocal = 0;
        for (int64_t i = tileStart[t]; i < tileStart[t + 1]; ++i) {
            const int64_t sl = tileSlots[i];
            byL[lev[sl] - L0].push_back(sl);
            const int c = int(sl % n);
            if (stamp[c] != t) {
                stamp[c] = t;
                localOf[c] = nLocal++;
            }
        }
        o.maxTileCells = std::max(o.maxTileCells, nLocal);
        int q = 0;
        for (int L = L0; L < L1; ++L) {
            if (byL[L - L0].empty()) continue;
            for (int64_t sl : byL[L - L0]) segOf[sl] = q;
            segs.push_back(std::move(byL[L - L0]));
            segLevel.push_back(L);
            ++q;
        }
        nSegOf[t] = q;
        segBase[t + 1] = segBase[t] + q;
    }
    // second pass: groups, entries (local or global reads), waits
    std::fill(stamp.begin(), stamp.end(), -1);
    std::vector<int> nbs, srcs;
    std::vector<std::vector<int>> gnb(32), gsrc(32);
    std::vector<int> waitNeedOf(nTiles, 0), waitList;
    o.segWait.assign(1, 0);
    o.waitTile.clear();
    o.waitNeed.clear();
    auto need = [&](int p, int q) {  // tile p must have published q + 1 segments
        int k = q + 1;
        if (pubEvery > 1) k = std::min(((k + pubEvery - 1) / pubEvery) * pubEvery, nSegOf[p]);
        if (waitNeedOf[p] == 0) waitList.push_back(p);
        waitNeedOf[p] = std::max(waitNeedOf[p], k);
    };
    int64_t gseg = 0;
    for (int t = 0; t < nTiles; ++t) {
        // local indices again (the first pass's were overwritten by later tiles)
        int nLocal = 0;
        for (int64_t i = tileStart[t]; i < tileStart[t + 1]; ++i) {
            const int c = int(tileSlots[i] % n);
            if (stamp[c] != t) {
                stamp[c] = t;
                localOf[c] = nLocal++;
            }
        }
        for (int q = 0; q < nSegOf[t]; ++q, ++gseg) {
            const std::vector<int64_t>& seg = segs[gseg];
            waitList.clear();
            for (size_t g0 = 0; g0 < seg.size(); g0 += 32) {
                int K = 0;
                int cellsL[32];
                for (int j = 0; j < 32; ++j) {
                    const size_t i = g0 + j;
                    if (i < seg.size()) {
                        const int64_t sl = seg[i];
                        const int c = int(sl % n), sw = int(sl / n);
                        sched_entries(h, kind, c, nbs, srcs);
                        gnb[j].assign(nbs.size(), 0);
                        gsrc[j] = srcs;
                        for (size_t k = 0; k < nbs.size(); ++k) {
                            const int64_t pr = entry_producer(kind, n, sw, nbs[k], srcs[k]);
                            if (pr >= 0 && tileOf[pr] == t) {
                                gnb[j][k] = localOf[nbs[k]];
                            } else {
                                gnb[j][k] = -(nbs[k] + 1);
                                if (pr >= 0) need(tileOf[pr], segOf[pr]);
                            }
                        }
                        // a later sweep of the same cell overwrites the earlier one's value
                        if (sw > 0) {
                            const int64_t pr = sl - n;
                            if (tileOf[pr] != t) need(tileOf[pr], segOf[pr]);
                        }
                        o.cell.push_back(c);
                        o.cnt.push_back(int(nbs.size()));
                        o.slotLocal.push_back(localOf[c]);
                        cellsL[j] = c;
                        K = std::max(K, int(nbs.size()));
                    } else {
                        gnb[j].clear();
                        gsrc[j].clear();
                        o.cell.push_back(-1);
                        o.cnt.push_back(0);
                        o.slotLocal.push_back(0);
                        cellsL[j] = -1;
                    }
                }
                (void)cellsL;
                for (int k = 0; k < K; ++k)
                    for (int j = 0; j < 32; ++j) {
                        const bool has = k < int(gnb[j].size());
                        o.nb.push_back(has ? gnb[j][k] : -1);
                        o.src.push_back(has ? gsrc[j][k] : -1);
                    }
                o.maxK = std::max(o.maxK, K);
                o.groupEntry.push_back(int(o.nb.size()));
            }
            std::sort(waitList.begin(), waitList.end());
            for (int p : waitList) {
                o.waitTile.push_back(p);
                o.waitNeed.push_back(waitNeedOf[p]);
                waitNeedOf[p] = 0;
            }
            o.segWait.push_back(int(o.waitTile.size()));
            o.segGroup.push_back(int(o.groupEntry.size()) - 1);
        }
        o.tileSeg.push_back(int(gseg));
    }
    o.tiled = true;
    o.nTiles = nTiles;
    o.nSegs = int(gseg);
    o.pubEvery = std::max(1, pubEvery);
    int grid = 0;
    for (int b = 0; b < nb; ++b) grid = std::max(grid, bandTiles[b]);
    o.grid = grid;
    o.ctaTile.assign(grid + 1, 0);
    for (int t = 0; t < nTiles; ++t) o.ctaTile[tileFirst[t] + 1]++;
    for (int j = 0; j < grid; ++j) o.ctaTile[j + 1] += o.ctaTile[j];
    o.ctaTiles.assign(nTiles, 0);
    {
        std::vector<int> fill(o.ctaTile.begin(), o.ctaTile.end() - 1);
        for (int t = 0; t < nTiles; ++t) o.ctaTiles[fill[tileFirst[t]]++] = t;  // bands in order
    }
    (void)bandTile0;
    (void)segLevel;
    return true;
}


// Structural check of a tiled schedule against the sweep it stands for:
// every (sweep, cell) slot exactly once; each slot's entries in the
// reference's order, reading the neighbour the sweep reads; a value read from
// shared memory was produced earlier in the same tile and is still the
// version the sweep reads there; every value produced by another tile is read
// from global memory after a wait that covers the producing segment (or
// after the same CTA finished that tile); every wait is on a tile of an
// lower tile and every CTA takes its tiles in increasing order (with all
// CTAs resident this rules out deadlock); shared-memory indices stay below
// maxTileCells.
bool check_sched_tiled(const HostLevel& h, const HostSched& o, std::string& why) {
    const int n = h.n, S = o.nSweeps, kind = o.kind;
    auto fail = [&](const std::string& w) {
        why = w;
        return false;
    };
    if (!o.tiled) return fail("not tiled");
    const int64_t nSlot = int64_t(n) * S;
    std::vector<int> occ(n, 0), tileOfSlot(nSlot, -1), segOfSlot(nSlot, -1);
    // band and position of every tile, from the CTA lists (tile j of a band on CTA j)
    std::vector<int> ctaOf(o.nTiles, -1), orderOnCta(o.nTiles, -1);
    for (int j = 0; j < o.grid; ++j)
        for (int k = o.ctaTile[j]; k < o.ctaTile[j + 1]; ++k) {
            const int t = o.ctaTiles[k];
            if (t < 0 || t >= o.nTiles || ctaOf[t] >= 0) return fail("CTA lists do not cover each tile once");
            ctaOf[t] = j;
            orderOnCta[t] = k - o.ctaTile[j];
        }
    for (int t = 0; t < o.nTiles; ++t)
        if (ctaOf[t] < 0) return fail("a tile is on no CTA");
    // a CTA's tiles in increasing tile index (bands in order)
    for (int j = 0; j < o.grid; ++j)
        for (int k = o.ctaTile[j] + 1; k < o.ctaTile[j + 1]; ++k)
            if (o.ctaTiles[k] <= o.ctaTiles[k - 1]) return fail("a CTA's tiles are out of order");
    std::vector<int> sweepOf(o.cell.size(), -1);
    std::vector<int> nbs, srcs;
    std::vector<int> localCell(std::max(o.maxTileCells, 1), -1), localVer(std::max(o.maxTileCells, 1), -1);
    std::vector<int> guaranteed(o.nTiles, 0);
    for (int t = 0; t < o.nTiles; ++t) {
        std::fill(localCell.begin(), localCell.end(), -1);
        std::fill(localVer.begin(), localVer.end(), -1);
        std::fill(guaranteed.begin(), guaranteed.end(), 0);
        // tiles finished earlier on the same CTA
        for (int k = o.ctaTile[ctaOf[t]]; k < o.ctaTile[ctaOf[t]] + orderOnCta[t]; ++k) {
            const int p = o.ctaTiles[k];
            guaranteed[p] = o.tileSeg[p + 1] - o.tileSeg[p];
        }
        for (int q = o.tileSeg[t]; q < o.tileSeg[t + 1]; ++q) {
            const int qi = q - o.tileSeg[t];
            for (int k = o.segWait[q]; k < o.segWait[q + 1]; ++k) {
                const int p = o.waitTile[k];
                // waits only on lower tiles, and each CTA takes its tiles in
                // increasing order: the lowest unfinished tile can always run
                if (p < 0 || p >= t) return fail("a wait on the same or a later tile");
                const int np = o.tileSeg[p + 1] - o.tileSeg[p];
                if (o.waitNeed[k] < 1 || o.waitNeed[k] > np) return fail("a wait beyond the producer's segments");
                const int need = o.waitNeed[k];
                if (need % o.pubEvery != 0 && need != np) return fail("a wait on a count that is never published");
                guaranteed[p] = std::max(guaranteed[p], need);
            }
            for (int g = o.segGroup[q]; g < o.segGroup[q + 1]; ++g)
                for (int j = 0; j < 32; ++j) {
                    const int slot = g * 32 + j;
                    const int c = o.cell[slot];
                    if (c < 0) continue;
                    const int sw = occ[c]++;
                    if (sw >= S) return fail("a cell has more slots than sweeps");
                    const int64_t sl = int64_t(sw) * n + c;
                    tileOfSlot[sl] = t;
                    segOfSlot[sl] = qi;
                    sweepOf[slot] = sw;
                    sched_entries(h, kind, c, nbs, srcs);
                    if (o.cnt[slot] != int(nbs.size())) return fail("entry count");
                    for (int e = 0; e < o.cnt[slot]; ++e) {
                        const int ei = o.groupEntry[g] + 32 * e + j;
                        if (o.src[ei] != srcs[e]) return fail("entry order");
                        const int enc = o.nb[ei];
                        const int64_t pr = entry_producer(kind, n, sw, nbs[e], srcs[e]);
                        if (enc >= 0) {
                            if (enc >= o.maxTileCells || localCell[enc] != nbs[e])
                                return fail("a shared-memory read of another cell");
                            if (pr < 0 || tileOfSlot[pr] != t) return fail("a shared-memory read of a value from elsewhere");
                            if (localVer[enc] != int(pr / n)) return fail("a shared-memory read of a stale sweep");
                        } else {
                            if (-enc - 1 != nbs[e]) return fail("a global read of another cell");
                            if (pr >= 0) {
                                const int p = tileOfSlot[pr];
                                if (p < 0) return fail("a read of a value not yet produced");
                                if (p == t) return fail("a global read of a value of this tile");
                                if (guaranteed[p] < segOfSlot[pr] + 1) return fail("a cross-tile read without a wait");
                            }
                        }
                    }
                    if (sw > 0) {
                        const int p = tileOfSlot[sl - n];
                        if (p < 0) return fail("a later sweep before the earlier one");
                        if (p != t && guaranteed[p] < segOfSlot[sl - n] + 1)
                            return fail("an overwrite without waiting for the earlier sweep");
                    }
                    const int loc = o.slotLocal[slot];
                    if (loc < 0 || loc >= o.maxTileCells) return fail("local index out of range");
                    if (localCell[loc] >= 0 && localCell[loc] != c) return fail("two cells share a local index");
                    localCell[loc] = c;
                    localVer[loc] = sw;
                }
        }
    }
    for (int c = 0; c < n; ++c)
        if (occ[c] != S) return fail("a slot is missing");
    return true;
}

}  // namespace cfx
