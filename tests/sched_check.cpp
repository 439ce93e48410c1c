// The packed sweep schedules built on the host (build_sched in csrc/host.cpp),
// checked against the dependencies they must respect: every (cell, sweep)
// is exactly one slot; every entry names a real neighbour with the
// coefficient source of that neighbour's face; and every value a slot reads
// is produced at an earlier DAG level (or, for a Gauss-Seidel upper entry of
// the first sweep, is the value before the sweep).  The reference order:
// forward entries are the losort slots (lower neighbours) in order, backward
// entries the owned faces in decreasing order, Gauss-Seidel the losort slots
// then the owned faces.  The multicolour order (greedy colours, which must
// be a proper colouring): forward entries are the smaller-coloured
// neighbours, backward entries the larger-coloured ones, Gauss-Seidel the
// smaller-coloured (this sweep) then the larger-coloured (previous sweep).
// Input: a binary file of n, nf, l[nf], u[nf] (int32).  Prints one line per
// schedule and exits 1 on the first violation.
#include <cstdio>
#include <string>
#include <vector>

#include "internal.h"

namespace cfx {
void set_error(const std::string&) {}
}  // namespace cfx

using namespace cfx;

namespace {

int fail(const char* what, int kind, int colored, int slot) {
    std::printf("kind=%d colored=%d slot %d: %s\n", kind, colored, slot, what);
    return 1;
}

// the neighbour and the cell's own index that coefficient source src names
bool source_ok(const HostLevel& h, int c, int nb, int src) {
    if (src & SRC_UPPER) {
        const int f = src & (SRC_UPPER - 1);
        return f >= 0 && f < h.nf && h.l[f] == c && h.u[f] == nb;
    }
    return src >= h.losortStart[c] && src < h.losortStart[c + 1] && h.losortL[src] == nb;
}

int check(const HostLevel& h, int kind, int S, const std::vector<int>* color) {
    HostSched o;
    build_sched(h, kind, S, o, false, color);
    const int n = h.n;
    const int sweeps = kind == SCHED_GS ? S : 1;
    const bool col = color != nullptr;
    std::vector<int> levelOf(size_t(n) * sweeps, -1);
    // level of every slot
    for (int L = 0; L < o.nLevels; ++L)
        for (int t = o.levelSlot[L]; t < o.levelSlot[L + 1]; ++t) {
            const int c = o.cell[t];
            if (c < 0) continue;
            const int sw = kind == SCHED_GS ? o.slotSweep[t] : 0;
            if (c >= n || sw < 0 || sw >= sweeps) return fail("cell or sweep out of range", kind, col, t);
            int& lv = levelOf[size_t(sw) * n + c];
            if (lv >= 0) return fail("(cell, sweep) twice", kind, col, t);
            lv = L;
        }
    for (int v : levelOf)
        if (v < 0) return fail("a (cell, sweep) without a slot", kind, col, -1);
    for (int L = 0; L < o.nLevels; ++L)
        for (int t = o.levelSlot[L]; t < o.levelSlot[L + 1]; ++t) {
            const int c = o.cell[t];
            if (c < 0) continue;
            const int g = t / 32, lane = t % 32;
            const int sw = kind == SCHED_GS ? o.slotSweep[t] : 0;
            // the entries the slot must have, in order
            std::vector<int> want;
            std::vector<int> gsNb;  // Gauss-Seidel order: losort slots, then owned faces
            for (int q = h.losortStart[c]; q < h.losortStart[c + 1]; ++q) gsNb.push_back(h.losortL[q]);
            for (int f = h.ownerStart[c]; f < h.ownerStart[c + 1]; ++f) gsNb.push_back(h.u[f]);
            int nLower = 0;
            if (!col) {
                if (kind == SCHED_FWD || kind == SCHED_GS)
                    for (int q = h.losortStart[c]; q < h.losortStart[c + 1]; ++q) want.push_back(h.losortL[q]);
                if (kind == SCHED_GS)
                    for (int f = h.ownerStart[c]; f < h.ownerStart[c + 1]; ++f) want.push_back(h.u[f]);
                if (kind == SCHED_BWD)
                    for (int f = h.ownerStart[c + 1] - 1; f >= h.ownerStart[c]; --f) want.push_back(h.u[f]);
                nLower = h.losortStart[c + 1] - h.losortStart[c];
            } else {
                const std::vector<int>& k = *color;
                if (kind == SCHED_FWD || kind == SCHED_GS)
                    for (int nb : gsNb)
                        if (k[nb] < k[c]) want.push_back(nb);
                nLower = int(want.size());
                if (kind == SCHED_GS)
                    for (int nb : gsNb)
                        if (k[nb] > k[c]) want.push_back(nb);
                if (kind == SCHED_BWD)
                    for (int i = int(gsNb.size()) - 1; i >= 0; --i)
                        if (k[gsNb[i]] > k[c]) want.push_back(gsNb[i]);
            }
            if (o.cnt[t] != int(want.size())) return fail("entry count", kind, col, t);
            if (kind == SCHED_GS && o.slotLower[t] != nLower) return fail("lower-entry count", kind, col, t);
            for (int e = 0; e < o.cnt[t]; ++e) {
                const size_t i = size_t(o.groupEntry[g]) + 32 * size_t(e) + lane;
                const int nb = o.nb[i];
                if (nb != want[e]) return fail("entry order", kind, col, t);
                if (!source_ok(h, c, nb, o.src[i])) return fail("coefficient source", kind, col, t);
                // the value read: this sweep's for lower entries (forward,
                // backward: every entry), the previous sweep's for upper ones
                const bool lower = kind != SCHED_GS || e < nLower;
                const int rs = lower ? sw : sw - 1;
                if (rs < 0) continue;  // the value before the sweep
                if (levelOf[size_t(rs) * n + nb] >= L) return fail("reads a value not yet produced", kind, col, t);
            }
            if (kind == SCHED_GS && sw > 0 && levelOf[size_t(sw - 1) * n + c] >= L)
                return fail("runs before its own previous sweep", kind, col, t);
        }
    std::printf("kind=%d sweeps=%d colored=%d levels=%d slots=%d entries=%d ok\n", kind, sweeps, int(col), o.nLevels,
                int(o.cell.size()), int(o.nb.size()));
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 2) return 2;
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int n = 0, nf = 0;
    if (std::fread(&n, 4, 1, f) != 1 || std::fread(&nf, 4, 1, f) != 1) return 2;
    std::vector<int> l(nf), u(nf);
    if (std::fread(l.data(), 4, nf, f) != size_t(nf) || std::fread(u.data(), 4, nf, f) != size_t(nf)) return 2;
    std::fclose(f);
    HostLevel h;
    if (build_host_level(n, nf, l.data(), u.data(), h, true) != CFX_OK) return 3;
    std::vector<int> color;
    const int nc = greedy_colors(h, color);
    for (int fc = 0; fc < nf; ++fc)
        if (color[l[fc]] == color[u[fc]]) {
            std::printf("face %d joins two cells of colour %d\n", fc, color[l[fc]]);
            return 1;
        }
    std::printf("colours=%d\n", nc);
    for (int colored = 0; colored < 2; ++colored) {
        const std::vector<int>* cp = colored ? &color : nullptr;
        if (check(h, SCHED_FWD, 1, cp) || check(h, SCHED_BWD, 1, cp)) return 1;
        for (int S : {1, 2, 3})
            if (check(h, SCHED_GS, S, cp)) return 1;
    }
    return 0;
}
