// The sliced ELL rows built on the host (build_sell in csrc/host.cpp), read
// back the way the device reads them (Sell/sell_row in csrc/device.cuh):
// every row's entries must come back in the product's order (the losort
// neighbours, then the owned faces), with each entry's coefficient source,
// and every padding entry must name a valid column.  Input: a binary file of
// n, nf, l[nf], u[nf] (int32).  Prints one line per form and exits 1 on the
// first mismatch.
#include <cstdio>
#include <string>
#include <vector>

#include "internal.h"

namespace cfx {
void set_error(const std::string&) {}
}  // namespace cfx

using namespace cfx;

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
    for (int patterns = 0; patterns < 2; ++patterns) {
        HostSell s;
        if (!build_sell(h, patterns != 0, s)) {
            std::printf("patterns=%d not built\n", patterns);
            continue;
        }
        const int ns = (n + 31) / 32;
        for (int c = 0; c < n; ++c) {
            const int sl = c >> 5, j = c & 31;
            const int K = (s.start[sl + 1] - s.start[sl]) / 32;
            std::vector<int> col, src;
            for (int k = 0; k < K; ++k) {
                const long e = s.start[sl] + 64L * (k >> 1) + 2 * j + (k & 1);
                if (s.col[e] < 0 || s.col[e] >= n) {
                    std::printf("row %d entry %d: column %d out of range\n", c, k, s.col[e]);
                    return 1;
                }
                const int p = s.pat[sl];
                const bool present = p >= 0 ? ((s.cnt[c] >> k) & 1) != 0 : k < s.cnt[c];
                if (!present) continue;
                if (p >= 0 && s.col[e] != c + s.offs[8 * p + k]) {
                    std::printf("row %d entry %d: pattern offset disagrees with the column\n", c, k);
                    return 1;
                }
                col.push_back(s.col[e]);
                src.push_back(s.src[e]);
            }
            std::vector<int> rcol, rsrc;
            for (int q = h.losortStart[c]; q < h.losortStart[c + 1]; ++q) {
                rcol.push_back(h.losortL[q]);
                rsrc.push_back(q);
            }
            for (int g = h.ownerStart[c]; g < h.ownerStart[c + 1]; ++g) {
                rcol.push_back(h.u[g]);
                rsrc.push_back(g | SRC_UPPER);
            }
            if (col != rcol || src != rsrc) {
                std::printf("row %d: entries differ from the product's order\n", c);
                return 1;
            }
        }
        std::printf("patterns=%d slices=%d patternSlices=%d entries=%lld ok\n", patterns, ns, s.patternSlices,
                    static_cast<long long>(s.entries));
    }
    return 0;
}
