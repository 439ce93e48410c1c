// cases.cpp - seeded synthetic LDU systems (host only).  See cases.h.
//
// Compiled with -ffp-contract=off so that the geometry is evaluated with the
// same operation order and rounding as the reference's x86-64 build.

#include "cases.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <deque>
#include <limits>
#include <numeric>
#include <random>
#include <vector>

namespace {

struct V3 {
    double x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 operator/(V3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
// Foam::Vector operator^ (src/OpenFOAM/primitives/Vector/VectorI.H:152-160)
inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double mag(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline V3 ld(const double* p, int64_t i) { return {p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }
inline void st(double* p, int64_t i, V3 v) {
    p[3 * i] = v.x;
    p[3 * i + 1] = v.y;
    p[3 * i + 2] = v.z;
}

// OpenFOAM doubleScalarVSmall = numeric_limits<double>::min() and its root
// (src/OpenFOAM/primitives/Scalar/doubleScalar/doubleScalar.H:55-66)
const double vSmall = std::numeric_limits<double>::min();
const double rootVSmall = std::sqrt(std::numeric_limits<double>::min());

inline double u01(std::mt19937_64& g) { return double(g() >> 11) * 0x1.0p-53; }

}  // namespace

extern "C" {

int cfxc_box_counts(int nx, int ny, int nz, int64_t* nPoints, int64_t* nCells,
                    int64_t* nInternalFaces, int64_t* nBoundaryFaces) {
    if (nx < 1 || ny < 1 || nz < 1) return -1;
    const int64_t X = nx, Y = ny, Z = nz;
    if (nPoints) *nPoints = (X + 1) * (Y + 1) * (Z + 1);
    if (nCells) *nCells = X * Y * Z;
    if (nInternalFaces) *nInternalFaces = (X - 1) * Y * Z + X * (Y - 1) * Z + X * Y * (Z - 1);
    if (nBoundaryFaces) *nBoundaryFaces = 2 * (Y * Z + X * Z + X * Y);
    return 0;
}

int cfxc_box_points(int nx, int ny, int nz, double Lx, double Ly, double Lz,
                    double jitter, uint64_t seed, double* points) {
    if (nx < 1 || ny < 1 || nz < 1 || !points) return -1;
    std::mt19937_64 g(seed);
    const double hx = Lx / nx, hy = Ly / ny, hz = Lz / nz;
    int64_t p = 0;
    for (int k = 0; k <= nz; ++k)
        for (int j = 0; j <= ny; ++j)
            for (int i = 0; i <= nx; ++i, ++p) {
                const double rx = 2.0 * u01(g) - 1.0;
                const double ry = 2.0 * u01(g) - 1.0;
                const double rz = 2.0 * u01(g) - 1.0;
                double x = i * hx, y = j * hy, z = k * hz;
                if (jitter != 0.0) {
                    if (i > 0 && i < nx) x += rx * jitter * hx;
                    if (j > 0 && j < ny) y += ry * jitter * hy;
                    if (k > 0 && k < nz) z += rz * jitter * hz;
                }
                points[3 * p] = x;
                points[3 * p + 1] = y;
                points[3 * p + 2] = z;
            }
    return 0;
}

int cfxc_box_faces(int nx, int ny, int nz, int32_t* faces, int32_t* owner,
                   int32_t* neighbour, int32_t* patchStart) {
    if (nx < 1 || ny < 1 || nz < 1 || !faces || !owner) return -1;
    const int64_t PX = nx + 1, PY = ny + 1;
    auto P = [&](int64_t i, int64_t j, int64_t k) { return int32_t(i + PX * (j + PY * k)); };
    auto C = [&](int64_t i, int64_t j, int64_t k) { return int32_t(i + int64_t(nx) * (j + int64_t(ny) * k)); };
    int64_t f = 0;
    auto put = [&](int32_t a, int32_t b, int32_t c, int32_t d, int32_t o) {
        faces[4 * f] = a;
        faces[4 * f + 1] = b;
        faces[4 * f + 2] = c;
        faces[4 * f + 3] = d;
        owner[f] = o;
        ++f;
    };
    // Internal faces: per owner cell, its +x, +y, +z neighbours (ascending).
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const int32_t c = C(i, j, k);
                if (i + 1 < nx) {
                    if (neighbour) neighbour[f] = C(i + 1, j, k);
                    put(P(i + 1, j, k), P(i + 1, j + 1, k), P(i + 1, j + 1, k + 1), P(i + 1, j, k + 1), c);
                }
                if (j + 1 < ny) {
                    if (neighbour) neighbour[f] = C(i, j + 1, k);
                    put(P(i, j + 1, k), P(i, j + 1, k + 1), P(i + 1, j + 1, k + 1), P(i + 1, j + 1, k), c);
                }
                if (k + 1 < nz) {
                    if (neighbour) neighbour[f] = C(i, j, k + 1);
                    put(P(i, j, k + 1), P(i + 1, j, k + 1), P(i + 1, j + 1, k + 1), P(i, j + 1, k + 1), c);
                }
            }
    int p = 0;
    // xmin / xmax
    if (patchStart) patchStart[p] = int32_t(f);
    ++p;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            put(P(0, j, k), P(0, j, k + 1), P(0, j + 1, k + 1), P(0, j + 1, k), C(0, j, k));
    if (patchStart) patchStart[p] = int32_t(f);
    ++p;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            put(P(nx, j, k), P(nx, j + 1, k), P(nx, j + 1, k + 1), P(nx, j, k + 1), C(nx - 1, j, k));
    // ymin / ymax
    if (patchStart) patchStart[p] = int32_t(f);
    ++p;
    for (int k = 0; k < nz; ++k)
        for (int i = 0; i < nx; ++i)
            put(P(i, 0, k), P(i + 1, 0, k), P(i + 1, 0, k + 1), P(i, 0, k + 1), C(i, 0, k));
    if (patchStart) patchStart[p] = int32_t(f);
    ++p;
    for (int k = 0; k < nz; ++k)
        for (int i = 0; i < nx; ++i)
            put(P(i, ny, k), P(i, ny, k + 1), P(i + 1, ny, k + 1), P(i + 1, ny, k), C(i, ny - 1, k));
    // zmin / zmax
    if (patchStart) patchStart[p] = int32_t(f);
    ++p;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i)
            put(P(i, j, 0), P(i, j + 1, 0), P(i + 1, j + 1, 0), P(i + 1, j, 0), C(i, j, 0));
    if (patchStart) patchStart[p] = int32_t(f);
    ++p;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i)
            put(P(i, j, nz), P(i + 1, j, nz), P(i + 1, j + 1, nz), P(i, j + 1, nz), C(i, j, nz - 1));
    if (patchStart) patchStart[6] = int32_t(f);
    return 0;
}

// face::areaAndCentre for a polygon of n points, restated from
// src/OpenFOAM/meshes/meshShapes/face/faceTemplates.C:79-149 with the same
// operation order; n == 3 uses the direct triangle formula.
static void area_and_centre(const V3* ps, int n, V3& area, V3& centre) {
    if (n == 3) {
        area = (1.0 / 2.0) * cross(ps[1] - ps[0], ps[2] - ps[0]);
        centre = (1.0 / 3.0) * (ps[0] + ps[1] + ps[2]);
        return;
    }
    V3 pAvg{0, 0, 0};
    for (int i = 0; i < n; ++i) pAvg = pAvg + ps[i];
    pAvg = pAvg / double(n);
    V3 sumA{0, 0, 0};
    for (int i = 0; i < n; ++i) {
        const V3 p = ps[i], pNext = ps[(i + 1) % n];
        sumA = sumA + cross(pNext - p, pAvg - p);
    }
    const double m = mag(sumA);
    const V3 sumAHat = m > 0 ? sumA / m : V3{0, 0, 0};
    double sumAn = 0;
    V3 sumAnc{0, 0, 0};
    for (int i = 0; i < n; ++i) {
        const V3 p = ps[i], pNext = ps[(i + 1) % n];
        const V3 a = cross(pNext - p, pAvg - p);
        const V3 c = p + pNext + pAvg;
        const double an = dot(a, sumAHat);
        sumAn += an;
        sumAnc = sumAnc + an * c;
    }
    area = (1.0 / 2.0) * sumA;
    centre = sumAn > vSmall ? ((1.0 / 3.0) * sumAnc) / sumAn : pAvg;
}

int cfxc_face_geometry(int64_t nFaces, const int32_t* faces,
                       const double* points, double* Sf, double* Cf,
                       double* magSf) {
    if (nFaces < 0 || !faces || !points) return -1;
    for (int64_t f = 0; f < nFaces; ++f) {
        V3 ps[4];
        for (int q = 0; q < 4; ++q) ps[q] = ld(points, faces[4 * f + q]);
        V3 a, c;
        area_and_centre(ps, 4, a, c);
        if (Sf) st(Sf, f, a);
        if (Cf) st(Cf, f, c);
        if (magSf) magSf[f] = std::max(mag(a), rootVSmall);
    }
    return 0;
}

// primitiveMesh::makeCellCentresAndVols,
// src/OpenFOAM/meshes/primitiveMesh/primitiveMeshCellCentresAndVols.C:72-150
int cfxc_cell_geometry(int64_t nCells, int64_t nFaces, int64_t nInternalFaces,
                       const int32_t* owner, const int32_t* neighbour,
                       const double* Sf, const double* Cf, double* C,
                       double* V) {
    if (nCells < 0 || !owner || !Sf || !Cf || !C) return -1;
    std::vector<V3> cEst(nCells, V3{0, 0, 0}), ctr(nCells, V3{0, 0, 0});
    std::vector<int32_t> nCF(nCells, 0);
    std::vector<double> vol(nCells, 0.0);
    for (int64_t f = 0; f < nFaces; ++f) {
        cEst[owner[f]] = cEst[owner[f]] + ld(Cf, f);
        nCF[owner[f]] += 1;
    }
    for (int64_t f = 0; f < nInternalFaces; ++f) {
        cEst[neighbour[f]] = cEst[neighbour[f]] + ld(Cf, f);
        nCF[neighbour[f]] += 1;
    }
    for (int64_t c = 0; c < nCells; ++c) cEst[c] = cEst[c] / double(nCF[c]);
    for (int64_t f = 0; f < nFaces; ++f) {
        const int32_t o = owner[f];
        const double pyr3Vol = dot(ld(Sf, f), ld(Cf, f) - cEst[o]);
        const V3 pc = (3.0 / 4.0) * ld(Cf, f) + (1.0 / 4.0) * cEst[o];
        ctr[o] = ctr[o] + pyr3Vol * pc;
        vol[o] += pyr3Vol;
    }
    for (int64_t f = 0; f < nInternalFaces; ++f) {
        const int32_t n = neighbour[f];
        const double pyr3Vol = dot(ld(Sf, f), cEst[n] - ld(Cf, f));
        const V3 pc = (3.0 / 4.0) * ld(Cf, f) + (1.0 / 4.0) * cEst[n];
        ctr[n] = ctr[n] + pyr3Vol * pc;
        vol[n] += pyr3Vol;
    }
    for (int64_t c = 0; c < nCells; ++c) {
        const V3 cc = std::fabs(vol[c]) > vSmall ? ctr[c] / vol[c] : cEst[c];
        st(C, c, cc);
        if (V) V[c] = vol[c] * (1.0 / 3.0);
    }
    return 0;
}

int cfxc_laplacian(int64_t nCells, int64_t nFaces, int64_t nInternalFaces,
                   const int32_t* owner, const int32_t* neighbour,
                   const int32_t* patchStart, const double* magSf,
                   const double* Cf, const double* C, double gamma,
                   int dirichletMask, double* diag, double* upper) {
    if (nCells < 0 || !owner || !neighbour || !magSf || !C || !diag || !upper) return -1;
    for (int64_t f = 0; f < nInternalFaces; ++f) {
        const double d = mag(ld(C, neighbour[f]) - ld(C, owner[f]));
        upper[f] = -(gamma * magSf[f] / d);
    }
    // lduMatrix::negSumDiag (src/OpenFOAM/matrices/lduMatrix/lduMatrix/lduMatrixOperations.C:55-74)
    std::fill(diag, diag + nCells, 0.0);
    for (int64_t f = 0; f < nInternalFaces; ++f) {
        diag[owner[f]] -= upper[f];
        diag[neighbour[f]] -= upper[f];
    }
    if (patchStart && Cf) {
        for (int p = 0; p < 6; ++p) {
            if (!(dirichletMask & (1 << p))) continue;
            for (int64_t f = patchStart[p]; f < patchStart[p + 1]; ++f) {
                const double d = mag(ld(Cf, f) - ld(C, owner[f]));
                diag[owner[f]] += gamma * magSf[f] / d;
            }
        }
    }
    (void)nFaces;
    return 0;
}

int cfxc_convection_diffusion(int64_t nCells, int64_t nFaces,
                              int64_t nInternalFaces, const int32_t* owner,
                              const int32_t* neighbour,
                              const int32_t* patchStart, const double* Sf,
                              const double* magSf, const double* Cf,
                              const double* C, const double* U, double gamma,
                              int dirichletMask, double* diag, double* upper,
                              double* lower) {
    if (nCells < 0 || !owner || !neighbour || !Sf || !magSf || !C || !U || !diag || !upper || !lower) return -1;
    const V3 Uv{U[0], U[1], U[2]};
    for (int64_t f = 0; f < nInternalFaces; ++f) {
        const double phi = dot(Uv, ld(Sf, f));
        const double w = phi >= 0 ? 1.0 : 0.0;
        const double g = gamma * magSf[f] / mag(ld(C, neighbour[f]) - ld(C, owner[f]));
        lower[f] = -w * phi - g;
        upper[f] = (1.0 - w) * phi - g;
    }
    std::fill(diag, diag + nCells, 0.0);
    for (int64_t f = 0; f < nInternalFaces; ++f) {
        diag[owner[f]] -= lower[f];
        diag[neighbour[f]] -= upper[f];
    }
    if (patchStart && Cf) {
        for (int p = 0; p < 6; ++p) {
            const bool dir = (dirichletMask & (1 << p)) != 0;
            for (int64_t f = patchStart[p]; f < patchStart[p + 1]; ++f) {
                if (dir) {
                    const double d = mag(ld(Cf, f) - ld(C, owner[f]));
                    diag[owner[f]] += gamma * magSf[f] / d;
                } else {
                    diag[owner[f]] += dot(Uv, ld(Sf, f));
                }
            }
        }
    }
    (void)nFaces;
    return 0;
}

int cfxc_uniform(uint64_t seed, int64_t n, double lo, double hi, double* out) {
    if (n < 0 || !out) return -1;
    std::mt19937_64 g(seed);
    for (int64_t i = 0; i < n; ++i) out[i] = lo + (hi - lo) * u01(g);
    return 0;
}

int cfxc_random_order(uint64_t seed, int64_t nCells, int32_t* newOrder) {
    if (nCells < 0 || !newOrder) return -1;
    std::mt19937_64 g(seed);
    for (int64_t i = 0; i < nCells; ++i) newOrder[i] = int32_t(i);
    for (int64_t i = nCells - 1; i > 0; --i) {
        const int64_t j = int64_t(g() % uint64_t(i + 1));
        std::swap(newOrder[i], newOrder[j]);
    }
    return 0;
}

// bandCompression(cellCells), src/OpenFOAM/meshes/bandCompression/bandCompression.C:42-146.
// cellCells lists each cell's neighbours in face order (primitiveMesh::calcCellCells).
// The reference sorts the unvisited neighbours by connectivity but then
// appends nbrs[i] (not nbrs[order[i]]), so neighbours enter the queue in
// cellCells order; that behaviour is kept.
int cfxc_cuthill_mckee(int64_t nCells, int64_t nFaces, const int32_t* l,
                       const int32_t* u, int32_t* newOrder) {
    if (nCells < 0 || !l || !u || !newOrder) return -1;
    std::vector<int64_t> off(nCells + 1, 0);
    for (int64_t f = 0; f < nFaces; ++f) {
        off[l[f] + 1]++;
        off[u[f] + 1]++;
    }
    for (int64_t c = 0; c < nCells; ++c) off[c + 1] += off[c];
    std::vector<int32_t> cc(off[nCells]);
    std::vector<int64_t> fill(off.begin(), off.end() - 1);
    for (int64_t f = 0; f < nFaces; ++f) {
        cc[fill[l[f]]++] = u[f];
        cc[fill[u[f]]++] = l[f];
    }
    std::vector<char> visited(nCells, 0);
    std::deque<int32_t> next;
    int64_t inOrder = 0;
    while (true) {
        int64_t current = -1;
        int64_t minWeight = INT64_MAX;
        for (int64_t c = 0; c < nCells; ++c) {
            if (!visited[c] && off[c + 1] - off[c] < minWeight) {
                minWeight = off[c + 1] - off[c];
                current = c;
            }
        }
        if (current == -1) break;
        next.push_back(int32_t(current));
        while (!next.empty()) {
            const int32_t c = next.front();
            next.pop_front();
            if (visited[c]) continue;
            visited[c] = 1;
            newOrder[inOrder++] = c;
            for (int64_t k = off[c]; k < off[c + 1]; ++k)
                if (!visited[cc[k]]) next.push_back(cc[k]);
        }
    }
    return 0;
}

int cfxc_renumber(int64_t nCells, int64_t nFaces, const int32_t* newOrder,
                  int32_t* l, int32_t* u, double* diag, double* upper,
                  double* lower, int32_t* faceOrder, int32_t* faceFlip) {
    if (nCells < 0 || !newOrder || !l || !u) return -1;
    std::vector<int32_t> oldToNew(nCells);
    for (int64_t k = 0; k < nCells; ++k) oldToNew[newOrder[k]] = int32_t(k);
    if (diag) {
        std::vector<double> d(diag, diag + nCells);
        for (int64_t k = 0; k < nCells; ++k) diag[k] = d[newOrder[k]];
    }
    std::vector<int32_t> nl(nFaces), nu(nFaces);
    std::vector<char> flip(nFaces, 0);
    for (int64_t f = 0; f < nFaces; ++f) {
        int32_t a = oldToNew[l[f]], b = oldToNew[u[f]];
        if (a > b) {
            std::swap(a, b);
            flip[f] = 1;
        }
        nl[f] = a;
        nu[f] = b;
    }
    std::vector<int32_t> ord(nFaces);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int32_t x, int32_t y) {
        return nl[x] != nl[y] ? nl[x] < nl[y] : nu[x] < nu[y];
    });
    std::vector<double> up, lo;
    if (upper) up.assign(upper, upper + nFaces);
    if (lower) lo.assign(lower, lower + nFaces);
    for (int64_t k = 0; k < nFaces; ++k) {
        const int32_t f = ord[k];
        l[k] = nl[f];
        u[k] = nu[f];
        if (upper && lower) {
            upper[k] = flip[f] ? lo[f] : up[f];
            lower[k] = flip[f] ? up[f] : lo[f];
        } else if (upper) {
            upper[k] = up[f];
        }
        if (faceOrder) faceOrder[k] = f;
        if (faceFlip) faceFlip[k] = flip[f];
    }
    return 0;
}

}  // extern "C"
