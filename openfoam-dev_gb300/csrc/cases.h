/*
 * cases.h - seeded synthetic LDU systems for tests and benchmarks (host only).
 *
 * These routines build the meshes and matrices that the solver library is
 * exercised on: uniform or jittered hexahedral boxes, their face and cell
 * geometry, the -laplacian and upwind convection-diffusion LDU coefficients,
 * random permutation and Cuthill-McKee renumbering.  They are not part of the
 * solver path; an OpenFOAM case gets the same arrays from fvMatrix.
 *
 * Geometry follows the reference's own formulas so that face-area weights for
 * the faceAreaPair agglomeration are bit-identical with an OpenFOAM mesh of
 * the same points:
 *   face::areaAndCentre               src/OpenFOAM/meshes/meshShapes/face/faceTemplates.C:79-149
 *   primitiveMesh::makeFaceCentresAndAreas
 *                                     src/OpenFOAM/meshes/primitiveMesh/primitiveMeshFaceCentresAndAreas.C:75-95
 *   primitiveMesh::makeCellCentresAndVols
 *                                     src/OpenFOAM/meshes/primitiveMesh/primitiveMeshCellCentresAndVols.C:72-150
 *   bandCompression (Cuthill-McKee)   src/OpenFOAM/meshes/bandCompression/bandCompression.C:42-146
 *
 * All integer arrays are int32 (OpenFOAM label, WM_LABEL_SIZE=32); all
 * coordinates and coefficients are double.  Every function returns 0 on
 * success and a negative value on a bad argument.
 */
#ifndef CFX_CASES_H
#define CFX_CASES_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Patch order used by every box routine. */
enum { CFXC_XMIN = 0, CFXC_XMAX, CFXC_YMIN, CFXC_YMAX, CFXC_ZMIN, CFXC_ZMAX };

/* Sizes of an nx*ny*nz hex box (7-point connectivity). */
int cfxc_box_counts(int nx, int ny, int nz, int64_t* nPoints, int64_t* nCells,
                    int64_t* nInternalFaces, int64_t* nBoundaryFaces);

/* Vertex coordinates [nPoints*3] of a box of size Lx*Ly*Lz.  Interior vertices
 * move by U[-jitter*h, +jitter*h] per axis; boundary vertices move only along
 * the boundary so the box stays a box.  Point (i,j,k) has index
 * i + (nx+1)*(j + (ny+1)*k). */
int cfxc_box_points(int nx, int ny, int nz, double Lx, double Ly, double Lz,
                    double jitter, uint64_t seed, double* points);

/* Quad faces [nFaces*4] (internal faces first, in upper-triangular order,
 * then boundary patches xmin,xmax,ymin,ymax,zmin,zmax), owner[nFaces],
 * neighbour[nInternalFaces] and patchStart[7] (face index of each patch start,
 * patchStart[6] = nFaces).  Cell (i,j,k) has index i + nx*(j + ny*k). */
int cfxc_box_faces(int nx, int ny, int nz, int32_t* faces, int32_t* owner,
                   int32_t* neighbour, int32_t* patchStart);

/* Face area vectors Sf[nFaces*3], centres Cf[nFaces*3] and magnitudes
 * magSf[nFaces] (max(|Sf|, rootVSmall)) of quad faces. */
int cfxc_face_geometry(int64_t nFaces, const int32_t* faces,
                       const double* points, double* Sf, double* Cf,
                       double* magSf);

/* Cell centres C[nCells*3] and volumes V[nCells]. */
int cfxc_cell_geometry(int64_t nCells, int64_t nFaces, int64_t nInternalFaces,
                       const int32_t* owner, const int32_t* neighbour,
                       const double* Sf, const double* Cf, double* C,
                       double* V);

/* -laplacian(gamma, T) on the internal faces: upper[f] = -gamma*magSf/|d|,
 * d = C[nei]-C[own]; diag = negSumDiag; then for every face of the patches
 * flagged in dirichletMask (bit p = patch p) diag[owner] += gamma*magSf/|Cf-C|
 * (fixedValue T=0, so the source is unchanged). */
int cfxc_laplacian(int64_t nCells, int64_t nFaces, int64_t nInternalFaces,
                   const int32_t* owner, const int32_t* neighbour,
                   const int32_t* patchStart, const double* magSf,
                   const double* Cf, const double* C, double gamma,
                   int dirichletMask, double* diag, double* upper);

/* Upwind div(phi,T) - laplacian(gamma,T) with phi = U.Sf:
 * lower = -w*phi - g, upper = (1-w)*phi - g (w = phi>=0, g = gamma*magSf/|d|),
 * diag = negSumDiag(lower, upper); boundary faces add phi_b (zero-gradient
 * patches) or gamma*magSf/|Cf-C| (Dirichlet patches in dirichletMask). */
int cfxc_convection_diffusion(int64_t nCells, int64_t nFaces,
                              int64_t nInternalFaces, const int32_t* owner,
                              const int32_t* neighbour,
                              const int32_t* patchStart, const double* Sf,
                              const double* magSf, const double* Cf,
                              const double* C, const double* U, double gamma,
                              int dirichletMask, double* diag, double* upper,
                              double* lower);

/* n values uniform in [lo, hi) from mt19937_64(seed) (53-bit mantissa). */
int cfxc_uniform(uint64_t seed, int64_t n, double lo, double hi, double* out);

/* Random permutation newOrder[nCells] (Fisher-Yates, mt19937_64(seed)):
 * newOrder[k] = old cell placed at position k. */
int cfxc_random_order(uint64_t seed, int64_t nCells, int32_t* newOrder);

/* Cuthill-McKee order of an LDU graph, following bandCompression:
 * newOrder[k] = old cell placed at position k. */
int cfxc_cuthill_mckee(int64_t nCells, int64_t nFaces, const int32_t* l,
                       const int32_t* u, int32_t* newOrder);

/* Renumber an LDU system in place with newOrder (new -> old): cells are
 * reordered, each face gets owner = min(new l, new u) (upper and lower swap
 * when the orientation flips) and faces are re-sorted to upper-triangular
 * order (by owner, then neighbour).  lower may be NULL (symmetric).
 * faceOrder (optional, [nFaces]) receives old face index of each new face
 * and faceFlip (optional) 1 where the orientation flipped. */
int cfxc_renumber(int64_t nCells, int64_t nFaces, const int32_t* newOrder,
                  int32_t* l, int32_t* u, double* diag, double* upper,
                  double* lower, int32_t* faceOrder, int32_t* faceFlip);

#ifdef __cplusplus
}
#endif

#endif
