"""Seeded synthetic LDU systems (ctypes front end of ``lib/libcfxcase.so``).

Each system is a dict of numpy arrays in OpenFOAM's LDU layout:
``l``/``u`` (int32 lowerAddr/upperAddr, upper-triangular face order),
``diag``, ``upper``, ``lower`` (float64; ``lower`` is None when symmetric),
``source`` and, for geometric agglomeration, ``Sf`` (internal face-area
vectors, [nFaces, 3]).

The workloads match the solver benchmarks:

* ``pcg_cube``        uniform n^3 unit cube, -laplacian(1,T), Dirichlet T=0
                      on x=0, zero-gradient elsewhere, source U[-1,1]
* ``gamg_cube``       the same on a cube with interior vertices jittered by
                      U[-j*h, j*h] per axis (non-orthogonal, no corrections)
* ``bicgstab_cube``   jittered cube, upwind div(phi,T) - laplacian(1e-3,T)
                      with |U| = 1 in a seeded random direction, cells
                      randomly permuted then renumbered by Cuthill-McKee
* ``box``             an nx*ny*nz box of given aspect, Dirichlet on one face
"""
import ctypes
import math
import os

import numpy as np

from . import LIB_DIR

_lib = None

PATCHES = ("xmin", "xmax", "ymin", "ymax", "zmin", "zmax")

i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(LIB_DIR, "libcfxcase.so")
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: run __graft_entry__.build()")
        L = ctypes.CDLL(path)
        i64 = ctypes.c_int64
        i64p = ctypes.POINTER(ctypes.c_int64)
        L.cfxc_box_counts.argtypes = [ctypes.c_int] * 3 + [i64p] * 4
        L.cfxc_box_points.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 4 + [ctypes.c_uint64, f64p]
        L.cfxc_box_faces.argtypes = [ctypes.c_int] * 3 + [i32p] * 4
        L.cfxc_face_geometry.argtypes = [i64, i32p, f64p, f64p, f64p, f64p]
        L.cfxc_cell_geometry.argtypes = [i64, i64, i64, i32p, i32p, f64p, f64p, f64p, f64p]
        L.cfxc_laplacian.argtypes = [i64, i64, i64, i32p, i32p, i32p, f64p, f64p, f64p,
                                     ctypes.c_double, ctypes.c_int, f64p, f64p]
        L.cfxc_convection_diffusion.argtypes = [i64, i64, i64, i32p, i32p, i32p, f64p, f64p, f64p,
                                                f64p, f64p, ctypes.c_double, ctypes.c_int,
                                                f64p, f64p, f64p]
        L.cfxc_uniform.argtypes = [ctypes.c_uint64, i64, ctypes.c_double, ctypes.c_double, f64p]
        L.cfxc_random_order.argtypes = [ctypes.c_uint64, i64, i32p]
        L.cfxc_cuthill_mckee.argtypes = [i64, i64, i32p, i32p, i32p]
        L.cfxc_renumber.argtypes = [i64, i64, i32p, i32p, i32p, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p]
        _lib = L
    return _lib


def _chk(rc, what):
    if rc != 0:
        raise ValueError(f"{what} failed ({rc})")


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def box_mesh(nx, ny, nz, L=(1.0, 1.0, 1.0), jitter=0.0, seed=0, periodic_x=False):
    """Hex box mesh with OpenFOAM face geometry (points, faces, owner, ...).
    periodic_x: the xmax plane's points take the y, z of the xmin plane's, so
    the two patches are translations of each other (a cyclic pair)."""
    L_ = lib()
    c = [ctypes.c_int64() for _ in range(4)]
    _chk(L_.cfxc_box_counts(nx, ny, nz, *[ctypes.byref(x) for x in c]), "box_counts")
    nP, nC, nI, nB = (x.value for x in c)
    nF = nI + nB
    pts = np.empty(3 * nP)
    _chk(L_.cfxc_box_points(nx, ny, nz, L[0], L[1], L[2], jitter, seed, pts), "box_points")
    if periodic_x:
        P = pts.reshape(nz + 1, ny + 1, nx + 1, 3)
        P[:, :, nx, 1:] = P[:, :, 0, 1:]
    faces = np.empty(4 * nF, np.int32)
    owner = np.empty(nF, np.int32)
    nei = np.empty(max(nI, 1), np.int32)
    ps = np.empty(7, np.int32)
    _chk(L_.cfxc_box_faces(nx, ny, nz, faces, owner, nei, ps), "box_faces")
    nei = nei[:nI]
    Sf = np.empty(3 * nF)
    Cf = np.empty(3 * nF)
    magSf = np.empty(nF)
    _chk(L_.cfxc_face_geometry(nF, faces, pts, Sf, Cf, magSf), "face_geometry")
    C = np.empty(3 * nC)
    V = np.empty(nC)
    _chk(L_.cfxc_cell_geometry(nC, nF, nI, owner, np.ascontiguousarray(nei) if nI else np.zeros(1, np.int32),
                               Sf, Cf, C, V), "cell_geometry")
    return dict(nx=nx, ny=ny, nz=nz, nCells=nC, nInternalFaces=nI, nFaces=nF,
                points=pts, faces=faces, owner=owner, neighbour=nei, patchStart=ps,
                Sf=Sf, Cf=Cf, magSf=magSf, C=C, V=V)


def fv_geometry(mesh, snGrad="uncorrected"):
    """The face geometry an fvMesh hands to device-side assembly, by the
    reference's surfaceInterpolation (surfaceInterpolation.C:160-330) and
    fvPatch::delta (fvPatch.C:159-164): internal magSf; the snGrad scheme's
    deltaCoeffs -- nonOrthDeltaCoeffs 1/max(n . d, 0.05 |d|) for corrected
    and uncorrected (surfaceInterpolation.C:302-318), the plain
    deltaCoeffs 1/|d| for orthogonal -- with d = C_N - C_P; weights
    SfdNei/(SfdOwn + SfdNei); boundary faces (patch order) with their cell,
    magSf and 1/|n (n . (Cf - C_P))| (fvPatch::deltaCoeffs, which the
    boundary gradient coefficients use); cell volumes."""
    nI, nF = mesh["nInternalFaces"], mesh["nFaces"]
    own, nei = mesh["owner"], mesh["neighbour"]
    Sf = mesh["Sf"].reshape(nF, 3)
    Cf = mesh["Cf"].reshape(nF, 3)
    C = mesh["C"].reshape(-1, 3)
    mag = lambda v: np.sqrt(v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1] + v[:, 2] * v[:, 2])
    dot = lambda a, b: a[:, 0] * b[:, 0] + a[:, 1] * b[:, 1] + a[:, 2] * b[:, 2]
    d = C[nei] - C[own[:nI]]
    if snGrad == "orthogonal":
        dc = 1.0 / mag(d)
    elif snGrad in ("corrected", "uncorrected"):
        unitArea = Sf[:nI] / mesh["magSf"][:nI, None]
        a, b = dot(unitArea, d), 0.05 * mag(d)
        dc = 1.0 / np.where(a > b, a, b)
    else:
        raise ValueError("snGrad scheme " + snGrad)
    sOwn = np.abs(dot(Sf[:nI], Cf[:nI] - C[own[:nI]]))
    sNei = np.abs(dot(Sf[:nI], C[nei] - Cf[:nI]))
    bo = own[nI:]
    nHat = Sf[nI:] / mesh["magSf"][nI:, None]
    delta = nHat * dot(nHat, Cf[nI:] - C[bo])[:, None]
    return dict(magSf=mesh["magSf"][:nI].copy(), deltaCoeffs=dc, weights=sNei / (sOwn + sNei),
                V=mesh["V"].copy(), bCell=bo.astype(np.int32), magSfB=mesh["magSf"][nI:].copy(),
                deltaCoeffsB=1.0 / mag(delta))


def cyclic_x(s, mesh, gamma=1.0, U=None):
    """Couples a box system's xmin and xmax patches as a cyclic pair (face k
    of one with face k of the other): two coupled interfaces, the cells and
    neighbour cells of their faces, interfaceBouCoeffs (result -= bou*psi_nbr,
    so the coupling coefficient is -bou) and interfaceIntCoeffs (the
    transpose's, for Tmul).  The coupling is diffusion gamma*magSf/d across
    the periodic face and, with U, the upwind flux U.Sf; the diagonals take
    the matching internal coefficients.  The system must have been built
    with xmin and xmax as non-Dirichlet patches (their boundary terms are
    replaced)."""
    ps = mesh["patchStart"]
    own = mesh["owner"]
    nF = mesh["nFaces"]
    Sf = mesh["Sf"].reshape(nF, 3)
    Cf = mesh["Cf"].reshape(nF, 3)
    C = mesh["C"].reshape(-1, 3)
    fa, fb = np.arange(ps[0], ps[1]), np.arange(ps[1], ps[2])
    a, b = own[fa], own[fb]
    dist = lambda v: np.sqrt(v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1] + v[:, 2] * v[:, 2])  # noqa: E731
    d = dist(Cf[fa] - C[a]) + dist(Cf[fb] - C[b])
    g = gamma * 0.5 * (mesh["magSf"][fa] + mesh["magSf"][fb]) / d
    diag = s["diag"].copy()
    if U is None:
        bouA, bouB = g, g.copy()
        diag[a] += g
        diag[b] += g
    else:
        Uv = np.asarray(U, np.float64)
        F = Sf[fb] @ Uv  # flux out through xmax = into the cell on xmin
        # the generator's zeroGradient outflow terms on both patches are replaced
        diag[a] -= Sf[fa] @ Uv
        diag[b] -= F
        Fp, Fm = np.maximum(F, 0.0), np.maximum(-F, 0.0)
        diag[a] += g + Fm
        diag[b] += g + Fp
        bouA, bouB = g + Fp, g + Fm
    n = len(fa)
    out = dict(s)
    out.update(diag=diag, ifSize=np.array([n, n], np.int32), ifCell=np.concatenate([a, b]).astype(np.int32),
               ifNbr=np.concatenate([b, a]).astype(np.int32), ifBou=np.concatenate([bouA, bouB]),
               ifInt=np.concatenate([bouB, bouA]), ifNbrPatch=np.array([1, 0], np.int32))
    return out


def cyclic_cube(n, jitter=0.2, seed=1, U=None, gamma=1.0):
    """An n^3 box, periodic in x (a cyclic pair), Dirichlet on ymin: the
    Laplacian, or with U the upwind convection-diffusion operator."""
    m = box_mesh(n, n, n, jitter=jitter, seed=seed)
    if U is None:
        s = laplacian(m, gamma=gamma, dirichlet=("ymin",))
    else:
        s = convection_diffusion(m, U, gamma, dirichlet=("ymin",))
    s = cyclic_x(s, m, gamma=gamma, U=U)
    s["source"] = uniform(seed + 7, s["diag"].size)
    s["name"] = f"cyclic-{n}"
    return s


def _mask(dirichlet):
    m = 0
    for p in dirichlet:
        m |= 1 << PATCHES.index(p)
    return m


def laplacian(mesh, gamma=1.0, dirichlet=("xmin",)):
    """Symmetric -laplacian(gamma,T): returns l, u, diag, upper (lower None)."""
    L_ = lib()
    nC, nI, nF = mesh["nCells"], mesh["nInternalFaces"], mesh["nFaces"]
    diag = np.empty(nC)
    upper = np.empty(max(nI, 1))
    nei = mesh["neighbour"] if nI else np.zeros(1, np.int32)
    _chk(L_.cfxc_laplacian(nC, nF, nI, mesh["owner"], np.ascontiguousarray(nei), mesh["patchStart"],
                           mesh["magSf"], mesh["Cf"], mesh["C"], gamma, _mask(dirichlet),
                           diag, upper), "laplacian")
    return dict(l=mesh["owner"][:nI].copy(), u=mesh["neighbour"].copy(), diag=diag,
                upper=upper[:nI].copy(), lower=None,
                Sf=mesh["Sf"][: 3 * nI].reshape(nI, 3).copy())


def convection_diffusion(mesh, U, gamma, dirichlet=("xmin",)):
    """Asymmetric upwind div(phi,T) - laplacian(gamma,T)."""
    L_ = lib()
    nC, nI, nF = mesh["nCells"], mesh["nInternalFaces"], mesh["nFaces"]
    diag = np.empty(nC)
    upper = np.empty(nI)
    lower = np.empty(nI)
    Uv = np.asarray(U, dtype=np.float64)
    _chk(L_.cfxc_convection_diffusion(nC, nF, nI, mesh["owner"], mesh["neighbour"], mesh["patchStart"],
                                      mesh["Sf"], mesh["magSf"], mesh["Cf"], mesh["C"], Uv, gamma,
                                      _mask(dirichlet), diag, upper, lower), "convection_diffusion")
    return dict(l=mesh["owner"][:nI].copy(), u=mesh["neighbour"].copy(), diag=diag,
                upper=upper, lower=lower, Sf=mesh["Sf"][: 3 * nI].reshape(nI, 3).copy())


def uniform(seed, n, lo=-1.0, hi=1.0):
    out = np.empty(n)
    _chk(lib().cfxc_uniform(seed, n, lo, hi, out), "uniform")
    return out


def random_order(seed, n):
    out = np.empty(n, np.int32)
    _chk(lib().cfxc_random_order(seed, n, out), "random_order")
    return out


def cuthill_mckee(sys_):
    n = sys_["diag"].size
    out = np.empty(n, np.int32)
    _chk(lib().cfxc_cuthill_mckee(n, sys_["l"].size, sys_["l"], sys_["u"], out), "cuthill_mckee")
    return out


def renumber(sys_, new_order):
    """Renumber a system in place (cells by new_order, faces re-sorted)."""
    n, nf = sys_["diag"].size, sys_["l"].size
    fo = np.empty(nf, np.int32)
    ff = np.empty(nf, np.int32)
    _chk(lib().cfxc_renumber(n, nf, np.ascontiguousarray(new_order, np.int32), sys_["l"], sys_["u"],
                             _ptr(sys_["diag"]), _ptr(sys_["upper"]), _ptr(sys_.get("lower")),
                             _ptr(fo), _ptr(ff)), "renumber")
    if sys_.get("Sf") is not None:
        Sf = sys_["Sf"][fo]
        Sf[ff == 1] *= -1.0
        sys_["Sf"] = np.ascontiguousarray(Sf)
    if sys_.get("source") is not None:
        sys_["source"] = sys_["source"][new_order].copy()
    return sys_


def pcg_cube(n=64, seed=1):
    """C1: uniform n^3 unit cube Laplacian, Dirichlet x=0, source U[-1,1]."""
    s = laplacian(box_mesh(n, n, n, jitter=0.0, seed=seed))
    s["source"] = uniform(seed, s["diag"].size)
    s["name"] = f"laplacian-cube-{n}"
    return s


def gamg_cube(n=256, jitter=0.2, seed=1):
    """C2: jittered n^3 cube Laplacian, Dirichlet x=0, source U[-1,1]."""
    s = laplacian(box_mesh(n, n, n, jitter=jitter, seed=seed))
    s["source"] = uniform(seed + 1000, s["diag"].size)
    s["name"] = f"laplacian-jittered-cube-{n}"
    return s


def bicgstab_cube(n=128, jitter=0.2, seed=1, gamma=1e-3):
    """C3: jittered cube, upwind convection-diffusion, random + CM order.

    |U| = 1 in a seeded direction with U_x > 0 (x=0 is the Dirichlet inflow)."""
    rng = np.random.default_rng(seed)
    d = rng.normal(size=3)
    U = d / np.linalg.norm(d)
    # Orient the seeded direction so that the Dirichlet face x=0 is an inflow
    # boundary: with the only fixed value on an outflow face the global
    # Peclet number |U|L/gamma = 1000 makes the system singular to rounding.
    if U[0] < 0:
        U = -U
    s = convection_diffusion(box_mesh(n, n, n, jitter=jitter, seed=seed), U, gamma)
    renumber(s, random_order(seed + 7, s["diag"].size))
    renumber(s, cuthill_mckee(s))
    s["source"] = uniform(seed + 2000, s["diag"].size)
    s["name"] = f"upwind-convection-diffusion-cube-{n}"
    s["U"] = U
    return s


def box(nx, ny, nz, dirichlet="xmin", seed=1):
    """C4 member: box of nx*ny*nz cells (cell size 1/max(n)), one Dirichlet face."""
    h = 1.0 / max(nx, ny, nz)
    s = laplacian(box_mesh(nx, ny, nz, L=(nx * h, ny * h, nz * h), seed=seed), dirichlet=(dirichlet,))
    s["source"] = uniform(seed, s["diag"].size)
    s["name"] = f"laplacian-box-{nx}x{ny}x{nz}"
    return s


def batch_boxes(count=512, lo=4096, hi=500000, seed=1):
    """C4: box shapes with cell counts log-uniform in [lo, hi], aspect U[1,4]."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        N = math.exp(rng.uniform(math.log(lo), math.log(hi)))
        a = rng.uniform(1.0, 4.0, size=3)
        scale = (N / np.prod(a)) ** (1.0 / 3.0)
        dims = [max(2, int(round(x * scale))) for x in a]
        face = PATCHES[int(rng.integers(0, 6))]
        out.append((dims[0], dims[1], dims[2], face, int(seed * 100003 + k)))
    return out
