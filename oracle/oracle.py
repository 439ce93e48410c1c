"""ctypes front end of the C oracle (``oracle/_build/libldu_oracle.so``).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA solver library.  Used by
tests/, ``__graft_entry__.smoke()`` and bench.py's CPU baseline; never by the
product.  Systems are dicts in the layout of ``cases.py`` (l, u, diag, upper,
lower or None, source, Sf).
"""
import ctypes
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libldu_oracle.so")
# the same source built with the reference's optimisation flags (bit-identical
# results; loaded instead of LIB when CFX_ORACLE_TIMED=1, by the timed CPU legs)
LIB_TIMED = os.path.join(HERE, "_build", "libldu_oracle_timed.so")

# FDIC (preconditioner and smoother) is DIC's arithmetic and
# nonBlockingGaussSeidel without coupled interfaces is GaussSeidel's: the
# reference's own FDIC / nonBlockingGaussSeidel golden solves pin the aliases
PRECONDITIONERS = {"none": 0, "diagonal": 1, "DIC": 2, "DILU": 3, "FDIC": 2}
SMOOTHERS = {"GaussSeidel": 0, "DIC": 1, "symGaussSeidel": 2, "DILU": 3, "DICGaussSeidel": 4,
             "DILUGaussSeidel": 5, "FDIC": 1,
             "nonBlockingGaussSeidel": 0}

i32p = ctypes.POINTER(ctypes.c_int)
f64p = ctypes.POINTER(ctypes.c_double)


class LduMatrix(ctypes.Structure):
    _fields_ = [("nCells", ctypes.c_int), ("nFaces", ctypes.c_int),
                ("l", i32p), ("u", i32p), ("diag", f64p), ("upper", f64p), ("lower", f64p),
                ("ownerStart", i32p), ("losort", i32p), ("losortStart", i32p),
                ("nIf", ctypes.c_int), ("ifCell", i32p), ("ifNbr", i32p), ("ifBou", f64p), ("ifInt", f64p),
                ("nIfPatch", ctypes.c_int), ("ifPatchSize", i32p), ("ifNbrPatch", i32p)]


class LduPerf(ctypes.Structure):
    _fields_ = [("initialResidual", ctypes.c_double), ("finalResidual", ctypes.c_double),
                ("nIterations", ctypes.c_int), ("converged", ctypes.c_int), ("singular", ctypes.c_int)]


class LduControls(ctypes.Structure):
    _fields_ = [("tolerance", ctypes.c_double), ("relTol", ctypes.c_double),
                ("maxIter", ctypes.c_int), ("minIter", ctypes.c_int)]


class LduAgglomeration(ctypes.Structure):
    _fields_ = [("nLevels", ctypes.c_int), ("nCells", ctypes.c_int * 50), ("nFaces", ctypes.c_int * 50),
                ("restrictAddr", i32p * 50), ("faceRestrict", i32p * 50), ("faceFlip", i32p * 50),
                ("cl", i32p * 50), ("cu", i32p * 50)]


class LduGamgControls(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int) for k in (
        "nPreSweeps", "preSweepsLevelMultiplier", "maxPreSweeps", "nPostSweeps",
        "postSweepsLevelMultiplier", "maxPostSweeps", "nFinestSweeps", "scaleCorrection", "smoother",
        "interpolateCorrection", "directSolveCoarsest")]


@dataclass
class Perf:
    initialResidual: float
    finalResidual: float
    nIterations: int
    converged: bool
    singular: bool


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = LIB_TIMED if os.environ.get("CFX_ORACLE_TIMED") == "1" else LIB
        if not os.path.exists(path):
            raise RuntimeError(f"{path} missing: run `make -C oracle`")
        _lib = ctypes.CDLL(path)
        for name in ("ldu_sum", "ldu_sum_mag", "ldu_sum_sqr", "ldu_average"):
            getattr(_lib, name).restype = ctypes.c_double
        _lib.ldu_sum_prod.restype = ctypes.c_double
        _lib.ldu_norm_factor.restype = ctypes.c_double
    return _lib


def _p(a, t=f64p):
    return None if a is None else a.ctypes.data_as(t)


def lu_solve(A, b):
    """LUscalarMatrix: LUDecompose then LUBacksubstitute of a dense matrix
    (scalarMatrices.C:77-180, scalarMatricesTemplates.C:117-163).  Raises
    ValueError("Singular matrix") for an all-zero row."""
    n = A.shape[0]
    lu = np.ascontiguousarray(A, np.float64).copy()
    piv = np.zeros(n, np.int32)
    if lib().ldu_lu_decompose(n, _p(lu), _p(piv, i32p)) != 0:
        raise ValueError("Singular matrix")
    x = np.ascontiguousarray(b, np.float64).copy()
    lib().ldu_lu_backsubstitute(n, _p(lu), _p(piv, i32p), _p(x))
    return x, lu, piv


class Matrix:
    """Holds a system's arrays and the C view (with derived addressing)."""

    def __init__(self, s):
        self.l = np.ascontiguousarray(s["l"], np.int32)
        self.u = np.ascontiguousarray(s["u"], np.int32)
        self.diag = np.ascontiguousarray(s["diag"], np.float64)
        self.upper = np.ascontiguousarray(s["upper"], np.float64)
        lo = s.get("lower")
        self.lower = None if lo is None else np.ascontiguousarray(lo, np.float64)
        self.c = LduMatrix(self.diag.size, self.l.size, _p(self.l, i32p), _p(self.u, i32p),
                           _p(self.diag), _p(self.upper), _p(self.lower), None, None, None)
        if s.get("ifCell") is not None:
            # coupled (cyclic) interfaces, faces concatenated in patch order
            self.ifc = [np.ascontiguousarray(s["ifCell"], np.int32), np.ascontiguousarray(s["ifNbr"], np.int32),
                        np.ascontiguousarray(s["ifBou"], np.float64),
                        np.ascontiguousarray(s.get("ifInt", s["ifBou"]), np.float64)]
            self.c.nIf = self.ifc[0].size
            self.c.ifCell, self.c.ifNbr = _p(self.ifc[0], i32p), _p(self.ifc[1], i32p)
            self.c.ifBou, self.c.ifInt = _p(self.ifc[2]), _p(self.ifc[3])
            if s.get("ifSize") is not None:
                self.ifc.append(np.ascontiguousarray(s["ifSize"], np.int32))
                self.c.nIfPatch, self.c.ifPatchSize = self.ifc[4].size, _p(self.ifc[4], i32p)
                if s.get("ifNbrPatch") is not None:
                    self.ifc.append(np.ascontiguousarray(s["ifNbrPatch"], np.int32))
                    self.c.ifNbrPatch = _p(self.ifc[5], i32p)
        lib().ldu_init_addr(ctypes.byref(self.c))
        self.n = self.diag.size

    def __del__(self):
        try:
            lib().ldu_free_addr(ctypes.byref(self.c))
        except Exception:
            pass

    def addr(self):
        n, nf = self.n, self.l.size
        return (np.ctypeslib.as_array(self.c.ownerStart, (n + 1,)).copy(),
                np.ctypeslib.as_array(self.c.losort, (max(nf, 1),))[:nf].copy(),
                np.ctypeslib.as_array(self.c.losortStart, (n + 1,)).copy())

    def _vec_op(self, fn, *vecs):
        out = np.empty(self.n)
        args = [np.ascontiguousarray(v, np.float64) for v in vecs]
        fn(ctypes.byref(self.c), *[_p(a) for a in args], _p(out))
        return out

    def amul(self, x):
        return self._vec_op(lib().ldu_amul, x)

    def tmul(self, x):
        return self._vec_op(lib().ldu_tmul, x)

    def residual(self, x, b):
        return self._vec_op(lib().ldu_residual, x, b)

    def sumA(self):
        out = np.empty(self.n)
        lib().ldu_sumA(ctypes.byref(self.c), _p(out))
        return out

    def norm_factor(self, psi, b):
        Apsi = self.amul(psi)
        tmp = np.empty(self.n)
        psi = np.ascontiguousarray(psi, np.float64)
        b = np.ascontiguousarray(b, np.float64)
        return lib().ldu_norm_factor(ctypes.byref(self.c), _p(psi), _p(b), _p(Apsi), _p(tmp))

    def dic_rD(self):
        out = np.empty(self.n)
        lib().ldu_dic_rD(ctypes.byref(self.c), _p(out))
        return out

    def dilu_rD(self):
        out = np.empty(self.n)
        lib().ldu_dilu_rD(ctypes.byref(self.c), _p(out))
        return out

    def dic_precondition(self, r):
        return self._vec_op(lib().ldu_dic_precondition, self.dic_rD(), r)

    def dilu_precondition(self, r):
        return self._vec_op(lib().ldu_dilu_precondition, self.dilu_rD(), r)

    def dilu_preconditionT(self, r):
        return self._vec_op(lib().ldu_dilu_preconditionT, self.dilu_rD(), r)

    def gs_smooth(self, psi, b, n_sweeps):
        psi = np.ascontiguousarray(psi, np.float64).copy()
        b = np.ascontiguousarray(b, np.float64)
        lib().ldu_gs_smooth(ctypes.byref(self.c), _p(psi), _p(b), n_sweeps)
        return psi

    def dic_smooth(self, psi, b, n_sweeps):
        psi = np.ascontiguousarray(psi, np.float64).copy()
        b = np.ascontiguousarray(b, np.float64)
        rD = self.dic_rD()
        lib().ldu_dic_smooth(ctypes.byref(self.c), _p(rD), _p(psi), _p(b), n_sweeps)
        return psi

    def smooth(self, smoother, psi, b, n_sweeps):
        """lduMatrix::smoother by name (GaussSeidel, symGaussSeidel, DIC, DILU,
        DICGaussSeidel, DILUGaussSeidel), n_sweeps sweeps."""
        psi = np.ascontiguousarray(psi, np.float64).copy()
        b = np.ascontiguousarray(b, np.float64)
        lib().ldu_smooth(ctypes.byref(self.c), SMOOTHERS[smoother], _p(psi), _p(b), int(n_sweeps))
        return psi


def _perf(p):
    return Perf(p.initialResidual, p.finalResidual, p.nIterations, bool(p.converged), bool(p.singular))


def _controls(tol, rel_tol, max_iter, min_iter):
    return LduControls(tol, rel_tol, max_iter, min_iter)


def pcg(s, psi, tol=1e-6, rel_tol=0.0, max_iter=1000, min_iter=0, precond="DIC"):
    """PCG::solve; psi (float64, contiguous) is updated in place."""
    m = Matrix(s)
    b = np.ascontiguousarray(s["source"], np.float64)
    perf = LduPerf()
    c = _controls(tol, rel_tol, max_iter, min_iter)
    lib().ldu_pcg(ctypes.byref(m.c), _p(psi), _p(b), ctypes.byref(c),
                  PRECONDITIONERS[precond], ctypes.byref(perf))
    return _perf(perf)


def smooth_solve(s, psi, smoother="GaussSeidel", n_sweeps=1, tol=1e-6, rel_tol=0.0, max_iter=1000, min_iter=0):
    """smoothSolver::solve (smoothSolver.C:77-196); psi is updated in place."""
    m = Matrix(s)
    b = np.ascontiguousarray(s["source"], np.float64)
    perf = LduPerf()
    c = _controls(tol, rel_tol, max_iter, min_iter)
    lib().ldu_smooth_solve(ctypes.byref(m.c), _p(psi), _p(b), ctypes.byref(c), SMOOTHERS[smoother],
                           int(n_sweeps), ctypes.byref(perf))
    return _perf(perf)


def pbicg(s, psi, tol=1e-6, rel_tol=0.0, max_iter=1000, min_iter=0, precond="DILU"):
    """PBiCG::solve (asymmetric matrices); psi is updated in place."""
    m = Matrix(s)
    b = np.ascontiguousarray(s["source"], np.float64)
    perf = LduPerf()
    c = _controls(tol, rel_tol, max_iter, min_iter)
    rc = lib().ldu_pbicg(ctypes.byref(m.c), _p(psi), _p(b), ctypes.byref(c), PRECONDITIONERS[precond],
                         ctypes.byref(perf))
    if rc == -2:
        raise ValueError("PBiCG has failed to converge within the maximum number of iterations")
    return _perf(perf)


def pbicgstab(s, psi, tol=1e-6, rel_tol=0.0, max_iter=1000, min_iter=0, precond="DILU"):
    """PBiCGStab::solve; psi is updated in place."""
    m = Matrix(s)
    b = np.ascontiguousarray(s["source"], np.float64)
    perf = LduPerf()
    c = _controls(tol, rel_tol, max_iter, min_iter)
    lib().ldu_pbicgstab(ctypes.byref(m.c), _p(psi), _p(b), ctypes.byref(c),
                        PRECONDITIONERS[precond], ctypes.byref(perf))
    return _perf(perf)


def gamg_coarse_interfaces(R, patchSize, faceCells, nbrCells, bou):
    """One GAMG level's coarse cyclic interfaces: (patch sizes, face cells,
    partner cells, summed coefficients, each fine face's coarse face)."""
    i = lambda a: np.ascontiguousarray(a, np.int32)  # noqa: E731
    R, ps, fc, nc = i(R), i(patchSize), i(faceCells), i(nbrCells)
    bou = np.ascontiguousarray(bou, np.float64)
    n = max(fc.size, 1)
    cps, cfc, cnc, f2c = np.zeros(max(ps.size, 1), np.int32), np.zeros(n, np.int32), np.zeros(n, np.int32), \
        np.zeros(n, np.int32)
    cb = np.zeros(n)
    k = lib().ldu_gamg_coarse_interfaces(_p(R, i32p), ps.size, _p(ps, i32p), _p(fc, i32p), _p(nc, i32p), _p(bou),
                                         _p(cps, i32p), _p(cfc, i32p), _p(cnc, i32p), _p(cb), _p(f2c, i32p))
    return cps[:ps.size], cfc[:k], cnc[:k], cb[:k], f2c[:fc.size]


def face_area_pair_weights(Sf):
    Sf = np.ascontiguousarray(Sf, np.float64).reshape(-1)
    w = np.empty(Sf.size // 3)
    lib().ldu_face_area_pair_weights(w.size, _p(Sf), _p(w))
    return w


class Agglomeration:
    def __init__(self, s, weights=None, n_coarsest=10, forward=True):
        if weights is None:
            weights = face_area_pair_weights(s["Sf"])
        self.w = np.ascontiguousarray(weights, np.float64)
        self.l = np.ascontiguousarray(s["l"], np.int32)
        self.u = np.ascontiguousarray(s["u"], np.int32)
        self.c = LduAgglomeration()
        rc = lib().ldu_gamg_agglomerate(s["diag"].size, self.l.size, _p(self.l, i32p), _p(self.u, i32p),
                                        _p(self.w), n_coarsest, int(forward), ctypes.byref(self.c))
        if rc != 0:
            raise ValueError("no coarse level created")
        self.nCellsFine = s["diag"].size
        self.nFacesFine = self.l.size

    def __del__(self):
        try:
            lib().ldu_gamg_free(ctypes.byref(self.c))
        except Exception:
            pass

    @property
    def n_levels(self):
        return self.c.nLevels

    def level(self, i):
        """(restrictAddr, faceRestrict, faceFlip, nCells, nFaces, coarse l, coarse u)."""
        nf_cells = self.nCellsFine if i == 0 else self.c.nCells[i - 1]
        nf_faces = self.nFacesFine if i == 0 else self.c.nFaces[i - 1]
        nc, ncf = self.c.nCells[i], self.c.nFaces[i]
        A = np.ctypeslib.as_array
        return (A(self.c.restrictAddr[i], (nf_cells,)).copy(),
                A(self.c.faceRestrict[i], (max(nf_faces, 1),))[:nf_faces].copy(),
                A(self.c.faceFlip[i], (max(nf_faces, 1),))[:nf_faces].copy(),
                nc, ncf,
                A(self.c.cl[i], (max(ncf, 1),))[:ncf].copy(),
                A(self.c.cu[i], (max(ncf, 1),))[:ncf].copy())


def gamg(s, psi, agg=None, tol=1e-6, rel_tol=0.0, max_iter=1000, min_iter=0, smoother="GaussSeidel",
         nPreSweeps=0, nPostSweeps=2, nFinestSweeps=2, maxPreSweeps=4, maxPostSweeps=4,
         preSweepsLevelMultiplier=1, postSweepsLevelMultiplier=1, scaleCorrection=None,
         nCellsInCoarsestLevel=10, interpolateCorrection=False, directSolveCoarsest=False):
    """GAMGSolver::solve with faceAreaPair agglomeration; psi updated in place."""
    if agg is None:
        agg = Agglomeration(s, n_coarsest=nCellsInCoarsestLevel)
    m = Matrix(s)
    b = np.ascontiguousarray(s["source"], np.float64)
    g = LduGamgControls(nPreSweeps, preSweepsLevelMultiplier, maxPreSweeps, nPostSweeps,
                        postSweepsLevelMultiplier, maxPostSweeps, nFinestSweeps,
                        -1 if scaleCorrection is None else int(scaleCorrection), SMOOTHERS[smoother],
                        int(bool(interpolateCorrection)), int(bool(directSolveCoarsest)))
    perf = LduPerf()
    c = _controls(tol, rel_tol, max_iter, min_iter)
    rc = lib().ldu_gamg(ctypes.byref(m.c), ctypes.byref(agg.c), _p(psi), _p(b), ctypes.byref(c),
                        ctypes.byref(g), ctypes.byref(perf))
    if rc == -2:
        raise ValueError("Singular matrix")
    if rc == -3:
        raise ValueError("directSolveCoarsest with interfaces needs each patch's partner patch")
    if rc != 0:
        raise ValueError("GAMG failed")
    return _perf(perf)


def pcg_gamg(s, psi, agg=None, tol=1e-6, rel_tol=0.0, max_iter=1000, min_iter=0, nVcycles=2, pre_tol=1e-6,
             pre_rel_tol=0.0, smoother="GaussSeidel", nPreSweeps=0, nPostSweeps=2, nFinestSweeps=2,
             maxPreSweeps=4, maxPostSweeps=4, preSweepsLevelMultiplier=1, postSweepsLevelMultiplier=1,
             scaleCorrection=None, nCellsInCoarsestLevel=10, interpolateCorrection=False,
             directSolveCoarsest=False):
    """PCG with the GAMG preconditioner (GAMGPreconditioner.C:81-148)."""
    if agg is None:
        agg = Agglomeration(s, n_coarsest=nCellsInCoarsestLevel)
    m = Matrix(s)
    b = np.ascontiguousarray(s["source"], np.float64)
    g = LduGamgControls(nPreSweeps, preSweepsLevelMultiplier, maxPreSweeps, nPostSweeps,
                        postSweepsLevelMultiplier, maxPostSweeps, nFinestSweeps,
                        -1 if scaleCorrection is None else int(scaleCorrection), SMOOTHERS[smoother],
                        int(bool(interpolateCorrection)), int(bool(directSolveCoarsest)))
    perf = LduPerf()
    c = _controls(tol, rel_tol, max_iter, min_iter)
    pc = _controls(pre_tol, pre_rel_tol, 1000, 0)
    rc = lib().ldu_pcg_gamg(ctypes.byref(m.c), ctypes.byref(agg.c), _p(psi), _p(b), ctypes.byref(c),
                            ctypes.byref(g), ctypes.byref(pc), int(nVcycles), ctypes.byref(perf))
    if rc != 0:
        raise ValueError("PCG/GAMG failed")
    return _perf(perf)


def coarse_matrix(fine, agg, i):
    """Coarse (diag, upper, lower) of level i from the fine system dict."""
    ra, fra, flip, nc, ncf, _, _ = agg.level(i)
    cd = np.empty(nc)
    cu = np.empty(max(ncf, 1))
    lo = fine.get("lower")
    cl = None if lo is None else np.empty(max(ncf, 1))
    lib().ldu_gamg_coarse_matrix(fine["diag"].size, fra.size, _p(np.ascontiguousarray(fine["diag"])),
                                 _p(np.ascontiguousarray(fine["upper"])),
                                 _p(None if lo is None else np.ascontiguousarray(lo)),
                                 _p(ra, i32p), _p(fra, i32p), _p(flip, i32p), nc, ncf,
                                 _p(cd), _p(cu), _p(cl))
    return cd, cu[:ncf], (None if cl is None else cl[:ncf])


class LduFvGeom(ctypes.Structure):
    _fields_ = [("nCells", ctypes.c_int), ("nFaces", ctypes.c_int), ("nBoundary", ctypes.c_int),
                ("l", i32p), ("u", i32p), ("magSf", f64p), ("deltaCoeffs", f64p), ("weights", f64p),
                ("V", f64p), ("bCell", i32p), ("magSfB", f64p), ("deltaCoeffsB", f64p)]


class LduFvmTerms(ctypes.Structure):
    _fields_ = [("rDeltaT", ctypes.c_double), ("psi0", f64p), ("phi", f64p), ("phiB", f64p),
                ("divScheme", ctypes.c_int), ("lapSign", ctypes.c_int), ("gammaUniform", ctypes.c_double),
                ("gamma", f64p), ("gammaB", f64p), ("bcType", i32p), ("bcValue", f64p), ("su", f64p)]


DIV_SCHEMES = {"upwind": 0, "linear": 1}


def fvm_assemble(l, u, geom, rDeltaT=0.0, psi0=None, phi=None, phiB=None, div="upwind", lapSign=0, gamma=1.0,
                 gammaB=None, bcType=None, bcValue=None, su=None, coupled=False):
    """The lduMatrix (diag, upper, lower or None) and source that
    fvMatrix::solveSegregated hands to the solver for
    fvm::ddt + fvm::div - or + fvm::laplacian == su (ldu_fvm_assemble).
    geom: magSf, deltaCoeffs, weights, V, bCell, magSfB, deltaCoeffsB.
    coupled: also return the cyclic faces' (bcType 3) interfaceBouCoeffs
    and interfaceIntCoeffs, in boundary-face order."""
    f = lambda a: None if a is None else np.ascontiguousarray(a, np.float64)
    i = lambda a: None if a is None else np.ascontiguousarray(a, np.int32)
    l, u = i(l), i(u)
    g = {k: f(geom[k]) if k != "bCell" else i(geom[k]) for k in geom}
    nC, nF, nB = g["V"].size, l.size, g["bCell"].size
    keep = [l, u, g]
    gc = LduFvGeom(nC, nF, nB, _p(l, i32p), _p(u, i32p), _p(g["magSf"]), _p(g["deltaCoeffs"]),
                   _p(g.get("weights")), _p(g["V"]), _p(g["bCell"], i32p), _p(g["magSfB"]), _p(g["deltaCoeffsB"]))
    uniform = np.isscalar(gamma)
    arrs = dict(psi0=f(psi0), phi=f(phi), phiB=f(phiB), gamma=None if uniform else f(gamma), gammaB=f(gammaB),
                bcType=i(bcType), bcValue=f(bcValue), su=f(su))
    keep.append(arrs)
    t = LduFvmTerms(float(rDeltaT), _p(arrs["psi0"]), _p(arrs["phi"]), _p(arrs["phiB"]), DIV_SCHEMES[div],
                    int(lapSign), float(gamma) if uniform else 0.0, _p(arrs["gamma"]), _p(arrs["gammaB"]),
                    _p(arrs["bcType"], i32p), _p(arrs["bcValue"]), _p(arrs["su"]))
    diag, upper, source = np.empty(nC), np.empty(max(nF, 1)), np.empty(nC)
    lower = np.empty(max(nF, 1)) if phi is not None else None
    nCyc = int(np.count_nonzero(arrs["bcType"] == 3)) if arrs["bcType"] is not None else 0
    ifBou, ifInt = np.empty(max(nCyc, 1)), np.empty(max(nCyc, 1))
    rc = lib().ldu_fvm_assemble_coupled(ctypes.byref(gc), ctypes.byref(t), _p(diag), _p(upper), _p(lower),
                                        _p(source), _p(ifBou), _p(ifInt))
    if rc == -2:
        raise ValueError("linear div with cyclic faces")
    if rc != 0:
        raise ValueError("no term")
    del keep
    out = (diag, upper[:nF], None if lower is None else lower[:nF], source)
    return out + (ifBou[:nCyc], ifInt[:nCyc]) if coupled else out
