"""Python front end of libcudaLduSolvers.so, mirroring OpenFOAM's interface.

    mesh   = LduMesh(ctx, nCells, lowerAddr, upperAddr)          # lduAddressing
    A      = LduMatrix(mesh, diag, upper, lower=None)             # lduMatrix
    solver = solver_new("T", A, {"solver": "cudaPCG",             # lduMatrix::solver::New
                                 "preconditioner": "DIC",
                                 "tolerance": 1e-8, "relTol": 0})
    perf   = solver.solve(psi, source)                            # SolverPerformance

Names, defaults and errors follow the reference (lduMatrixSolver.C:40-164,
GAMGSolver.C:48-388, SolverPerformance.C:96-126): an unknown solver name
raises ``FatalError`` with "Unknown symmetric matrix solver <name>"; numerical
failure is reported through ``perf.singular`` / ``perf.converged``.  Solver
names are the plugin's (``cudaPCG``, ``cudaPBiCGStab``, ``cudaGAMG``); the
reference names ``PCG``/``PBiCGStab``/``GAMG`` are accepted as aliases.

Everything runs on the GPU through the C ABI in include/cfx.h.  There is no
CPU fallback: without the shared library, or without a CUDA device, every
call raises.
"""
import atexit
import ctypes
import os
import weakref
from dataclasses import dataclass

import numpy as np

from . import LIB_DIR

LIB_PATH = os.path.join(LIB_DIR, "libcudaLduSolvers.so")

SOLVER_PCG, SOLVER_PBICGSTAB, SOLVER_GAMG, SOLVER_SMOOTH, SOLVER_PBICG = 0, 1, 2, 3, 4
PRECONDITIONERS = {"none": 0, "diagonal": 1, "DIC": 2, "DILU": 3, "GAMG": 4, "FDIC": 5}
SMOOTHERS = {"GaussSeidel": 0, "DIC": 1, "symGaussSeidel": 2, "DILU": 3, "DICGaussSeidel": 4,
             "DILUGaussSeidel": 5, "FDIC": 6, "nonBlockingGaussSeidel": 7}
# the smoothers' run-time tables by matrix symmetry
SYM_SMOOTHERS = ("DIC", "DICGaussSeidel", "FDIC", "GaussSeidel", "nonBlockingGaussSeidel", "symGaussSeidel")
ASYM_SMOOTHERS = ("DILU", "DILUGaussSeidel", "GaussSeidel", "nonBlockingGaussSeidel", "symGaussSeidel")
SOLVERS = {"cudaPCG": SOLVER_PCG, "cudaPBiCGStab": SOLVER_PBICGSTAB, "cudaGAMG": SOLVER_GAMG,
           "cudaSmoothSolver": SOLVER_SMOOTH, "cudaPBiCG": SOLVER_PBICG,
           "PCG": SOLVER_PCG, "PBiCGStab": SOLVER_PBICGSTAB, "GAMG": SOLVER_GAMG, "smoothSolver": SOLVER_SMOOTH,
           "PBiCG": SOLVER_PBICG}
SYM_SOLVERS = ("cudaGAMG", "cudaPBiCGStab", "cudaPCG", "cudaSmoothSolver")
ASYM_SOLVERS = ("cudaGAMG", "cudaPBiCG", "cudaPBiCGStab", "cudaSmoothSolver")

STATUS = {0: "ok", -1: "bad argument", -2: "bad addressing", -3: "CUDA error", -4: "out of memory",
          -5: "admission refused", -6: "device wait timed out", -7: "bad configuration", -8: "bad state",
          -9: "fatal error"}


class FatalError(RuntimeError):
    """The reference's FatalError / FatalIOError (configuration errors)."""


class CfxError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class Perf(ctypes.Structure):
    _fields_ = [("solverName", ctypes.c_char * 32), ("initialResidual", ctypes.c_double),
                ("finalResidual", ctypes.c_double), ("nIterations", ctypes.c_int), ("converged", ctypes.c_int),
                ("singular", ctypes.c_int), ("status", ctypes.c_int), ("nOuter", ctypes.c_int),
                ("pad", ctypes.c_int)]


class Controls(ctypes.Structure):
    _fields_ = [("solver", ctypes.c_int), ("preconditioner", ctypes.c_int), ("tolerance", ctypes.c_double),
                ("relTol", ctypes.c_double), ("maxIter", ctypes.c_int), ("minIter", ctypes.c_int),
                ("smoother", ctypes.c_int), ("nPreSweeps", ctypes.c_int),
                ("preSweepsLevelMultiplier", ctypes.c_int), ("maxPreSweeps", ctypes.c_int),
                ("nPostSweeps", ctypes.c_int), ("postSweepsLevelMultiplier", ctypes.c_int),
                ("maxPostSweeps", ctypes.c_int), ("nFinestSweeps", ctypes.c_int),
                ("scaleCorrection", ctypes.c_int), ("nCellsInCoarsestLevel", ctypes.c_int),
                ("precision", ctypes.c_int), ("nSweeps", ctypes.c_int), ("nVcycles", ctypes.c_int),
                ("interpolateCorrection", ctypes.c_int), ("pcTolerance", ctypes.c_double),
                ("pcRelTol", ctypes.c_double), ("directSolveCoarsest", ctypes.c_int), ("reserved", ctypes.c_int)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbmBudget", ctypes.c_int64), ("largeCells", ctypes.c_int), ("maxBatch", ctypes.c_int),
                ("nCellsInCoarsestLevel", ctypes.c_int), ("groupCells", ctypes.c_int), ("groupSize", ctypes.c_int),
                ("lanes", ctypes.c_int)]


class ServerStats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int64) for k in ("submitted", "completed", "cancelled", "failed", "refused", "batches",
                                              "batchedSolves", "largeSolves", "queueDepth", "running",
                                              "residentMatrices", "hbmInUse", "hbmBudget")] + \
               [(k, ctypes.c_double) for k in ("elapsedS", "solvesPerS", "p50Ms", "p99Ms", "meanMs", "maxMs")] + \
               [("largeYields", ctypes.c_int64)] + \
               [(k, ctypes.c_double) for k in ("queueP50Ms", "queueP99Ms", "runP50Ms", "runP99Ms")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# exported symbols and their signatures (every declaration of include/cfx.h)
_vp = ctypes.c_void_p
_i = ctypes.c_int
_d = ctypes.c_double
class FvmTerms(ctypes.Structure):
    """cfx_fvm_terms: the terms of a device-side fvMatrix assembly."""
    _fields_ = [("rDeltaT", ctypes.c_double), ("psi0", ctypes.c_void_p), ("phi", ctypes.c_void_p),
                ("phiB", ctypes.c_void_p), ("divScheme", ctypes.c_int), ("lapSign", ctypes.c_int),
                ("gammaUniform", ctypes.c_double), ("gamma", ctypes.c_void_p), ("gammaB", ctypes.c_void_p),
                ("bcType", ctypes.c_void_p), ("bcValue", ctypes.c_void_p), ("su", ctypes.c_void_p)]


DIV_SCHEMES = {"upwind": 0, "linear": 1}
BC_TYPES = {"zeroGradient": 0, "fixedValue": 1, "fixedGradient": 2, "cyclic": 3}


_SIG = {
    "cfx_default_controls": (None, [ctypes.POINTER(Controls)]),
    "cfx_last_error": (ctypes.c_char_p, []),
    "cfx_version": (_i, []),
    "cfx_ctx_create": (_i, [_i, ctypes.POINTER(_vp)]),
    "cfx_ctx_destroy": (_i, [_vp]),
    "cfx_ctx_stream": (_i, [_vp, ctypes.POINTER(_vp)]),
    "cfx_ctx_synchronize": (_i, [_vp]),
    "cfx_ctx_launch_count": (_i, [_vp, ctypes.POINTER(ctypes.c_int64)]),
    "cfx_mesh_create": (_i, [_vp, _i, _i, _vp, _vp, ctypes.POINTER(_vp)]),
    "cfx_mesh_destroy": (_i, [_vp]),
    "cfx_mesh_set_interface_partners": (_i, [_vp, _vp]),
    "cfx_mesh_info": (_i, [_vp, ctypes.POINTER(_i), ctypes.POINTER(_i)]),
    "cfx_mesh_sell_info": (_i, [_vp, ctypes.POINTER(_i), ctypes.POINTER(_i), ctypes.POINTER(ctypes.c_int64)]),
    "cfx_face_area_pair_weights": (_i, [_i, _vp, _vp]),
    "cfx_gamg_agglomerate": (_i, [_vp, _vp, _i, _i]),
    "cfx_gamg_coarse_interfaces": (_i, [_i, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "cfx_gamg_set_levels": (_i, [_vp, _i, _vp, _vp]),
    "cfx_gamg_level_info": (_i, [_vp, _i, ctypes.POINTER(_i), ctypes.POINTER(_i), _vp, _vp, _vp, _vp, _vp]),
    "cfx_gamg_n_levels": (_i, [_vp, ctypes.POINTER(_i)]),
    "cfx_matrix_create": (_i, [_vp, _vp, _vp, _vp, ctypes.POINTER(_vp)]),
    "cfx_matrix_update": (_i, [_vp, _vp, _vp, _vp]),
    "cfx_matrix_update_device": (_i, [_vp, _vp, _vp, _vp]),
    "cfx_matrix_create_empty": (_i, [_vp, _i, ctypes.POINTER(_vp)]),
    "cfx_mesh_set_interfaces": (_i, [_vp, _i, _vp, _vp, _vp]),
    "cfx_matrix_set_interface_coeffs": (_i, [_vp, _vp, _vp]),
    "cfx_fv_geometry": (_i, [_vp, _vp, _vp, _vp, _vp, _i, _vp, _vp, _vp]),
    "cfx_fvm_assemble": (_i, [_vp, ctypes.POINTER(FvmTerms), _vp]),
    "cfx_matrix_destroy": (_i, [_vp]),
    "cfx_matrix_coarse": (_i, [_vp, _i, _vp, _vp, _vp]),
    "cfx_solve": (_i, [_vp, ctypes.POINTER(Controls), _vp, _vp, ctypes.POINTER(Perf)]),
    "cfx_solve_device": (_i, [_vp, ctypes.POINTER(Controls), _vp, _vp, ctypes.POINTER(Perf)]),
    "cfx_tune_set": (_i, [_i, _i]),
    "cfx_tune_get": (_i, [_i, ctypes.POINTER(_i)]),
    "cfx_amul": (_i, [_vp, _vp, _vp]),
    "cfx_tmul": (_i, [_vp, _vp, _vp]),
    "cfx_residual": (_i, [_vp, _vp, _vp, _vp]),
    "cfx_sumA": (_i, [_vp, _vp]),
    "cfx_reduce": (_i, [_vp, _i, _i, _vp, _vp, ctypes.POINTER(_d)]),
    "cfx_norm_factor": (_i, [_vp, _vp, _vp, ctypes.POINTER(_d)]),
    "cfx_precondition": (_i, [_vp, _i, _i, _vp, _vp]),
    "cfx_reciprocal_d": (_i, [_vp, _i, _vp]),
    "cfx_smooth": (_i, [_vp, _i, _vp, _vp, _i]),
    "cfx_diag_sweep_stall": (_i, [_vp, _i, ctypes.POINTER(_i)]),
    "cfx_diag_smooth_f32": (_i, [_vp, _i, _vp, _vp, _i, ctypes.POINTER(_i)]),
    "cfx_reduce_noalloc": (_i, [_i, _i, _vp, _vp, _vp, _vp]),
    "cfx_batch_create": (_i, [_vp, _i, _vp, _vp, _vp, _vp, ctypes.POINTER(_vp)]),
    "cfx_batch_destroy": (_i, [_vp]),
    "cfx_batch_set_matrix": (_i, [_vp, _i, _vp, _vp, _vp]),
    "cfx_batch_solve": (_i, [_vp, ctypes.POINTER(Controls), _vp, _vp, _vp]),
    "cfx_batch_vectors": (_i, [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp), _vp]),
    "cfx_batch_solve_device": (_i, [_vp, ctypes.POINTER(Controls), _vp]),
    "cfx_batch_timings": (_i, [_vp, _vp, _vp]),
    "cfx_batch_set_ctas_per_sm": (_i, [_vp, _i]),
    "cfx_batch_set_groups": (_i, [_vp, _i, _i]),
    "cfx_server_default_config": (None, [ctypes.POINTER(ServerConfig)]),
    "cfx_server_create": (_i, [_vp, ctypes.POINTER(ServerConfig), ctypes.POINTER(_vp)]),
    "cfx_server_destroy": (_i, [_vp]),
    "cfx_server_add_matrix": (_i, [_vp, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.POINTER(ctypes.c_int64)]),
    "cfx_server_remove_matrix": (_i, [_vp, ctypes.c_int64]),
    "cfx_server_submit": (_i, [_vp, ctypes.c_int64, ctypes.POINTER(Controls), _vp, _vp,
                               ctypes.POINTER(ctypes.c_int64)]),
    "cfx_server_wait": (_i, [_vp, ctypes.c_int64, _i, _vp, ctypes.POINTER(Perf)]),
    "cfx_server_cancel": (_i, [_vp, ctypes.c_int64]),
    "cfx_server_release": (_i, [_vp, ctypes.c_int64]),
    "cfx_server_stats": (_i, [_vp, ctypes.POINTER(ServerStats)]),
    "cfx_server_reset_stats": (_i, [_vp]),
    "cfx_batch_get_groups": (_i, [_vp, ctypes.POINTER(_i), ctypes.POINTER(_i), ctypes.POINTER(_i)]),
    "cfx_batch_tune": (_i, [_vp, ctypes.POINTER(Controls), ctypes.POINTER(_i), ctypes.POINTER(ctypes.c_float)]),
}

_lib = None

# Live handles by kind, closed at interpreter exit in dependency order
# (batches and matrices before the meshes they use, meshes before their
# context), while the library and the CUDA runtime are still intact.
_LIVE = {k: weakref.WeakSet() for k in ("server", "batch", "matrix", "mesh", "ctx")}


def _track(kind, obj):
    _LIVE[kind].add(obj)


@atexit.register
def _close_all():
    for kind in ("server", "batch", "matrix", "mesh", "ctx"):
        for obj in list(_LIVE[kind]):
            try:
                obj.close()
            except Exception:
                pass


def lib():
    """Load the solver library (raises when it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() (no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIG.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    return list(_SIG)


def _check(rc, what=""):
    if rc != 0:
        msg = lib().cfx_last_error().decode(errors="replace")
        if rc in (-7, -9):
            raise FatalError(msg)
        raise CfxError(rc, f"{what}: {msg}")


def _hp(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def _dp(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


class Context:
    """A device context: one CUDA stream on one GPU."""

    def __init__(self, device=0):
        h = ctypes.c_void_p()
        _check(lib().cfx_ctx_create(device, ctypes.byref(h)), "cfx_ctx_create")
        self.h = h
        self.device = device
        _track("ctx", self)

    def stream(self):
        s = ctypes.c_void_p()
        _check(lib().cfx_ctx_stream(self.h, ctypes.byref(s)), "cfx_ctx_stream")
        return s.value

    def synchronize(self):
        _check(lib().cfx_ctx_synchronize(self.h), "cfx_ctx_synchronize")

    def launch_count(self):
        c = ctypes.c_int64()
        _check(lib().cfx_ctx_launch_count(self.h, ctypes.byref(c)), "launch_count")
        return c.value

    def reduce(self, which, a, b=None):
        out = ctypes.c_double()
        _check(lib().cfx_reduce(self.h, which, a.numel(), _dp(a), _dp(b), ctypes.byref(out)), "cfx_reduce")
        return out.value

    def close(self):
        h, self.h = getattr(self, "h", None), None
        if h:
            lib().cfx_ctx_destroy(h)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None


def default_context():
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


class LduMesh:
    """lduAddressing resident on the device (with level schedules)."""

    def __init__(self, ctx, nCells, lowerAddr, upperAddr):
        self.ctx = ctx
        self.l = np.ascontiguousarray(lowerAddr, np.int32)
        self.u = np.ascontiguousarray(upperAddr, np.int32)
        self.nCells = int(nCells)
        h = ctypes.c_void_p()
        _check(lib().cfx_mesh_create(ctx.h, self.nCells, self.l.size, _hp(self.l), _hp(self.u), ctypes.byref(h)),
               "cfx_mesh_create")
        self.h = h
        self.gamg_key = None
        _track("mesh", self)

    def schedule_depth(self):
        a, b = ctypes.c_int(), ctypes.c_int()
        _check(lib().cfx_mesh_info(self.h, ctypes.byref(a), ctypes.byref(b)), "cfx_mesh_info")
        return a.value, b.value

    def sell_info(self):
        """(slices, pattern slices, entries) of the finest level's sliced rows."""
        a, b, e = ctypes.c_int(), ctypes.c_int(), ctypes.c_int64()
        _check(lib().cfx_mesh_sell_info(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(e)),
               "cfx_mesh_sell_info")
        return a.value, b.value, e.value

    def agglomerate(self, weights=None, Sf=None, nCellsInCoarsestLevel=10, forward=True):
        """faceAreaPair agglomeration (weights from Sf when not given)."""
        if weights is None:
            weights = face_area_pair_weights(Sf)
        w = np.ascontiguousarray(weights, np.float64)
        _check(lib().cfx_gamg_agglomerate(self.h, _hp(w), int(nCellsInCoarsestLevel), int(bool(forward))),
               "cfx_gamg_agglomerate")
        self.gamg_key = ("faceAreaPair", int(nCellsInCoarsestLevel))

    def set_levels(self, restrict_maps):
        """Use a caller's agglomeration: list of fine->coarse maps."""
        maps = [np.ascontiguousarray(m, np.int32) for m in restrict_maps]
        nco = np.array([int(m.max()) + 1 for m in maps], np.int32)
        arr = (ctypes.c_void_p * len(maps))(*[m.ctypes.data for m in maps])
        _check(lib().cfx_gamg_set_levels(self.h, len(maps), arr, _hp(nco)), "cfx_gamg_set_levels")
        self.gamg_key = ("given", len(maps))

    def n_levels(self):
        n = ctypes.c_int()
        _check(lib().cfx_gamg_n_levels(self.h, ctypes.byref(n)), "cfx_gamg_n_levels")
        return n.value

    def level(self, i, fine_cells, fine_faces):
        nc, ncf = ctypes.c_int(), ctypes.c_int()
        _check(lib().cfx_gamg_level_info(self.h, i, ctypes.byref(nc), ctypes.byref(ncf), None, None, None, None,
                                         None), "level_info")
        ra = np.empty(fine_cells, np.int32)
        fra = np.empty(fine_faces, np.int32)
        fl = np.empty(fine_faces, np.int32)
        cl = np.empty(ncf.value, np.int32)
        cu = np.empty(ncf.value, np.int32)
        _check(lib().cfx_gamg_level_info(self.h, i, None, None, _hp(ra), _hp(fra), _hp(fl), _hp(cl), _hp(cu)),
               "level_info")
        return ra, fra, fl, nc.value, ncf.value, cl, cu

    def set_interfaces(self, patchSizes, faceCells, nbrFaceCells, nbrPatch=None):
        """Coupled (cyclic) interfaces: faces concatenated in patch order;
        nbrPatch: each patch's partner patch (the direct coarsest-level
        solve needs it)."""
        self._if = [np.ascontiguousarray(a, np.int32) for a in (patchSizes, faceCells, nbrFaceCells)]
        _check(lib().cfx_mesh_set_interfaces(self.h, len(self._if[0]), _hp(self._if[0]), _hp(self._if[1]),
                                             _hp(self._if[2])), "cfx_mesh_set_interfaces")
        if nbrPatch is not None:
            self._if.append(np.ascontiguousarray(nbrPatch, np.int32))
            _check(lib().cfx_mesh_set_interface_partners(self.h, _hp(self._if[3])),
                   "cfx_mesh_set_interface_partners")

    def fv_geometry(self, magSf, deltaCoeffs, V, bCell, magSfB, deltaCoeffsB, weights=None):
        """Face geometry for device-side assembly (host arrays, uploaded once):
        internal faces in lduAddressing order, boundary faces in patch order."""
        f = lambda a: None if a is None else np.ascontiguousarray(a, np.float64)
        self._fv = [f(magSf), f(deltaCoeffs), f(weights), f(V), np.ascontiguousarray(bCell, np.int32),
                    f(magSfB), f(deltaCoeffsB)]
        a = self._fv
        _check(lib().cfx_fv_geometry(self.h, _hp(a[0]), _hp(a[1]), _hp(a[2]), _hp(a[3]), len(a[4]), _hp(a[4]),
                                     _hp(a[5]), _hp(a[6])), "cfx_fv_geometry")

    def close(self):
        h, self.h = getattr(self, "h", None), None
        if h:
            lib().cfx_mesh_destroy(h)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LduMatrix:
    """lduMatrix: diag/upper(/lower) coefficients on an LduMesh."""

    def __init__(self, mesh, diag, upper=None, lower=None):
        """upper = lower = None: a diagonal matrix (lduMatrix::diagonal())."""
        self.mesh = mesh
        self.diag = np.ascontiguousarray(diag, np.float64)
        self.upper = None if upper is None else np.ascontiguousarray(upper, np.float64)
        self.lower = None if lower is None else np.ascontiguousarray(lower, np.float64)
        h = ctypes.c_void_p()
        _check(lib().cfx_matrix_create(mesh.h, _hp(self.diag), _hp(self.upper), _hp(self.lower), ctypes.byref(h)),
               "cfx_matrix_create")
        self.h = h
        _track("matrix", self)

    def set_interface_coeffs(self, bou, intc=None):
        """interfaceBouCoeffs / interfaceIntCoeffs, faces concatenated in patch order."""
        self._ifc = [np.ascontiguousarray(bou, np.float64), None if intc is None else
                     np.ascontiguousarray(intc, np.float64)]
        _check(lib().cfx_matrix_set_interface_coeffs(self.h, _hp(self._ifc[0]), _hp(self._ifc[1])),
               "cfx_matrix_set_interface_coeffs")

    @classmethod
    def empty(cls, mesh, symmetric):
        """A matrix of zero coefficients to be assembled on the device."""
        A = cls.__new__(cls)
        A.mesh = mesh
        A.diag = np.zeros(0)
        A.upper = np.zeros(0)
        A.lower = None if symmetric else np.zeros(0)
        h = ctypes.c_void_p()
        _check(lib().cfx_matrix_create_empty(mesh.h, int(bool(symmetric)), ctypes.byref(h)), "cfx_matrix_create_empty")
        A.h = h
        _track("matrix", A)
        return A

    def assemble(self, source, rDeltaT=0.0, psi0=None, phi=None, phiB=None, div="upwind", lapSign=0, gamma=1.0,
                 gammaB=None, bcType=None, bcValue=None, su=None):
        """fvm::ddt(psi) + fvm::div(phi, psi) + lapSign*fvm::laplacian(gamma, psi) == su into this
        matrix and `source` (CUDA float64 tensors; gamma a float or per-face tensors gamma/gammaB;
        bcType an int32 tensor of BC_TYPES values)."""
        import torch
        uniform = not isinstance(gamma, torch.Tensor)
        t = FvmTerms(float(rDeltaT), _dp(psi0), _dp(phi), _dp(phiB), DIV_SCHEMES[div], int(lapSign),
                     float(gamma) if uniform else 0.0, None if uniform else _dp(gamma), _dp(gammaB),
                     _dp(bcType), _dp(bcValue), _dp(su))
        _check(lib().cfx_fvm_assemble(self.h, ctypes.byref(t), _dp(source)), "cfx_fvm_assemble")

    def diagonal(self):
        return self.upper is None and self.lower is None

    def symmetric(self):
        return self.upper is not None and self.lower is None

    def asymmetric(self):
        return self.lower is not None

    def update(self, diag, upper=None, lower=None):
        self.diag = np.ascontiguousarray(diag, np.float64)
        self.upper = None if upper is None else np.ascontiguousarray(upper, np.float64)
        self.lower = None if lower is None else np.ascontiguousarray(lower, np.float64)
        _check(lib().cfx_matrix_update(self.h, _hp(self.diag), _hp(self.upper), _hp(self.lower)), "update")

    # single operations on torch CUDA tensors (float64)
    def Amul(self, x, y):
        _check(lib().cfx_amul(self.h, _dp(x), _dp(y)), "cfx_amul")

    def Tmul(self, x, y):
        _check(lib().cfx_tmul(self.h, _dp(x), _dp(y)), "cfx_tmul")

    def residual(self, x, b, r):
        _check(lib().cfx_residual(self.h, _dp(x), _dp(b), _dp(r)), "cfx_residual")

    def sumA(self, s):
        _check(lib().cfx_sumA(self.h, _dp(s)), "cfx_sumA")

    def normFactor(self, psi, b):
        out = ctypes.c_double()
        _check(lib().cfx_norm_factor(self.h, _dp(psi), _dp(b), ctypes.byref(out)), "normFactor")
        return out.value

    def precondition(self, kind, r, w, transpose=False):
        _check(lib().cfx_precondition(self.h, PRECONDITIONERS[kind], int(transpose), _dp(r), _dp(w)), "precondition")

    def reciprocalD(self, kind, rD):
        _check(lib().cfx_reciprocal_d(self.h, PRECONDITIONERS[kind], _dp(rD)), "reciprocalD")

    def smooth(self, kind, psi, b, nSweeps):
        _check(lib().cfx_smooth(self.h, SMOOTHERS[kind], _dp(psi), _dp(b), int(nSweeps)), "smooth")

    def smooth_f32(self, kind, psi, b, nSweeps):
        """The FP32 inner cycles' smoothing of this matrix alone (psi, b:
        float32 CUDA tensors); returns the Gauss-Seidel schedule's execution
        form (cfx_diag_smooth_f32)."""
        form = ctypes.c_int(-1)
        _check(lib().cfx_diag_smooth_f32(self.h, SMOOTHERS[kind], _dp(psi), _dp(b), int(nSweeps),
                                         ctypes.byref(form)), "cfx_diag_smooth_f32")
        return form.value

    def diag_sweep_stall(self, timeout_ms):
        """Device status of a sweep whose bounded waits are made to expire."""
        st = ctypes.c_int()
        _check(lib().cfx_diag_sweep_stall(self.h, int(timeout_ms), ctypes.byref(st)), "cfx_diag_sweep_stall")
        return st.value

    def coarse(self, level, nCells, nFaces):
        d = np.empty(nCells)
        up = np.empty(nFaces)
        lo = None if self.lower is None else np.empty(nFaces)
        _check(lib().cfx_matrix_coarse(self.h, level, _hp(d), _hp(up), _hp(lo)), "coarse")
        return d, up, lo

    def close(self):
        h, self.h = getattr(self, "h", None), None
        if h:
            lib().cfx_matrix_destroy(h)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class SolverPerformance:
    solverName: str
    fieldName: str
    initialResidual: float
    finalResidual: float
    nIterations: int
    converged: bool
    singular: bool
    nOuter: int = 0

    def __str__(self):
        # SolverPerformance::print (SolverPerformance.C:96-126)
        if self.singular:
            return f"{self.solverName}:  Solving for {self.fieldName}:  solution singularity"
        return (f"{self.solverName}:  Solving for {self.fieldName}, Initial residual = {self.initialResidual:g}, "
                f"Final residual = {self.finalResidual:g}, No Iterations {self.nIterations}")


TUNE_SMALL_SWEEP, TUNE_CLUSTER_GLOBAL, TUNE_CLUSTER_SIZE, TUNE_BATCH_INNER_DIGITS, TUNE_SMEM_BYTES = 0, 1, 2, 3, 4
TUNE_GRID_WAVE = 5
TUNE_CLUSTER_PRE = 6
TUNE_FLOW = 7
TUNE_FLOW_AHEAD = 8
TUNE_AMUL_SELL = 9
TUNE_GRID_STRIDE, TUNE_GRID_POLL_NS, TUNE_CHUNK_GROUPS, TUNE_CTA_XL = 10, 11, 12, 13
TUNE_COLORED_GS = 14
TUNE_COLORED_PRE = 15
TUNE_LEVEL_LAUNCH = 16


def tune_set(key, value):
    _check(lib().cfx_tune_set(int(key), int(value)), "cfx_tune_set")


def tune_get(key):
    v = ctypes.c_int()
    _check(lib().cfx_tune_get(int(key), ctypes.byref(v)), "cfx_tune_get")
    return v.value


def gamg_coarse_interfaces(restrictAddr, patchSize, faceCells, nbrCells):
    """One GAMG level's coarse cyclic interfaces (cfx_gamg_coarse_interfaces,
    host only): (coarse patch sizes, face cells, partner cells, each fine
    face's coarse face)."""
    R = np.ascontiguousarray(restrictAddr, np.int32)
    ps = np.ascontiguousarray(patchSize, np.int32)
    fc = np.ascontiguousarray(faceCells, np.int32)
    nc = np.ascontiguousarray(nbrCells, np.int32)
    cps, cfc, cnc, f2c = (np.zeros(max(a, 1), np.int32) for a in (ps.size, fc.size, fc.size, fc.size))
    n = ctypes.c_int32()
    _check(lib().cfx_gamg_coarse_interfaces(R.size, _hp(R), ps.size, _hp(ps), _hp(fc), _hp(nc), _hp(cps), _hp(cfc),
                                            _hp(cnc), _hp(f2c), ctypes.byref(n)), "cfx_gamg_coarse_interfaces")
    return cps[:ps.size], cfc[:n.value], cnc[:n.value], f2c[:fc.size]


def face_area_pair_weights(Sf):
    Sf = np.ascontiguousarray(Sf, np.float64).reshape(-1)
    w = np.empty(Sf.size // 3)
    _check(lib().cfx_face_area_pair_weights(w.size, _hp(Sf), _hp(w)), "weights")
    return w


def _controls(d, sym):
    c = Controls()
    lib().cfx_default_controls(ctypes.byref(c))
    name = d.get("solver")
    if name is None:
        raise FatalError("keyword solver is undefined in dictionary")
    table = SYM_SOLVERS if sym else ASYM_SOLVERS
    if name not in SOLVERS or SOLVERS[name] not in [SOLVERS[t] for t in table]:
        kind = "symmetric" if sym else "asymmetric"
        raise FatalError(f"Unknown {kind} matrix solver {name}\n\nValid {kind} matrix solvers are : {list(table)}")
    c.solver = SOLVERS[name]
    gd = d  # the dictionary of the GAMG keys (the solver's, or the GAMG preconditioner's)
    if c.solver not in (SOLVER_GAMG, SOLVER_SMOOTH):
        pre = d.get("preconditioner", "none")
        pd = None
        if isinstance(pre, dict):
            pd = pre
            pre = pre.get("preconditioner", "none")
        if pre not in PRECONDITIONERS or (pre == "GAMG" and pd is None):
            raise FatalError(f"Unknown {'symmetric' if sym else 'asymmetric'} matrix preconditioner {pre}")
        c.preconditioner = PRECONDITIONERS[pre]
        if pre == "GAMG":
            gd = pd
            c.nVcycles = int(pd.get("nVcycles", 2))
            c.pcTolerance = float(pd.get("tolerance", 1e-6))
            c.pcRelTol = float(pd.get("relTol", 0.0))
    c.tolerance = float(d.get("tolerance", 1e-6))
    c.relTol = float(d.get("relTol", 0.0))
    c.maxIter = int(d.get("maxIter", 1000))
    c.minIter = int(d.get("minIter", 0))
    sm = gd.get("smoother", "GaussSeidel")
    uses_smoother = c.solver in (SOLVER_GAMG, SOLVER_SMOOTH) or c.preconditioner == PRECONDITIONERS["GAMG"]
    if uses_smoother and sm not in (SYM_SMOOTHERS if sym else ASYM_SMOOTHERS):
        kind = "symmetric" if sym else "asymmetric"
        table = list(SYM_SMOOTHERS if sym else ASYM_SMOOTHERS)
        raise FatalError(f"Unknown {kind} matrix smoother {sm}\n\nValid {kind} matrix smoothers are : {table}")
    c.smoother = SMOOTHERS.get(sm, 0)
    c.nSweeps = int(d.get("nSweeps", 1))
    for k in ("nPreSweeps", "preSweepsLevelMultiplier", "maxPreSweeps", "nPostSweeps",
              "postSweepsLevelMultiplier", "maxPostSweeps", "nFinestSweeps", "nCellsInCoarsestLevel"):
        if k in gd:
            setattr(c, k, int(gd[k]))
    if "minCellsPerProcessor" in gd:
        c.nCellsInCoarsestLevel = int(gd["minCellsPerProcessor"])
    if "scaleCorrection" in gd:
        c.scaleCorrection = int(bool(gd["scaleCorrection"]))
    c.interpolateCorrection = int(bool(gd.get("interpolateCorrection", False)))
    c.directSolveCoarsest = int(bool(gd.get("directSolveCoarsest", False)))
    if gd.get("agglomerator", "faceAreaPair") != "faceAreaPair":
        raise FatalError(f"Unknown GAMGAgglomeration type {gd['agglomerator']}")
    prec = str(d.get("precision", "FP64"))
    if prec not in ("FP64", "mixed"):
        raise FatalError(f"Unknown precision {prec} (FP64 or mixed)")
    c.precision = 1 if prec == "mixed" else 0
    return c


class Solver:
    """lduMatrix::solver for cudaPCG / cudaPBiCGStab / cudaGAMG."""

    def __init__(self, fieldName, matrix, controls):
        self.fieldName = fieldName
        self.matrix = matrix
        self.read(controls)

    def read(self, controls):
        self.controlDict = dict(controls)
        if getattr(self.matrix, "diagonal", lambda: False)():
            # diagonalSolver: chosen before the solver name is looked at
            # (lduMatrixSolver.C:52-66); the keyword must still be present
            if "solver" not in self.controlDict:
                raise FatalError("keyword solver is undefined in dictionary")
            self.c = Controls()
            lib().cfx_default_controls(ctypes.byref(self.c))
            return
        self.c = _controls(self.controlDict, self.matrix.symmetric())

    def _perf(self, p):
        return SolverPerformance(p.solverName.decode(), self.fieldName, p.initialResidual, p.finalResidual,
                                 p.nIterations, bool(p.converged), bool(p.singular), p.nOuter)

    def solve(self, psi, source):
        """psi: float64 numpy array (updated in place) or CUDA tensor."""
        p = Perf()
        if isinstance(psi, np.ndarray):
            if psi.dtype != np.float64 or not psi.flags["C_CONTIGUOUS"]:
                raise TypeError("psi must be a contiguous float64 array")
            src = np.ascontiguousarray(source, np.float64)
            rc = lib().cfx_solve(self.matrix.h, ctypes.byref(self.c), _hp(psi), _hp(src), ctypes.byref(p))
        else:
            rc = lib().cfx_solve_device(self.matrix.h, ctypes.byref(self.c), _dp(psi), _dp(source), ctypes.byref(p))
        _check(rc, "solve")
        return self._perf(p)


def solver_new(fieldName, matrix, controls):
    """lduMatrix::solver::New (lduMatrixSolver.C:40-130)."""
    return Solver(fieldName, matrix, controls)


# ---------------------------------------------------------------- convenience
_PRE_FOR = {"PCG": "DIC", "PBiCGStab": "DILU"}


def system_matrix(s, ctx=None):
    """(LduMesh, LduMatrix) for a system dict of cases.py, cached on the dict."""
    if "_cfx" not in s:
        ctx = ctx or default_context()
        mesh = LduMesh(ctx, s["diag"].size, s["l"], s["u"])
        if s.get("ifCell") is not None:  # coupled (cyclic) interfaces
            mesh.set_interfaces(s["ifSize"], s["ifCell"], s["ifNbr"], s.get("ifNbrPatch"))
        A = LduMatrix(mesh, s["diag"], s["upper"], s.get("lower"))
        if s.get("ifCell") is not None:
            A.set_interface_coeffs(s["ifBou"], s.get("ifInt"))
        s["_cfx"] = (mesh, A)
    return s["_cfx"]


def solve(s, psi, controls, field="psi"):
    """Solve system dict s (cases.py layout) with a controls dict."""
    mesh, A = system_matrix(s)
    name = controls["solver"]
    pre = controls.get("preconditioner")
    gd = pre if isinstance(pre, dict) and pre.get("preconditioner") == "GAMG" else None
    if SOLVERS.get(name) == SOLVER_GAMG or gd is not None:
        src = gd if gd is not None else controls
        key = ("faceAreaPair", int(src.get("nCellsInCoarsestLevel", 10)))
        if mesh.gamg_key != key:
            mesh.agglomerate(Sf=s["Sf"], nCellsInCoarsestLevel=key[1])
    return solver_new(field, A, controls).solve(psi, s["source"])


class Batch:
    """Many independent systems solved by one launch (cfx_batch_*).

    ``systems``: list of dicts with ``l``, ``u``, ``diag``, ``upper`` and
    optionally ``lower`` (cases.py layout).  ``solve(psi, source, controls)``
    takes the concatenated vectors (numpy, float64) and returns one
    SolverPerformance per system; ``solve_device`` uses the resident device
    vectors (``vectors()``)."""

    def __init__(self, ctx, systems):
        self.ctx = ctx
        n = len(systems)
        self.nCells = np.array([s["diag"].size for s in systems], np.int32)
        self.nFaces = np.array([s["l"].size for s in systems], np.int32)
        self._l = [np.ascontiguousarray(s["l"], np.int32) for s in systems]
        self._u = [np.ascontiguousarray(s["u"], np.int32) for s in systems]
        la = (ctypes.c_void_p * n)(*[a.ctypes.data for a in self._l])
        ua = (ctypes.c_void_p * n)(*[a.ctypes.data for a in self._u])
        h = ctypes.c_void_p()
        _check(lib().cfx_batch_create(ctx.h, n, _hp(self.nCells), _hp(self.nFaces), la, ua, ctypes.byref(h)),
               "cfx_batch_create")
        self.h = h
        self.n = n
        self.sym = []
        _track("batch", self)
        for i, s in enumerate(systems):
            self.set_matrix(i, s["diag"], s["upper"], s.get("lower"))
        self.offsets = np.concatenate([[0], np.cumsum(self.nCells, dtype=np.int64)])

    def set_matrix(self, i, diag, upper, lower=None):
        d = np.ascontiguousarray(diag, np.float64)
        up = np.ascontiguousarray(upper, np.float64)
        lo = None if lower is None else np.ascontiguousarray(lower, np.float64)
        _check(lib().cfx_batch_set_matrix(self.h, int(i), _hp(d), _hp(up), _hp(lo)), "cfx_batch_set_matrix")
        if len(self.sym) <= i:
            self.sym.extend([True] * (i + 1 - len(self.sym)))
        self.sym[i] = lo is None

    def _c(self, controls):
        c = _controls(controls, all(self.sym))
        if not all(self.sym) and c.solver == SOLVER_PCG:
            raise FatalError("Unknown asymmetric matrix solver cudaPCG")
        return c

    def _perfs(self, arr, field):
        return [SolverPerformance(p.solverName.decode(), field, p.initialResidual, p.finalResidual, p.nIterations,
                                  bool(p.converged), bool(p.singular), p.nOuter) for p in arr]

    def solve(self, psi, source, controls, field="psi"):
        if psi.dtype != np.float64 or not psi.flags["C_CONTIGUOUS"] or psi.size != self.offsets[-1]:
            raise TypeError("psi must be a contiguous float64 array of sum(nCells)")
        src = np.ascontiguousarray(source, np.float64)
        arr = (Perf * self.n)()
        c = self._c(controls)
        _check(lib().cfx_batch_solve(self.h, ctypes.byref(c), _hp(psi), _hp(src), arr), "cfx_batch_solve")
        return self._perfs(arr, field)

    def vectors(self):
        p, b = ctypes.c_void_p(), ctypes.c_void_p()
        _check(lib().cfx_batch_vectors(self.h, ctypes.byref(p), ctypes.byref(b), None), "cfx_batch_vectors")
        return p.value, b.value

    def solve_device(self, controls, field="psi"):
        arr = (Perf * self.n)()
        c = self._c(controls)
        _check(lib().cfx_batch_solve_device(self.h, ctypes.byref(c), arr), "cfx_batch_solve_device")
        return self._perfs(arr, field)

    def timings(self):
        """(start, end) in ms of each system's solve in the last launch."""
        a = np.empty(self.n)
        b = np.empty(self.n)
        _check(lib().cfx_batch_timings(self.h, _hp(a), _hp(b)), "cfx_batch_timings")
        return a, b

    def set_ctas_per_sm(self, k):
        _check(lib().cfx_batch_set_ctas_per_sm(self.h, int(k)), "cfx_batch_set_ctas_per_sm")

    def set_groups(self, cluster_size, big_cells):
        _check(lib().cfx_batch_set_groups(self.h, int(cluster_size), int(big_cells)), "cfx_batch_set_groups")

    def groups(self):
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(lib().cfx_batch_get_groups(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)), "groups")
        return a.value, b.value, c.value

    def tune(self, controls):
        k, ms = ctypes.c_int(), ctypes.c_float()
        c = self._c(controls)
        _check(lib().cfx_batch_tune(self.h, ctypes.byref(c), ctypes.byref(k), ctypes.byref(ms)), "cfx_batch_tune")
        return k.value, ms.value

    def close(self):
        h, self.h = getattr(self, "h", None), None
        if h:
            lib().cfx_batch_destroy(h)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """The solve server (cfx_server_*): resident matrices, continuous batching,
    HBM admission.  ``add_matrix(system)`` registers a cases.py system dict
    (face weights from its Sf when large and ``gamg``); ``submit`` returns a
    request id; ``wait`` returns (psi, SolverPerformance).  Thread-safe: the
    ctypes calls release the GIL, so client threads submit and wait
    concurrently."""

    def __init__(self, ctx=None, **cfg):
        self.ctx = ctx or default_context()
        c = ServerConfig()
        lib().cfx_server_default_config(ctypes.byref(c))
        for k, v in cfg.items():
            setattr(c, k, int(v))
        self.config = c
        h = ctypes.c_void_p()
        _check(lib().cfx_server_create(self.ctx.h, ctypes.byref(c), ctypes.byref(h)), "cfx_server_create")
        self.h = h
        self._n = {}
        self._sym = {}
        _track("server", self)

    def add_matrix(self, s, gamg=False):
        l = np.ascontiguousarray(s["l"], np.int32)
        u = np.ascontiguousarray(s["u"], np.int32)
        d = np.ascontiguousarray(s["diag"], np.float64)
        up = np.ascontiguousarray(s["upper"], np.float64)
        lo = None if s.get("lower") is None else np.ascontiguousarray(s["lower"], np.float64)
        w = face_area_pair_weights(s["Sf"]) if gamg else None
        mid = ctypes.c_int64()
        _check(lib().cfx_server_add_matrix(self.h, d.size, l.size, _hp(l), _hp(u), _hp(d), _hp(up), _hp(lo), _hp(w),
                                           ctypes.byref(mid)), "cfx_server_add_matrix")
        self._n[mid.value] = d.size
        self._sym[mid.value] = lo is None
        return mid.value

    def remove_matrix(self, mid):
        _check(lib().cfx_server_remove_matrix(self.h, ctypes.c_int64(mid)), "cfx_server_remove_matrix")

    def submit(self, mid, source, controls, psi0=None):
        c = _controls(controls, self._sym[mid])
        src = np.ascontiguousarray(source, np.float64)
        p0 = None if psi0 is None else np.ascontiguousarray(psi0, np.float64)
        rid = ctypes.c_int64()
        _check(lib().cfx_server_submit(self.h, ctypes.c_int64(mid), ctypes.byref(c), _hp(p0), _hp(src),
                                       ctypes.byref(rid)), "cfx_server_submit")
        self._n[("r", rid.value)] = self._n[mid]
        return rid.value

    def wait(self, rid, timeout_ms=-1, field="psi"):
        n = self._n.pop(("r", rid), None)
        psi = np.empty(n if n is not None else 0)
        p = Perf()
        rc = lib().cfx_server_wait(self.h, ctypes.c_int64(rid), int(timeout_ms), _hp(psi) if n else None,
                                   ctypes.byref(p))
        if rc == -6 and n is not None:
            self._n[("r", rid)] = n
        _check(rc, "cfx_server_wait")
        return psi, SolverPerformance(p.solverName.decode(), field, p.initialResidual, p.finalResidual,
                                      p.nIterations, bool(p.converged), bool(p.singular), p.nOuter)

    def cancel(self, rid):
        _check(lib().cfx_server_cancel(self.h, ctypes.c_int64(rid)), "cfx_server_cancel")

    def release(self, rid):
        self._n.pop(("r", rid), None)
        _check(lib().cfx_server_release(self.h, ctypes.c_int64(rid)), "cfx_server_release")

    def stats(self):
        st = ServerStats()
        _check(lib().cfx_server_stats(self.h, ctypes.byref(st)), "cfx_server_stats")
        return st.as_dict()

    def metrics_json(self):
        """One JSON line of the server's metrics (solves/s, p50/p99, queue
        depth, HBM in use)."""
        import json
        return json.dumps(self.stats(), sort_keys=True)

    def reset_stats(self):
        _check(lib().cfx_server_reset_stats(self.h), "cfx_server_reset_stats")

    def close(self):
        h, self.h = getattr(self, "h", None), None
        if h:
            lib().cfx_server_destroy(h)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
