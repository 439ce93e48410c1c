"""Device-side assembly and solve against the reference's fvMatrix itself.

This file sorts last: its fixtures and its cyclic GAMG and mixed-precision
cases are the newest GPU checks, so a run stopping at the first failure has
run every other test first.

The fixtures come from the reference's own finiteVolume library
(tests/golden/make_golden.py, oracle/fv_harness.C):

* fvm_*.npz: fvm::ddt + fvm::div +/- fvm::laplacian == su on a jittered
  7x6x5 box with fixedValue, zeroGradient and fixedGradient patches.
  cfx_fvm_assemble, given the geometry the reference's schemes used, writes
  the same diag, upper, lower and source bit for bit.
* fvsolve_*.npz: fvMatrix::solve of those equations on a 14x12x10 box (GAMG
  agglomerating with faceAreaPair from the fvMesh, PCG with the GAMG
  preconditioner, PCG+DIC, PBiCGStab+DILU, smoothSolver).  Assembling on the
  device from cases.fv_geometry (equal to the reference's geometry bit for
  bit) gives the same matrix (digest); solving it gives the solution within
  relative L2 1e-10 and the iteration count within +-1 (PBiCGStab: within
  10 % and 4; its per-iteration reductions are summed in another order).
* fvcyc_*.npz: fvMatrix::solve on an x-periodic box with the reference's
  own cyclic patches.  The lduMatrix and interfaces the reference's solver
  received, solved through the plugin solvers with coupled interfaces (GAMG
  with its cyclicGAMGInterface levels included), give the reference's psi
  within the same bounds.
GAMG and the GAMG preconditioner with cyclic interfaces also follow the
oracle on a 16^3 periodic cube; directSolveCoarsest with interfaces is
refused.  Mixed precision (FP32 inner solves, FP64 refinement) with
interfaces reaches the FP64 tolerance by the oracle's FP64 residual and
stays within relative L2 1e-6 of the FP64 solution.
"""
import numpy as np
import pytest

from golden_cases import SPECS, fvcyc_case, fvcyc_names, fvm_case, fvm_names, fvsolve_case, fvsolve_names, matrix_digest
from oracle import oracle as orc
from golden_cases import gamg_kwargs
from openfoam_dev_gb300 import cases, ldu

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

_PLUGIN_NAMES = {"PCG": "cudaPCG", "PBiCGStab": "cudaPBiCGStab", "GAMG": "cudaGAMG",
                 "smoothSolver": "cudaSmoothSolver", "PBiCG": "cudaPBiCG"}


def _dev(a, dtype=torch.float64):
    return None if a is None else torch.as_tensor(np.ascontiguousarray(a), device="cuda").to(dtype)


def _dev_terms(terms):
    return {k: (_dev(v, torch.int32 if k == "bcType" else torch.float64) if isinstance(v, np.ndarray) else v)
            for k, v in terms.items()}


def _mesh(n, l, u, geom):
    mesh = ldu.LduMesh(ldu.default_context(), n, l, u)
    mesh.fv_geometry(geom["magSf"], geom["deltaCoeffs"], geom["V"], geom["bCell"], geom["magSfB"],
                     geom["deltaCoeffsB"], weights=geom["weights"])
    return mesh


@pytest.mark.parametrize("name", fvm_names())
def test_assembly_bit_exact_against_the_reference(name):
    l, u, geom, terms, ref = fvm_case(name)
    n = geom["V"].size
    A = ldu.LduMatrix.empty(_mesh(n, l, u, geom), symmetric=ref["lower"] is None)
    source = torch.empty(n, dtype=torch.float64, device="cuda")
    A.assemble(source, **_dev_terms(terms))
    torch.cuda.synchronize()
    got_d, got_u, got_l = A.coarse(0, n, l.size)
    np.testing.assert_array_equal(got_d, ref["diag"])
    np.testing.assert_array_equal(got_u, ref["upper"])
    if ref["lower"] is not None:
        np.testing.assert_array_equal(got_l, ref["lower"])
    np.testing.assert_array_equal(source.cpu().numpy(), ref["source"])


@pytest.mark.parametrize("name", fvsolve_names())
def test_assemble_and_solve_match_fvmatrix_solve(name):
    m, terms, ctl, g = fvsolve_case(name)
    nI, n = m["nInternalFaces"], m["nCells"]
    mesh = _mesh(n, m["owner"][:nI], m["neighbour"], cases.fv_geometry(m))
    asym = "phi" in terms
    A = ldu.LduMatrix.empty(mesh, symmetric=not asym)
    source = torch.empty(n, dtype=torch.float64, device="cuda")
    A.assemble(source, **_dev_terms(terms))
    torch.cuda.synchronize()
    d, up, lo = A.coarse(0, n, nI)
    b = source.cpu().numpy()
    assert matrix_digest(d, up, lo if asym else None, b) == g["matrixDigest"]
    pre = ctl.get("preconditioner")
    gd = pre if isinstance(pre, dict) else (ctl if ctl["solver"] == "GAMG" else None)
    if gd is not None:
        mesh.agglomerate(Sf=m["Sf_internal"], nCellsInCoarsestLevel=gd.get("nCellsInCoarsestLevel", 10))
    start = terms["psi0"] if "psi0" in terms else np.zeros(n)
    psi = _dev(start)
    perf = ldu.solver_new("T", A, dict(ctl, solver=_PLUGIN_NAMES[ctl["solver"]])).solve(psi, source)
    torch.cuda.synchronize()
    ref_it = int(g["nIterations"][0])
    assert perf.solverName == g["solverName"]
    assert perf.converged == bool(g["converged"][0])
    assert perf.initialResidual == pytest.approx(float(g["initialResidual"][0]), rel=1e-12)
    x, xr = psi.cpu().numpy(), g["psi"]
    rel = float(np.linalg.norm(x - xr) / np.linalg.norm(xr))
    if ctl["solver"] == "PBiCGStab":
        assert abs(perf.nIterations - ref_it) <= max(4, ref_it // 10), (perf, ref_it)
    else:
        assert abs(perf.nIterations - ref_it) <= 1, (perf, ref_it)
    if perf.nIterations == ref_it and ctl["solver"] != "PBiCGStab":
        assert rel <= 1e-10, rel
    else:
        # another iteration count: ours meets the tolerance by the oracle's
        # FP64 residual, normalised as the solver does (normFactor of the
        # starting psi)
        om = orc.Matrix(dict(l=m["owner"][:nI], u=m["neighbour"], diag=d, upper=up, lower=lo if asym else None))
        nf = om.norm_factor(start, b)
        assert np.abs(om.residual(x, b)).sum() / nf < 1.5 * ctl["tolerance"]
        assert rel <= 1e-6, rel


def _check_against(perf, x, g, ctl, om, b, start):
    ref_it = int(g["nIterations"][0])
    assert perf.solverName == g["solverName"]
    assert perf.converged == bool(g["converged"][0])
    assert perf.initialResidual == pytest.approx(float(g["initialResidual"][0]), rel=1e-12)
    rel = float(np.linalg.norm(x - g["psi"]) / np.linalg.norm(g["psi"]))
    krylov_bicg = ctl["solver"] in ("PBiCGStab", "PBiCG")
    if krylov_bicg:
        assert abs(perf.nIterations - ref_it) <= max(4, ref_it // 10), (perf, ref_it)
    else:
        assert abs(perf.nIterations - ref_it) <= 1, (perf, ref_it)
    if perf.nIterations == ref_it and not krylov_bicg:
        assert rel <= 1e-10, rel
    else:
        r = om.residual(x, b)
        assert np.abs(r).sum() / om.norm_factor(start, b) < 1.5 * ctl["tolerance"]
        assert rel <= 1e-6, rel


@pytest.mark.parametrize("name", fvcyc_names())
def test_cyclic_solve_matches_fvmatrix_solve(name):
    s, psi0, ctl, g = fvcyc_case(name)
    start = np.zeros_like(s["source"]) if psi0 is None else np.array(psi0)
    x = start.copy()
    perf = ldu.solve(s, x, dict(ctl, solver=_PLUGIN_NAMES[ctl["solver"]]))
    _check_against(perf, x, g, ctl, orc.Matrix(s), s["source"], start)


@pytest.mark.parametrize("ctl", [
    dict(solver="GAMG", smoother="GaussSeidel", tolerance=1e-9, relTol=0.0),
    dict(solver="GAMG", smoother="DIC", nPreSweeps=1, interpolateCorrection=True, tolerance=1e-9, relTol=0.0),
    dict(solver="PCG", tolerance=1e-9, relTol=0.0,
         preconditioner=dict(preconditioner="GAMG", smoother="symGaussSeidel")),
], ids=["gamg_gs", "gamg_dic_interp", "pcg_gamg"])
def test_gamg_with_cyclic_interfaces_against_the_oracle(ctl):
    s = cases.cyclic_cube(16, jitter=0.2, seed=4)
    ref = np.zeros_like(s["source"])
    pre = ctl.get("preconditioner")
    if ctl["solver"] == "GAMG":
        rp = orc.gamg(s, ref, tol=ctl["tolerance"], **gamg_kwargs(ctl))
    else:
        rp = orc.pcg_gamg(s, ref, tol=ctl["tolerance"], **gamg_kwargs(pre))
    psi = np.zeros_like(s["source"])
    perf = ldu.solve(s, psi, dict(ctl, solver=_PLUGIN_NAMES[ctl["solver"]]))
    assert perf.converged and abs(perf.nIterations - rp.nIterations) <= 1, (perf, rp)
    rel = float(np.linalg.norm(psi - ref) / np.linalg.norm(ref))
    if perf.nIterations == rp.nIterations:
        assert rel <= 1e-10, rel
    else:
        assert rel <= 1e-6, rel


def test_direct_coarsest_solve_with_interfaces_needs_the_partner_patches():
    s = cases.cyclic_cube(8, jitter=0.2, seed=2)
    s.pop("ifNbrPatch")
    with pytest.raises(ldu.FatalError, match="directSolveCoarsest"):
        ldu.solve(s, np.zeros_like(s["source"]), {"solver": "cudaGAMG", "directSolveCoarsest": True})


@pytest.mark.parametrize("U", [None, (1.0, 0.3, 0.0)], ids=["laplacian", "upwind"])
def test_direct_coarsest_solve_with_interfaces_against_the_oracle(U):
    """LUscalarMatrix::convert with cyclic interfaces: the coarsest level's
    dense matrix takes each patch's faces with the partner patch's
    coefficients (LUscalarMatrix.C:236-262), on the device as in the
    oracle."""
    s = cases.cyclic_cube(16, jitter=0.2, seed=4, U=U)
    ctl = dict(solver="GAMG", smoother="GaussSeidel", directSolveCoarsest=True, tolerance=1e-9, relTol=0.0)
    ref = np.zeros_like(s["source"])
    rp = orc.gamg(s, ref, tol=ctl["tolerance"], **gamg_kwargs(ctl))
    psi = np.zeros_like(s["source"])
    perf = ldu.solve(s, psi, dict(ctl, solver="cudaGAMG"))
    assert perf.converged and abs(perf.nIterations - rp.nIterations) <= 1, (perf, rp)
    rel = float(np.linalg.norm(psi - ref) / np.linalg.norm(ref))
    assert rel <= (1e-10 if perf.nIterations == rp.nIterations else 1e-6), rel


@pytest.mark.parametrize("ctl", [
    {"solver": "cudaPCG", "preconditioner": "DIC"},
    {"solver": "cudaPBiCGStab", "preconditioner": "DIC"},
    {"solver": "cudaGAMG", "smoother": "GaussSeidel"},
], ids=["pcg", "pbicgstab", "gamg"])
def test_mixed_precision_with_cyclic_interfaces(ctl):
    s = cases.cyclic_cube(16, jitter=0.2, seed=4)
    ref = np.zeros_like(s["source"])
    orc.pcg(s, ref, tol=1e-12, max_iter=5000)
    psi = np.zeros_like(s["source"])
    perf = ldu.solve(s, psi, dict(ctl, tolerance=1e-8, relTol=0.0, precision="mixed"))
    assert perf.converged
    om = orc.Matrix(s)
    nf = om.norm_factor(np.zeros_like(psi), s["source"])
    assert np.abs(om.residual(psi, s["source"])).sum() / nf < 1.5e-8
    assert float(np.linalg.norm(psi - ref) / np.linalg.norm(ref)) <= 1e-6
