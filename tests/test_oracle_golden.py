"""The C oracle against the reference's own outputs (golden fixtures).

The fixtures were produced by the reference code built from source
(tests/golden/make_golden.py); the oracle must reproduce them bit for bit:
same operation order, no FMA contraction.  This pins the oracle that every
GPU parity test compares against.
"""
import numpy as np
import pytest

from golden_cases import (CHECKSUMS, SPECS, checksum, fvcyc_case, fvcyc_names, fvm_case, fvm_names, fvsolve_case,
                          fvsolve_names, gamg_kwargs, load, matrix_digest, solve_case, system)
from oracle import oracle as orc
from openfoam_dev_gb300 import cases


def test_case_inputs_unchanged():
    for name, digest in CHECKSUMS.items():
        assert checksum(system(name)) == digest, name


def test_geometry_matches_polymesh():
    g = load("geom_box567.npz")
    m = cases.box_mesh(int(g["nx"]), int(g["ny"]), int(g["nz"]), jitter=float(g["jitter"]), seed=int(g["seed"]))
    for k in ("Sf", "Cf", "magSf", "C", "V"):
        np.testing.assert_array_equal(m[k], g[k], err_msg=k)


@pytest.mark.parametrize("name", ["cube6", "jcube7", "cd6", "box", "cyc7", "cycd7"])
def test_single_operations(name):
    s = system(name)
    g = load(f"ops_{name}.npz")
    m = orc.Matrix(s)
    x, b = g["x"], s["source"]
    os_, lo, ls = m.addr()
    np.testing.assert_array_equal(os_, g["ownerStart"])
    np.testing.assert_array_equal(lo, g["losort"])
    np.testing.assert_array_equal(ls, g["losortStart"])
    np.testing.assert_array_equal(m.amul(x), g["Amul"])
    np.testing.assert_array_equal(m.tmul(x), g["Tmul"])
    np.testing.assert_array_equal(m.residual(x, b), g["residual"])
    np.testing.assert_array_equal(m.sumA(), g["sumA"])
    assert m.norm_factor(x, b) == g["normFactor"][0]
    L = orc.lib()
    bp = b.ctypes.data_as(orc.f64p)
    xp = x.ctypes.data_as(orc.f64p)
    assert L.ldu_sum_mag(b.size, bp) == g["sumMag"][0]
    assert L.ldu_sum_prod(b.size, xp, bp) == g["sumProd"][0]
    assert L.ldu_sum_sqr(b.size, bp) == g["sumSqr"][0]
    assert L.ldu_sum(b.size, bp) == g["sum"][0]
    assert L.ldu_average(x.size, xp) == g["average"][0]
    if s.get("lower") is None:
        np.testing.assert_array_equal(m.dic_rD(), g["DIC_rD"])
        np.testing.assert_array_equal(m.dic_precondition(b), g["DIC_precondition"])
        np.testing.assert_array_equal(m.dic_smooth(x, b, 2), g["DIC_smooth2"])
    else:
        np.testing.assert_array_equal(m.dilu_rD(), g["DILU_rD"])
        np.testing.assert_array_equal(m.dilu_precondition(b), g["DILU_precondition"])
        np.testing.assert_array_equal(m.dilu_preconditionT(b), g["DILU_preconditionT"])
    np.testing.assert_array_equal(m.gs_smooth(x, b, 1), g["GS_smooth1"])
    np.testing.assert_array_equal(m.gs_smooth(x, b, 3), g["GS_smooth3"])
    others = ("symGaussSeidel", "DICGaussSeidel") if s.get("lower") is None else \
        ("symGaussSeidel", "DILU", "DILUGaussSeidel")
    for sm in others:
        np.testing.assert_array_equal(m.smooth(sm, x, b, 2), g[f"{sm}_smooth2"], err_msg=sm)


def _run_oracle(s, ctl, psi0=None):
    psi = np.zeros_like(s["source"]) if psi0 is None else np.array(psi0, np.float64)
    kw = dict(tol=ctl.get("tolerance", 1e-6), rel_tol=ctl.get("relTol", 0.0), max_iter=ctl.get("maxIter", 1000),
              min_iter=ctl.get("minIter", 0))
    pre = ctl.get("preconditioner")
    if ctl["solver"] == "PCG" and isinstance(pre, dict):
        p = orc.pcg_gamg(s, psi, nVcycles=pre.get("nVcycles", 2), pre_tol=pre.get("tolerance", 1e-6),
                         pre_rel_tol=pre.get("relTol", 0.0), **kw, **gamg_kwargs(pre))
    elif ctl["solver"] == "PCG":
        p = orc.pcg(s, psi, precond=ctl["preconditioner"], **kw)
    elif ctl["solver"] == "PBiCG":
        p = orc.pbicg(s, psi, precond=ctl["preconditioner"], **kw)
    elif ctl["solver"] == "PBiCGStab":
        p = orc.pbicgstab(s, psi, precond=ctl["preconditioner"], **kw)
    elif ctl["solver"] == "smoothSolver":
        p = orc.smooth_solve(s, psi, ctl["smoother"], ctl.get("nSweeps", 1), **kw)
    else:
        p = orc.gamg(s, psi, **kw, **gamg_kwargs(ctl))
    return psi, p


@pytest.mark.parametrize("name", sorted(SPECS["solves"]))
def test_solvers_bit_exact(name):
    s, ctl, g = solve_case(name)
    psi, p = _run_oracle(s, ctl)
    np.testing.assert_array_equal(psi, g["psi"])
    assert p.nIterations == g["nIterations"][0]
    assert p.initialResidual == g["initialResidual"][0]
    assert p.finalResidual == g["finalResidual"][0]
    assert p.converged == bool(g["converged"][0])
    assert p.singular == bool(g["singular"][0])


@pytest.mark.parametrize("name", [n for n, (_, c) in sorted(SPECS["solves"].items()) if c["solver"] == "GAMG"])
def test_agglomeration_and_coarse_matrices(name):
    s, ctl, g = solve_case(name)
    agg = orc.Agglomeration(s, n_coarsest=ctl.get("nCellsInCoarsestLevel", 10))
    assert agg.n_levels == g["nLevels"][0]
    fine = s
    for i in range(agg.n_levels):
        ra, fra, flip, nc, ncf, cl, cu = agg.level(i)
        np.testing.assert_array_equal(ra, g[f"restrict{i}"])
        np.testing.assert_array_equal(fra, g[f"faceRestrict{i}"])
        np.testing.assert_array_equal(flip, g[f"faceFlip{i}"])
        np.testing.assert_array_equal(cl, g[f"coarseL{i}"])
        np.testing.assert_array_equal(cu, g[f"coarseU{i}"])
        assert nc == g[f"nCells{i}"][0] and ncf == g[f"nFaces{i}"][0]
        cd, cup, clo = orc.coarse_matrix(fine, agg, i)
        np.testing.assert_array_equal(cd, g[f"coarseDiag{i}"])
        np.testing.assert_array_equal(cup, g[f"coarseUpper{i}"])
        fine = dict(l=cl, u=cu, diag=cd, upper=cup, lower=clo)


def test_lu_restatement_solves_and_detects_singular_rows():
    """The oracle's LUscalarMatrix (pinned bit for bit by the golden
    directSolveCoarsest solves) solves a pivoting-heavy dense system to
    rounding and refuses an all-zero row like LUDecompose."""
    rng = np.random.default_rng(3)
    A = rng.uniform(-1, 1, (40, 40))
    A[np.arange(40), np.arange(40)] *= 1e-3  # small diagonals force row interchanges
    b = rng.uniform(-1, 1, 40)
    x, _, piv = orc.lu_solve(A, b)
    assert np.any(piv != np.arange(40))
    np.testing.assert_allclose(A @ x, b, rtol=0, atol=1e-10)
    A[7, :] = 0.0
    with pytest.raises(ValueError, match="Singular matrix"):
        orc.lu_solve(A, b)


@pytest.mark.parametrize("name", fvm_names())
def test_fvm_assembly_bit_exact(name):
    """fvm::ddt + fvm::div +/- fvm::laplacian == su as the reference's
    finiteVolume library assembles it (fixedValue, zeroGradient and
    fixedGradient patches; upwind and linear; face and uniform diffusivity)
    and as the oracle restates it, from the same geometry: diag, upper,
    lower and source equal bit for bit."""
    l, u, geom, terms, ref = fvm_case(name)
    d, up, lo, src = orc.fvm_assemble(l, u, geom, **terms)
    np.testing.assert_array_equal(d, ref["diag"])
    np.testing.assert_array_equal(up, ref["upper"])
    assert (lo is None) == (ref["lower"] is None)
    if lo is not None:
        np.testing.assert_array_equal(lo, ref["lower"])
    np.testing.assert_array_equal(src, ref["source"])


@pytest.mark.skipif(not fvm_names(), reason="no fvm fixtures")
def test_fv_geometry_matches_surface_interpolation():
    """cases.fv_geometry (the geometry handed to the device assembly)
    against the reference's surfaceInterpolation and fvPatch on the same
    mesh, bit for bit: magSf, nonOrthDeltaCoeffs, weights, V and the
    boundary faces' cells, magSf and deltaCoeffs."""
    _, _, geom, _, _ = fvm_case(fvm_names()[0])
    g = cases.fv_geometry(cases.box_mesh(**SPECS["fvm"]["mesh"]))
    for k in geom:
        np.testing.assert_array_equal(g[k], geom[k], err_msg=k)


def _fvsolve_system(name):
    m, terms, ctl, g = fvsolve_case(name)
    nI = m["nInternalFaces"]
    d, up, lo, src = orc.fvm_assemble(m["owner"][:nI], m["neighbour"], cases.fv_geometry(m), **terms)
    s = dict(l=m["owner"][:nI], u=m["neighbour"], diag=d, upper=up, lower=lo, source=src, Sf=m["Sf_internal"])
    return s, terms, ctl, g


@pytest.mark.parametrize("name", fvsolve_names())
def test_fvmatrix_solve_bit_exact(name):
    """The equation as a solver application solves it (fvMatrix::solve on
    the fvMesh, GAMG agglomerating with faceAreaPair from the mesh's own Sf):
    the oracle's assembly from cases.fv_geometry gives the reference's
    matrix (digest), its faceAreaPair levels and its solve give the
    reference's psi, iteration count and residuals bit for bit."""
    s, terms, ctl, g = _fvsolve_system(name)
    assert matrix_digest(s["diag"], s["upper"], s["lower"], s["source"]) == g["matrixDigest"]
    if "nLevels" in g:
        pre = ctl.get("preconditioner")
        gctl = pre if isinstance(pre, dict) else ctl
        agg = orc.Agglomeration(s, n_coarsest=gctl.get("nCellsInCoarsestLevel", 10))
        assert agg.n_levels == g["nLevels"][0]
        for i in range(agg.n_levels):
            ra, fra, flip, nc, _, _, _ = agg.level(i)
            np.testing.assert_array_equal(ra, g[f"restrict{i}"])
            np.testing.assert_array_equal(fra, g[f"faceRestrict{i}"])
            np.testing.assert_array_equal(flip, g[f"faceFlip{i}"])
            assert nc == g[f"nCells{i}"][0]
    start = terms.get("psi0")
    psi, p = _run_oracle(s, ctl, psi0=start)
    np.testing.assert_array_equal(psi, g["psi"])
    assert p.nIterations == g["nIterations"][0]
    assert p.initialResidual == g["initialResidual"][0]
    assert p.finalResidual == g["finalResidual"][0]
    assert p.converged == bool(g["converged"][0])


@pytest.mark.parametrize("name", fvcyc_names())
def test_cyclic_fvmatrix_solve_bit_exact(name):
    """The reference's own cyclicPolyPatch / cyclicFvPatchField on an
    x-periodic box: from the lduMatrix and interfaces its fvMatrix handed to
    the solver (interfaceBouCoeffs = boundaryCoeffs, interfaceIntCoeffs =
    internalCoeffs), the oracle's PCG, PBiCGStab, PBiCG, smoothSolver and
    GAMG (its cyclicGAMGInterface levels restated) reproduce psi, iterations
    and residuals bit for bit, and GAMG's levels."""
    s, psi0, ctl, g = fvcyc_case(name)
    if "nLevels" in g:
        agg = orc.Agglomeration(s, n_coarsest=ctl.get("nCellsInCoarsestLevel", 10))
        assert agg.n_levels == g["nLevels"][0]
        for i in range(agg.n_levels):
            ra, fra, flip, nc, _, _, _ = agg.level(i)
            np.testing.assert_array_equal(ra, g[f"restrict{i}"])
            np.testing.assert_array_equal(fra, g[f"faceRestrict{i}"])
    psi, p = _run_oracle(s, ctl, psi0=psi0)
    np.testing.assert_array_equal(psi, g["psi"])
    assert p.nIterations == g["nIterations"][0]
    assert p.initialResidual == g["initialResidual"][0]
    assert p.finalResidual == g["finalResidual"][0]
    assert p.converged == bool(g["converged"][0])


_TIMED_CHILD = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
import __graft_entry__ as ge
ge.load_package()
from openfoam_dev_gb300 import cases
from oracle import oracle as orc
s = cases.gamg_cube(12, jitter=0.2, seed=4)
psi = np.zeros_like(s["source"])
p = orc.gamg(s, psi, tol=1e-10, rel_tol=0.0, smoother="GaussSeidel", nPreSweeps=2, nPostSweeps=2)
t = cases.bicgstab_cube(10, seed=2)
x = np.zeros_like(t["source"])
q = orc.pbicgstab(t, x, tol=1e-10, precond="DILU")
np.save(sys.argv[2], np.concatenate([psi, x, [p.nIterations, q.nIterations]]))
"""


def test_timed_oracle_build_is_bit_identical(tmp_path):
    """The oracle built with the reference's optimisation flags (the one the
    bench times) gives the same bits as the build the tests pin."""
    import os
    import subprocess
    import sys
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = {}
    for timed in ("0", "1"):
        f = str(tmp_path / f"r{timed}.npy")
        env = dict(os.environ, CFX_ORACLE_TIMED=timed)
        subprocess.run([sys.executable, "-c", _TIMED_CHILD, repo, f], env=env, check=True)
        out[timed] = np.load(f)
    np.testing.assert_array_equal(out["0"], out["1"])


@pytest.mark.parametrize("U", [None, (1.0, 0.3, 0.0)], ids=["laplacian", "upwind"])
def test_direct_coarsest_with_interfaces(U):
    """LUscalarMatrix::convert with cyclic interfaces (LUscalarMatrix.C:236-262)
    in the oracle: it needs each patch's partner patch, and the GAMG solve
    with the direct coarsest solve reaches the iterative coarsest solve's
    answer."""
    s = cases.cyclic_cube(12, jitter=0.2, seed=4, U=U)
    a = np.zeros_like(s["source"])
    pa = orc.gamg(s, a, tol=1e-9, directSolveCoarsest=True)
    b = np.zeros_like(s["source"])
    orc.gamg(s, b, tol=1e-9)
    assert pa.converged
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-8
    t = dict(s)
    t.pop("ifNbrPatch")
    with pytest.raises(ValueError, match="partner"):
        orc.gamg(t, np.zeros_like(s["source"]), tol=1e-9, directSolveCoarsest=True)


@pytest.mark.parametrize("name", fvcyc_names())
def test_cyclic_fvmatrix_assembly_bit_exact(name):
    """The reference's assembly with a cyclicFvPatchField pair
    (coupledFvPatchField's value and gradient coefficients; addBoundaryDiag
    over every patch, addBoundarySource over the uncoupled ones): the
    oracle reproduces the lduMatrix, the source and the interfaceBouCoeffs /
    interfaceIntCoeffs the solver received, bit for bit."""
    from golden_cases import fvcyc_assembly_case
    l, u, geom, terms, ref = fvcyc_assembly_case(name)
    d, up, lo, src, ib, ii = orc.fvm_assemble(l, u, geom, coupled=True, **terms)
    np.testing.assert_array_equal(d, ref["diag"])
    np.testing.assert_array_equal(up, ref["upper"])
    if ref["lower"] is not None:
        np.testing.assert_array_equal(lo, ref["lower"])
    np.testing.assert_array_equal(src, ref["source"])
    np.testing.assert_array_equal(ib, ref["ifBou"])
    np.testing.assert_array_equal(ii, ref["ifInt"])
