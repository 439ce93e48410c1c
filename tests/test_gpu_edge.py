"""Edge cases of the solver path against the oracle (the reference's
algorithms restated): one cell and no faces, cells without neighbours next
to connected ones, a zero source (converged at start), a negative-definite
matrix (fvm::laplacian with its own sign, as the pressure equation is
assembled), a two-cell system, and a mesh too small for any GAMG level.
"""
import numpy as np
import pytest

from oracle import oracle as orc
from openfoam_dev_gb300 import cases, ldu

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

KRYLOV = [("cudaPCG", "DIC", orc.pcg, "DIC"), ("cudaPBiCGStab", "DIC", orc.pbicgstab, "DIC"),
          ("cudaPCG", "diagonal", orc.pcg, "diagonal"), ("cudaPCG", "none", orc.pcg, "none")]


def _system(n, l, u, diag, upper, source):
    return dict(l=np.asarray(l, np.int32), u=np.asarray(u, np.int32), diag=np.asarray(diag, np.float64),
                upper=np.asarray(upper, np.float64), lower=None, source=np.asarray(source, np.float64))


def _chain_with_isolated(seed=3):
    """cells 0..5 in a chain, 6..9 with no faces at all"""
    rng = np.random.default_rng(seed)
    l, u = np.arange(5), np.arange(1, 6)
    upper = -rng.uniform(0.5, 1.0, 5)
    diag = rng.uniform(3.0, 4.0, 10)
    return _system(10, l, u, diag, upper, rng.uniform(-1, 1, 10))


CASES = {
    "one_cell": lambda: _system(1, [], [], [2.5], [], [1.0]),
    "two_cells": lambda: _system(2, [0], [1], [3.0, 2.0], [-1.0], [1.0, -2.0]),
    "chain_and_isolated": _chain_with_isolated,
}


def _solve(s, ctl):
    psi = np.zeros_like(s["source"])
    perf = ldu.solve(s, psi, ctl)
    return psi, perf


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("solver,pre,fn,opre", KRYLOV)
def test_small_and_disconnected_systems(case, solver, pre, fn, opre):
    s = CASES[case]()
    ref = np.zeros_like(s["source"])
    rp = fn(s, ref, tol=1e-12, precond=opre)
    psi, perf = _solve(s, {"solver": solver, "preconditioner": pre, "tolerance": 1e-12, "relTol": 0})
    assert perf.converged == rp.converged and abs(perf.nIterations - rp.nIterations) <= 1
    np.testing.assert_allclose(psi, ref, rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("case", sorted(CASES))
def test_smooth_solver_on_small_systems(case):
    s = CASES[case]()
    ref = np.zeros_like(s["source"])
    rp = orc.smooth_solve(s, ref, "symGaussSeidel", 1, tol=1e-12, max_iter=500)
    psi, perf = _solve(s, {"solver": "cudaSmoothSolver", "smoother": "symGaussSeidel", "tolerance": 1e-12,
                           "relTol": 0, "maxIter": 500})
    assert abs(perf.nIterations - rp.nIterations) <= 1
    np.testing.assert_allclose(psi, ref, rtol=1e-12, atol=1e-14)


def test_zero_source_is_converged_at_start():
    s = cases.pcg_cube(6, seed=2)
    s["source"] = np.zeros_like(s["source"])
    ref = np.zeros_like(s["source"])
    rp = orc.pcg(s, ref, tol=1e-6)
    psi, perf = _solve(s, {"solver": "cudaPCG", "preconditioner": "DIC", "tolerance": 1e-6})
    assert rp.nIterations == 0 and perf.nIterations == 0 and perf.converged
    assert perf.initialResidual == rp.initialResidual == 0.0
    assert np.all(psi == 0)


def test_negative_definite_pressure_type_matrix():
    """fvm::laplacian(rAU, p) keeps its own sign (negative diagonal,
    positive off-diagonals): PCG+DIC, GAMG and the mixed path solve it as
    the reference does."""
    s = cases.gamg_cube(12, jitter=0.2, seed=8)
    s["diag"], s["upper"] = -s["diag"], -s["upper"]
    ref = np.zeros_like(s["source"])
    rp = orc.pcg(s, ref, tol=1e-10, max_iter=2000)
    psi, perf = _solve(s, {"solver": "cudaPCG", "preconditioner": "DIC", "tolerance": 1e-10, "relTol": 0,
                           "maxIter": 2000})
    assert perf.converged and abs(perf.nIterations - rp.nIterations) <= 1
    np.testing.assert_allclose(psi, ref, rtol=1e-9, atol=1e-12)
    rg = np.zeros_like(s["source"])
    gp = orc.gamg(s, rg, tol=1e-10)
    s.pop("_cfx", None)
    psi, perf = _solve(s, {"solver": "cudaGAMG", "tolerance": 1e-10, "relTol": 0})
    assert perf.converged and abs(perf.nIterations - gp.nIterations) <= 1
    s.pop("_cfx", None)
    psi, perf = _solve(s, {"solver": "cudaGAMG", "tolerance": 1e-10, "relTol": 0, "precision": "mixed"})
    assert perf.converged


def test_gamg_without_coarse_levels_is_an_error():
    s = cases.pcg_cube(2, seed=1)  # 8 cells: no level below nCellsInCoarsestLevel 10
    with pytest.raises(ldu.CfxError) as e:
        _solve(s, {"solver": "cudaGAMG", "tolerance": 1e-8})
    assert e.value.status == -8
