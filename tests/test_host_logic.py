"""Host-side logic that needs no GPU: the C ABI's exports, control parsing
with the reference's error behaviour, and the case generator's invariants."""
import ctypes
import os
import re

import numpy as np
import pytest

from oracle import oracle as orc
from openfoam_dev_gb300 import INCLUDE_DIR, cases, ldu


def _declared_symbols():
    with open(os.path.join(INCLUDE_DIR, "cfx.h")) as fh:
        text = fh.read()
    return sorted(set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(cfx_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(ldu.LIB_PATH)
    declared = _declared_symbols()
    assert len(declared) >= 30
    for name in declared:
        assert hasattr(lib, name), name
    assert sorted(ldu.exported_symbols()) == declared


def test_default_controls_are_the_reference_defaults():
    c = ldu.Controls()
    ldu.lib().cfx_default_controls(ctypes.byref(c))
    # lduMatrixSolver.C:158-164, lduMatrix.C:38, GAMGSolver.C:70-80, GAMGAgglomeration.C:250-257
    assert (c.tolerance, c.relTol, c.maxIter, c.minIter) == (1e-6, 0.0, 1000, 0)
    assert (c.nPreSweeps, c.preSweepsLevelMultiplier, c.maxPreSweeps) == (0, 1, 4)
    assert (c.nPostSweeps, c.postSweepsLevelMultiplier, c.maxPostSweeps, c.nFinestSweeps) == (2, 1, 4, 2)
    assert c.scaleCorrection == -1 and c.nCellsInCoarsestLevel == 10


class _FakeMatrix:
    def __init__(self, sym):
        self.lower = None if sym else np.zeros(1)

    def symmetric(self):
        return self.lower is None


def test_unknown_solver_is_fatal_like_the_reference():
    with pytest.raises(ldu.FatalError, match="Unknown symmetric matrix solver PBiCG"):
        ldu.solver_new("p", _FakeMatrix(True), {"solver": "PBiCG"})
    with pytest.raises(ldu.FatalError, match="Unknown asymmetric matrix solver cudaPCG"):
        ldu.solver_new("U", _FakeMatrix(False), {"solver": "cudaPCG", "preconditioner": "DILU"})
    with pytest.raises(ldu.FatalError, match="keyword solver is undefined"):
        ldu.solver_new("p", _FakeMatrix(True), {"tolerance": 1e-6})
    with pytest.raises(ldu.FatalError, match="preconditioner"):
        ldu.solver_new("p", _FakeMatrix(True), {"solver": "cudaPCG", "preconditioner": "ILU0"})
    with pytest.raises(ldu.FatalError, match="smoother"):
        ldu.solver_new("p", _FakeMatrix(True), {"solver": "cudaGAMG", "smoother": "DILU"})
    with pytest.raises(ldu.FatalError, match="Unknown asymmetric matrix smoother DICGaussSeidel"):
        ldu.solver_new("U", _FakeMatrix(False), {"solver": "cudaSmoothSolver", "smoother": "DICGaussSeidel"})
    with pytest.raises(ldu.FatalError, match="GAMGAgglomeration"):
        ldu.solver_new("p", _FakeMatrix(True), {"solver": "cudaGAMG", "agglomerator": "algebraicPair"})


class _FakeDiagonal:
    def diagonal(self):
        return True

    def symmetric(self):
        return False


def test_diagonal_matrix_selects_diagonal_solver_before_the_name():
    """lduMatrix::solver::New (lduMatrixSolver.C:52-66): a diagonal matrix
    gets diagonalSolver whatever the solver name; the keyword must exist."""
    s = ldu.solver_new("p", _FakeDiagonal(), {"solver": "PBiCG", "preconditioner": "ILU0"})
    assert s.c.solver == ldu.SOLVER_PCG  # unused: the library solves psi = source/diag
    with pytest.raises(ldu.FatalError, match="keyword solver is undefined"):
        ldu.solver_new("p", _FakeDiagonal(), {"tolerance": 1e-6})


def test_smooth_solver_controls_parse():
    s = ldu.solver_new("p", _FakeMatrix(True), {"solver": "cudaSmoothSolver", "smoother": "symGaussSeidel",
                                                "nSweeps": 2, "tolerance": 1e-7})
    assert s.c.solver == ldu.SOLVER_SMOOTH and s.c.smoother == 2 and s.c.nSweeps == 2
    s = ldu.solver_new("U", _FakeMatrix(False), {"solver": "smoothSolver", "smoother": "DILUGaussSeidel"})
    assert s.c.smoother == 5 and s.c.nSweeps == 1


def test_controls_parse():
    s = ldu.solver_new("p", _FakeMatrix(True), {"solver": "cudaGAMG", "tolerance": 1e-8, "relTol": 0.01,
                                                "nPreSweeps": 2, "smoother": "DIC", "precision": "mixed",
                                                "minCellsPerProcessor": 20})
    c = s.c
    assert c.solver == ldu.SOLVER_GAMG and c.tolerance == 1e-8 and c.relTol == 0.01
    assert c.nPreSweeps == 2 and c.smoother == 1 and c.precision == 1 and c.nCellsInCoarsestLevel == 20


def test_gamg_preconditioner_controls_parse():
    """The GAMG preconditioner's keys come from its own dictionary
    (GAMGPreconditioner.C:40-79): nVcycles (default 2), its tolerance
    (default 1e-6) and relTol, the smoother and sweeps; the solver's own
    tolerance stays the outer one."""
    s = ldu.solver_new("p", _FakeMatrix(True), {
        "solver": "cudaPCG", "tolerance": 1e-9, "nPreSweeps": 3,
        "preconditioner": {"preconditioner": "GAMG", "smoother": "DICGaussSeidel", "nPreSweeps": 1,
                           "tolerance": 1e-4, "nVcycles": 1}})
    c = s.c
    assert c.preconditioner == ldu.PRECONDITIONERS["GAMG"] and c.tolerance == 1e-9
    assert (c.pcTolerance, c.pcRelTol, c.nVcycles, c.smoother, c.nPreSweeps) == (1e-4, 0.0, 1, 4, 1)
    c = ldu.solver_new("p", _FakeMatrix(True), {"solver": "cudaPCG",
                                                "preconditioner": {"preconditioner": "GAMG"}}).c
    assert (c.pcTolerance, c.nVcycles, c.smoother) == (1e-6, 2, 0)
    # the word form has no dictionary for the GAMG keys (the reference
    # constructs GAMGPreconditioner from an empty one): refused here
    with pytest.raises(ldu.FatalError, match="preconditioner GAMG"):
        ldu.solver_new("p", _FakeMatrix(True), {"solver": "cudaPCG", "preconditioner": "GAMG"})


def test_solver_performance_print_format():
    p = ldu.SolverPerformance("DICPCG", "T", 1.0, 5e-9, 32, True, False)
    assert str(p) == "DICPCG:  Solving for T, Initial residual = 1, Final residual = 5e-09, No Iterations 32"
    p.singular = True
    assert str(p) == "DICPCG:  Solving for T:  solution singularity"


def test_weights_match_oracle():
    s = cases.gamg_cube(9, jitter=0.3, seed=4)
    np.testing.assert_array_equal(ldu.face_area_pair_weights(s["Sf"]), orc.face_area_pair_weights(s["Sf"]))


def test_renumbering_keeps_upper_triangular_order_and_operator():
    s = cases.bicgstab_cube(7, seed=3)
    l, u = s["l"], s["u"]
    assert np.all(l < u)
    assert np.all(np.diff(l) >= 0)
    same = np.diff(l) == 0
    assert np.all(np.diff(u)[same] > 0)
    # the renumbered operator is a permutation of the original one
    s0 = cases.convection_diffusion(cases.box_mesh(7, 7, 7, jitter=0.2, seed=3), s["U"], 1e-3)
    order = cases.random_order(3 + 7, s0["diag"].size)
    s1 = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in s0.items()}
    cases.renumber(s1, order)
    x = np.random.default_rng(0).uniform(-1, 1, s0["diag"].size)
    y0 = orc.Matrix(s0).amul(x)
    y1 = orc.Matrix(s1).amul(x[order])
    np.testing.assert_allclose(y1, y0[order], rtol=0, atol=1e-14)


def test_cuthill_mckee_is_a_permutation_and_reduces_bandwidth():
    s = cases.convection_diffusion(cases.box_mesh(6, 6, 6, seed=1), [1.0, 0.0, 0.0], 1e-3)
    cases.renumber(s, cases.random_order(5, s["diag"].size))
    bw0 = int(np.max(s["u"] - s["l"]))
    order = cases.cuthill_mckee(s)
    assert np.array_equal(np.sort(order), np.arange(s["diag"].size))
    cases.renumber(s, order)
    assert int(np.max(s["u"] - s["l"])) < bw0


def test_batch_box_shapes_log_uniform():
    boxes = cases.batch_boxes(64, seed=3)
    n = np.array([a * b * c for a, b, c, _, _ in boxes])
    assert n.min() >= 2000 and n.max() <= 700000
    assert len({f for *_, f, _ in boxes}) > 1


REF_FARM = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref", "lnInclude")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF_FARM, "OpenFOAM")),
                    reason="reference headers (oracle/_ref) not built here")
def test_plugin_compiles_against_reference_headers():
    import subprocess
    src = os.path.join(os.path.dirname(INCLUDE_DIR), "openfoam-dev_gb300", "plugin", "cudaLduSolvers.C")
    r = subprocess.run(["g++", "-std=c++14", "-fsyntax-only", "-DWM_DP", "-DWM_LABEL_SIZE=32", "-DNoRepository",
                        "-Dlinux64", "-ftemplate-depth-256", "-w", "-I" + os.path.join(REF_FARM, "OpenFOAM"),
                        "-I" + os.path.join(REF_FARM, "POSIX"), "-I" + INCLUDE_DIR, src],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_fvm_oracle_agrees_with_the_case_generator_on_an_orthogonal_mesh():
    """The oracle's fvMatrix assembly (ldu_fvm_assemble) and the case
    generator build div(phi,T) - laplacian(gamma,T) with Dirichlet xmin by
    different (equivalent) formulas: on an orthogonal box they agree to
    rounding, which checks the signs and boundary terms of the restatement."""
    m = cases.box_mesh(5, 4, 3, jitter=0.0, seed=2)
    g = cases.fv_geometry(m)
    nI, nB = m["nInternalFaces"], g["bCell"].size
    np.testing.assert_allclose(g["weights"], 0.5, rtol=1e-14)
    ps = m["patchStart"]
    bcType = np.zeros(nB, np.int32)
    bcType[ps[0] - nI:ps[1] - nI] = 1
    Sf = m["Sf"].reshape(-1, 3)
    phi = Sf @ np.array([1.0, 0.3, -0.2])
    cd = cases.convection_diffusion(m, [1.0, 0.3, -0.2], 0.05, dirichlet=("xmin",))
    d, up, lo, src = orc.fvm_assemble(m["owner"][:nI], m["neighbour"], g, phi=phi[:nI], phiB=phi[nI:], lapSign=-1,
                                      gamma=0.05, bcType=bcType, bcValue=np.zeros(nB))
    np.testing.assert_allclose(d, cd["diag"], rtol=1e-13)
    np.testing.assert_allclose(up, cd["upper"], rtol=1e-13, atol=1e-16)
    np.testing.assert_allclose(lo, cd["lower"], rtol=1e-13, atol=1e-16)
    assert np.all(src == 0)


@pytest.mark.parametrize("which", ["cube16", "channel"])
def test_coarse_cyclic_interfaces_match_the_oracle(which):
    """The library's GAMG coarse cyclic interfaces (the host grouping the
    device levels are built from) equal the oracle's restatement of
    cyclicGAMGInterface on every level, and summing each coarse face's fine
    coefficients in ascending fine-face order (the device gather) gives the
    oracle's coarse coefficients bit for bit."""
    if which == "cube16":
        s = cases.cyclic_cube(16, jitter=0.2, seed=4)
    else:
        s = cases.cyclic_cube(12, jitter=0.1, seed=5, U=[1.0, 0.3, 0.2], gamma=0.05)
    agg = orc.Agglomeration(s)
    size, cell, nbr, bou = s["ifSize"], s["ifCell"], s["ifNbr"], s["ifBou"]
    for i in range(agg.n_levels):
        R = agg.level(i)[0]
        ps, fc, nc, f2c = ldu.gamg_coarse_interfaces(R, size, cell, nbr)
        ops, ofc, onc, ob, of2c = orc.gamg_coarse_interfaces(R, size, cell, nbr, bou)
        for a, b in ((ps, ops), (fc, ofc), (nc, onc), (f2c, of2c)):
            np.testing.assert_array_equal(a, b)
        summed = np.zeros(fc.size)
        for k in range(f2c.size):
            summed[f2c[k]] += bou[k]
        np.testing.assert_array_equal(summed, ob)
        assert fc.size <= cell.size and ps.sum() == fc.size
        size, cell, nbr, bou = ps, fc, nc, ob


def _ldu_file(path, s):
    with open(path, "wb") as fh:
        np.array([s["diag"].size, s["l"].size], np.int32).tofile(fh)
        np.ascontiguousarray(s["l"], np.int32).tofile(fh)
        np.ascontiguousarray(s["u"], np.int32).tofile(fh)


def test_sliced_rows_layout_on_the_host(tmp_path):
    """build_sell (csrc/host.cpp), compiled on its own with a checker that reads
    the rows back as the device does: every row's entries in the product's
    order with their coefficient sources, valid padding columns, pattern
    slices on a lexicographic cube, explicit ones on a renumbered mesh, none
    with a row of more than 255 entries."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    csrc = os.path.join(repo, "openfoam-dev_gb300", "csrc")
    cuda_inc = [d for d in ("/usr/local/cuda/include",) if os.path.isdir(d)]
    exe = str(tmp_path / "sell_check")
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-I", csrc, "-I", INCLUDE_DIR] + [f"-I{d}" for d in cuda_inc] +
                       [os.path.join(repo, "tests", "sell_layout_check.cpp"), os.path.join(csrc, "host.cpp"),
                        "-o", exe], capture_output=True, text=True)
    if r.returncode != 0 and "cuda_runtime.h" in r.stderr:
        pytest.skip("no CUDA headers")
    assert r.returncode == 0, r.stderr[-3000:]
    cube = cases.pcg_cube(12, seed=1)
    perm = cases.gamg_cube(9, seed=5)
    cases.renumber(perm, cases.random_order(5, perm["diag"].size))
    n = 300
    faces = sorted([(0, k) for k in range(1, n)] + [(k, k + 1) for k in range(1, n - 1)])
    hub = {"l": np.array([a for a, _ in faces]), "u": np.array([b for _, b in faces]), "diag": np.zeros(n)}
    out = {}
    for name, s in (("cube", cube), ("perm", perm), ("hub", hub)):
        path = str(tmp_path / f"{name}.bin")
        _ldu_file(path, s)
        p = subprocess.run([exe, path], capture_output=True, text=True)
        assert p.returncode == 0, (name, p.stdout, p.stderr)
        out[name] = p.stdout
    assert "patterns=1 slices=54 patternSlices=54" in out["cube"]
    assert "patterns=0 slices=54 patternSlices=0" in out["cube"]
    assert "ok" in out["perm"]
    assert out["hub"].count("not built") == 2


def test_sweep_schedules_respect_their_dependencies(tmp_path):
    """build_sched (csrc/host.cpp), compiled on its own with a checker: in the
    reference order and in the multicolour order (greedy colours, which must
    be proper), the forward, backward and fused 1-3-sweep Gauss-Seidel
    schedules hold every (cell, sweep) once, each entry is the right
    neighbour in the right order with its face's coefficient source, and
    every value a slot reads comes from an earlier DAG level."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    csrc = os.path.join(repo, "openfoam-dev_gb300", "csrc")
    cuda_inc = [d for d in ("/usr/local/cuda/include",) if os.path.isdir(d)]
    exe = str(tmp_path / "sched_check")
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-I", csrc, "-I", INCLUDE_DIR] + [f"-I{d}" for d in cuda_inc] +
                       [os.path.join(repo, "tests", "sched_check.cpp"), os.path.join(csrc, "host.cpp"),
                        "-o", exe], capture_output=True, text=True)
    if r.returncode != 0 and "cuda_runtime.h" in r.stderr:
        pytest.skip("no CUDA headers")
    assert r.returncode == 0, r.stderr[-3000:]
    cube = cases.pcg_cube(10, seed=1)
    perm = cases.gamg_cube(9, seed=5)
    cases.renumber(perm, cases.random_order(5, perm["diag"].size))
    cm = cases.bicgstab_cube(10, seed=2)
    for name, s in (("cube", cube), ("perm", perm), ("cm", cm)):
        path = str(tmp_path / f"{name}.bin")
        _ldu_file(path, s)
        p = subprocess.run([exe, path], capture_output=True, text=True)
        assert p.returncode == 0, (name, p.stdout[-2000:], p.stderr[-2000:])
        assert p.stdout.count(" ok") == 10, (name, p.stdout)
    # the lexicographic hexahedral cube colours in two (red-black)
    p = subprocess.run([exe, str(tmp_path / "cube.bin")], capture_output=True, text=True)
    assert "colours=2" in p.stdout
