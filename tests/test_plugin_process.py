"""The OpenFOAM-side plugin inside a real OpenFOAM process (no GPU needed).

The plugin (openfoam-dev_gb300/plugin/cudaLduSolvers.C) is built against the
reference's libOpenFOAM, compiled from the reference sources by
oracle/build_ref.py, and loaded by the reference harness exactly as a case
loads it: libs.open (dlLibraryTable, dlLibraryTable.C:144-167, what
controlDict's `libs` entry does), then lduMatrix::solver::New with an
fvSolution-style dictionary (lduMatrixSolver.C:40-130).  The tests check the
registration in the symmetric and asymmetric tables, the dispatch into the
plugin's classes, that configuration errors are the reference's own
(FatalIOError texts of lduMatrixSolver.C, lduMatrixPreconditioner.C,
lduMatrixSmoother.C), raised before any device work, and that without a GPU
a solve ends in the plugin's FatalError carrying the library's status text.
They run where the reference build exists (the container that holds the
reference sources) and are skipped elsewhere.
"""
import pytest

from openfoam_dev_gb300 import cases

ref = pytest.importorskip("oracle.reference")

pytestmark = pytest.mark.skipif(not ref.plugin_available(),
                                reason="the reference build (oracle/build_ref.py) is not here")

SYM = cases.pcg_cube(6, seed=2)
ASYM = cases.bicgstab_cube(6, seed=2)


def _run(s, ctl, library=None):
    return ref.plugin_solve(s, ctl, library=ref.PLUGIN if library is None else library)


def _fatal(r):
    return r.get("fatal", "")


def test_library_loads_and_registers_its_solvers():
    r = _run(SYM, {"solver": "cudaNope", "tolerance": 1e-8})
    assert int(r["loaded"][0]) == 1
    msg = _fatal(r)
    assert msg.startswith("Unknown symmetric matrix solver cudaNope")
    for name in ("cudaPCG", "cudaPBiCGStab", "cudaGAMG", "cudaSmoothSolver", "PCG", "GAMG"):
        assert f"\n{name}\n" in msg, name
    r = _run(ASYM, {"solver": "cudaNope", "tolerance": 1e-8})
    msg = _fatal(r)
    assert msg.startswith("Unknown asymmetric matrix solver cudaNope")
    for name in ("cudaPBiCG", "cudaPBiCGStab", "cudaGAMG", "cudaSmoothSolver", "PBiCGStab"):
        assert f"\n{name}\n" in msg, name
    assert "\ncudaPCG\n" not in msg  # symmetric table only, like PCG


def test_without_the_library_the_names_are_unknown():
    r = _run(SYM, {"solver": "cudaPCG", "preconditioner": "DIC", "tolerance": 1e-8}, library="")
    assert int(r["loaded"][0]) == 0
    assert _fatal(r).startswith("Unknown symmetric matrix solver cudaPCG")


@pytest.mark.parametrize("s,ctl,cls", [
    (SYM, {"solver": "cudaPCG", "preconditioner": "DIC"}, "cudaPCG"),
    (SYM, {"solver": "cudaGAMG", "smoother": "GaussSeidel", "nPreSweeps": 2}, "cudaGAMG"),
    (SYM, {"solver": "cudaSmoothSolver", "smoother": "symGaussSeidel"}, "cudaSmoothSolver"),
    (ASYM, {"solver": "cudaPBiCGStab", "preconditioner": "DILU"}, "cudaPBiCGStab"),
    (ASYM, {"solver": "cudaPBiCG", "preconditioner": "DILU"}, "cudaPBiCG"),
    (SYM, {"solver": "cudaPCG", "preconditioner": {"preconditioner": "GAMG", "smoother": "DICGaussSeidel"}},
     "cudaPCG"),
])
def test_selection_dispatches_into_the_plugin(s, ctl, cls, gpu_absent):
    """solver::New builds the plugin's class; with no GPU the solve ends in
    the plugin's FatalError with the library's status text."""
    r = _run(s, dict(ctl, tolerance=1e-8, relTol=0.0))
    assert r["type"] == cls
    assert _fatal(r).startswith("cudaLduSolvers: ")


@pytest.mark.parametrize("s,bad,good", [
    (SYM, {"solver": "cudaPCG", "preconditioner": "foo"}, {"solver": "PCG", "preconditioner": "foo"}),
    (ASYM, {"solver": "cudaPBiCGStab", "preconditioner": "DIC"}, {"solver": "PBiCGStab", "preconditioner": "DIC"}),
    (SYM, {"solver": "cudaPCG"}, {"solver": "PCG"}),
    (SYM, {"solver": "cudaSmoothSolver", "smoother": "bar", "nSweeps": 1},
     {"solver": "smoothSolver", "smoother": "bar", "nSweeps": 1}),
    (ASYM, {"solver": "cudaSmoothSolver", "smoother": "DIC", "nSweeps": 1},
     {"solver": "smoothSolver", "smoother": "DIC", "nSweeps": 1}),
])
def test_configuration_errors_are_the_references(s, bad, good):
    """The plugin reads its dictionary before touching the device and
    reports an unknown or missing preconditioner or smoother with the
    reference's own FatalIOError text (the same valid-name lists)."""
    mine = _fatal(_run(s, dict(bad, tolerance=1e-8, relTol=0.0)))
    theirs = _fatal(_run(s, dict(good, tolerance=1e-8, relTol=0.0)))
    assert theirs and mine == theirs


def test_an_unknown_precision_is_a_configuration_error():
    r = _run(SYM, {"solver": "cudaPCG", "preconditioner": "DIC", "tolerance": 1e-8, "precision": "half"})
    assert _fatal(r) == "cudaLduSolvers: unknown precision half (FP64 or mixed)"


@pytest.fixture
def gpu_absent():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: the solve would run")
