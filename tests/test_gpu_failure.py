"""Failure detection without a GPU fault: a bounded device wait is made to
expire (a completion count that nothing reaches), the kernel reports
CFX_ERR_TIMEOUT through the status word the host reads, every CTA returns,
and the same context then solves normally."""
import time

import numpy as np
import pytest

from oracle import oracle as orc
from openfoam_dev_gb300 import cases, ldu

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_expired_wait_reports_timeout_and_the_context_stays_usable():
    s = cases.pcg_cube(16, seed=2)
    mesh = ldu.LduMesh(ldu.default_context(), s["diag"].size, s["l"], s["u"])
    A = ldu.LduMatrix(mesh, s["diag"], s["upper"])
    t0 = time.perf_counter()
    status = A.diag_sweep_stall(50)
    dt = time.perf_counter() - t0
    assert status == -6  # CFX_ERR_TIMEOUT
    assert dt < 5.0
    # a normal solve on the same context afterwards
    psi = np.zeros(s["diag"].size)
    perf = ldu.solver_new("T", A, {"solver": "cudaPCG", "preconditioner": "DIC", "tolerance": 1e-8,
                                   "relTol": 0}).solve(psi, s["source"])
    ref = np.zeros_like(psi)
    orc.pcg(s, ref, tol=1e-8)
    assert perf.converged
    assert np.linalg.norm(psi - ref) <= 1e-10 * np.linalg.norm(ref)


def test_diag_rejects_bad_arguments():
    s = cases.pcg_cube(6, seed=2)
    mesh = ldu.LduMesh(ldu.default_context(), s["diag"].size, s["l"], s["u"])
    A = ldu.LduMatrix(mesh, s["diag"], s["upper"])
    with pytest.raises(ldu.CfxError):
        A.diag_sweep_stall(0)
