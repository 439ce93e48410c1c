"""Handle lifetimes: a matrix may outlive its mesh and a mesh its context.

The library counts references (a matrix holds its mesh, a mesh, batch or
server holds its context), so handles can be destroyed in any order: a
garbage collector that finalises a cycle's mesh before its matrix, or a
plugin cache torn down at exit, must not touch freed memory.  Each test
destroys the parent first, collects the cycle, and solves again on the
same context.
"""
import gc

import numpy as np
import pytest

from oracle import oracle as orc
from openfoam_dev_gb300 import cases, ldu

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _mesh_matrix(ctx, s):
    mesh = ldu.LduMesh(ctx, s["diag"].size, s["l"], s["u"])
    A = ldu.LduMatrix(mesh, s["diag"], s["upper"], s.get("lower"))
    return mesh, A


def _amul_ref(s, x):
    """y = A x in the reference's per-cell order (lduMatrixATmul.C:34-92)."""
    y = s["diag"] * x
    np.add.at(y, s["u"], s["upper"] * x[s["l"]])
    np.add.at(y, s["l"], s["upper"] * x[s["u"]])
    return y


def test_matrix_used_after_its_mesh_handle_is_destroyed():
    s = cases.pcg_cube(8, seed=5)
    mesh, A = _mesh_matrix(ldu.default_context(), s)
    mesh.close()  # the creator's reference goes first
    x = torch.rand(s["diag"].size, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    A.Amul(x, y)
    torch.cuda.synchronize()
    np.testing.assert_allclose(y.cpu().numpy(), _amul_ref(s, x.cpu().numpy()), rtol=1e-14, atol=1e-15)
    A.close()  # frees the matrix, then the mesh


def test_cycle_collected_mesh_first_then_solve_on_the_same_context():
    ctx = ldu.default_context()
    for seed in range(4):
        s = cases.pcg_cube(6, seed=seed)
        mesh, A = _mesh_matrix(ctx, s)
        # a reference cycle holding both: the collector picks the order
        box = {"mesh": mesh, "A": A}
        box["self"] = box
        mesh.box = box
        A.box = box
        mesh.close()
        del mesh, A, box
    gc.collect()
    s = cases.pcg_cube(12, seed=9)
    psi = np.zeros_like(s["source"])
    perf = ldu.solve(s, psi, {"solver": "cudaPCG", "preconditioner": "DIC", "tolerance": 1e-10, "relTol": 0})
    ref = np.zeros_like(s["source"])
    rp = orc.pcg(s, ref, tol=1e-10, precond="DIC")
    assert perf.converged and abs(perf.nIterations - rp.nIterations) <= 1
    assert np.linalg.norm(psi - ref) <= 1e-10 * np.linalg.norm(ref)


def test_context_destroyed_before_its_mesh_and_matrix():
    ctx = ldu.Context(0)
    s = cases.pcg_cube(6, seed=11)
    mesh, A = _mesh_matrix(ctx, s)
    ctx.close()
    mesh.close()
    psi = np.zeros_like(s["source"])
    perf = ldu.solver_new("psi", A, {"solver": "cudaPCG", "preconditioner": "DIC", "tolerance": 1e-10,
                                     "relTol": 0}).solve(psi, s["source"])
    ref = np.zeros_like(s["source"])
    rp = orc.pcg(s, ref, tol=1e-10, precond="DIC")
    assert perf.converged and abs(perf.nIterations - rp.nIterations) <= 1
    assert np.linalg.norm(psi - ref) <= 1e-10 * np.linalg.norm(ref)
    A.close()  # the last reference: matrix, mesh and context go
