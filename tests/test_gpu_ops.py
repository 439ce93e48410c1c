"""Kernel parity on the GPU: every single operation through the C ABI must
equal the oracle (and so the reference) bit for bit.

The kernels gather each cell's contributions in the reference's per-cell face
order and the library is built without FMA contraction, so Amul, Tmul,
residual, sumA, the DIC/DILU reciprocal diagonals and preconditioners, and the
GaussSeidel / DIC smoothers are exact.  Both sweep forms (one CTA with block
barriers, and the multi-CTA level scheduler) are exercised, on the natural
lexicographic order and on randomly permuted meshes (many short levels).
"""
import numpy as np
import pytest

from golden_cases import system
from oracle import oracle as orc
from sweep_forms import FORMS, sweep_form as form_ctx
from openfoam_dev_gb300 import cases, ldu

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def _permuted(kind, seed):
    s = getattr(cases, kind)(**({"n": 9, "seed": seed} if kind != "bicgstab_cube" else {"n": 8, "seed": seed}))
    cases.renumber(s, cases.random_order(seed, s["diag"].size))
    s["source"] = cases.uniform(seed + 1, s["diag"].size)
    return s


SYSTEMS = {
    "cube6": lambda: system("cube6"),
    "jcube7": lambda: system("jcube7"),
    "cd6": lambda: system("cd6"),
    "box": lambda: system("box"),
    "cyc7": lambda: system("cyc7"),    # cyclic interfaces, symmetric
    "cycd7": lambda: system("cycd7"),  # cyclic interfaces, upwind asymmetric
    "cube24": lambda: cases.pcg_cube(24, seed=3),
    "perm_lap": lambda: _permuted("gamg_cube", 5),
    "perm_cd": lambda: _permuted("bicgstab_cube", 6),
}


@pytest.fixture(params=sorted(FORMS))
def sweep_form(request):
    with form_ctx(request.param):
        yield request.param


def _fresh(s):
    mesh = ldu.LduMesh(ldu.default_context(), s["diag"].size, s["l"], s["u"])
    if s.get("ifCell") is not None:
        mesh.set_interfaces(s["ifSize"], s["ifCell"], s["ifNbr"])
    A = ldu.LduMatrix(mesh, s["diag"], s["upper"], s.get("lower"))
    if s.get("ifCell") is not None:
        A.set_interface_coeffs(s["ifBou"], s.get("ifInt"))
    return mesh, A


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_matrix_products_exact(name):
    s = SYSTEMS[name]()
    _, A = _fresh(s)
    m = orc.Matrix(s)
    n = s["diag"].size
    x = cases.uniform(7, n)
    b = s["source"]
    dx, db, dy = dev(x), dev(b), torch.empty(n, dtype=torch.float64, device="cuda")
    A.Amul(dx, dy)
    np.testing.assert_array_equal(host(dy), m.amul(x))
    A.Tmul(dx, dy)
    np.testing.assert_array_equal(host(dy), m.tmul(x))
    A.residual(dx, db, dy)
    np.testing.assert_array_equal(host(dy), m.residual(x, b))
    A.sumA(dy)
    np.testing.assert_array_equal(host(dy), m.sumA())


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_sweeps_exact(name, sweep_form):
    s = SYSTEMS[name]()
    _, A = _fresh(s)
    m = orc.Matrix(s)
    n = s["diag"].size
    x = cases.uniform(8, n)
    b = s["source"]
    db = dev(b)
    rD = torch.empty(n, dtype=torch.float64, device="cuda")
    w = torch.empty(n, dtype=torch.float64, device="cuda")
    if A.symmetric():
        A.reciprocalD("DIC", rD)
        np.testing.assert_array_equal(host(rD), m.dic_rD())
        A.precondition("DIC", db, w)
        np.testing.assert_array_equal(host(w), m.dic_precondition(b))
        psi = dev(x)
        A.smooth("DIC", psi, db, 2)
        np.testing.assert_array_equal(host(psi), m.dic_smooth(x, b, 2))
    else:
        A.reciprocalD("DILU", rD)
        np.testing.assert_array_equal(host(rD), m.dilu_rD())
        A.precondition("DILU", db, w)
        np.testing.assert_array_equal(host(w), m.dilu_precondition(b))
    psi = dev(x)
    A.smooth("GaussSeidel", psi, db, 3)
    np.testing.assert_array_equal(host(psi), m.gs_smooth(x, b, 3))
    # the rest of the smoother table (symGaussSeidel, DIC/DILU + GaussSeidel, DILU)
    others = ("symGaussSeidel", "DICGaussSeidel") if A.symmetric() else ("symGaussSeidel", "DILU", "DILUGaussSeidel")
    for sm in others:
        psi = dev(x)
        A.smooth(sm, psi, db, 2)
        np.testing.assert_array_equal(host(psi), m.smooth(sm, x, b, 2), err_msg=sm)
    A.precondition("diagonal", db, w)
    np.testing.assert_array_equal(host(w), (1.0 / s["diag"]) * b)


def test_reductions_and_norm_factor():
    s = cases.gamg_cube(20, jitter=0.2, seed=2)
    _, A = _fresh(s)
    m = orc.Matrix(s)
    n = s["diag"].size
    x = cases.uniform(3, n)
    b = s["source"]
    ctx = ldu.default_context()
    dx, db = dev(x), dev(b)
    # fixed-order tree vs the reference's sequential sums: equal to rounding
    assert ctx.reduce(1, db) == pytest.approx(np.abs(b).sum(), rel=1e-13)
    assert ctx.reduce(3, dx, db) == pytest.approx(float(x @ b), rel=1e-11, abs=1e-12)
    assert ctx.reduce(2, db) == pytest.approx(float(b @ b), rel=1e-13)
    assert ctx.reduce(0, db) == pytest.approx(b.sum(), rel=1e-10, abs=1e-12)
    assert A.normFactor(dx, db) == pytest.approx(m.norm_factor(x, b), rel=1e-13)
    # deterministic: the same inputs give the same bits
    assert ctx.reduce(3, dx, db) == ctx.reduce(3, dx, db)


def test_bad_addressing_rejected():
    ctx = ldu.default_context()
    with pytest.raises(ldu.CfxError) as e:
        ldu.LduMesh(ctx, 4, [0, 2, 1], [1, 3, 2])  # lower not in incremental order
    assert e.value.status == -2
    with pytest.raises(ldu.CfxError) as e:
        ldu.LduMesh(ctx, 4, [0, 1], [1, 1])  # l == u
    assert e.value.status == -2
    with pytest.raises(ldu.CfxError) as e:
        ldu.LduMesh(ctx, 4, [0, 1], [1, 4])  # out of range
    assert e.value.status == -2
