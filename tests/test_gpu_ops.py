"""Kernel parity on the GPU: every single operation through the C ABI must
equal the oracle (and so the reference) bit for bit.

The kernels gather each cell's contributions in the reference's per-cell face
order and the library is built without FMA contraction, so Amul, Tmul,
residual, sumA, the DIC/DILU reciprocal diagonals and preconditioners, and the
GaussSeidel / DIC smoothers are exact.  Both sweep forms (one CTA with block
barriers, and the multi-CTA level scheduler) are exercised, on the natural
lexicographic order and on randomly permuted meshes (many short levels).

The A x products read each row either from the level's sliced ELL copy (the
default, with offset-pattern slices where the rows share their neighbour
offsets; or with explicit columns only) or through the losort/owner gathers;
all three are checked, and a row with more than 255 neighbours (no sliced
copy) falls back to the gathers.
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
    "hub": lambda: _hub(300),     # a row of 299 entries: no sliced copy
    "hub255": lambda: _hub(256),  # a row of 255 entries: a wide explicit slice
}


def _hub(n, seed=4):
    """Cell 0 neighbours every other cell (a row of n-1 > 255 entries), the
    others form a chain: faces in owner order, asymmetric, diagonally
    dominant."""
    faces = [(0, k) for k in range(1, n)] + [(k, k + 1) for k in range(1, n - 1)]
    faces.sort()
    l = np.array([f[0] for f in faces], np.int32)
    u = np.array([f[1] for f in faces], np.int32)
    rng = np.random.default_rng(seed)
    upper = -rng.uniform(0.1, 1.0, l.size)
    lower = -rng.uniform(0.1, 1.0, l.size)
    diag = np.zeros(n)
    np.add.at(diag, l, -upper)
    np.add.at(diag, u, -lower)
    diag += rng.uniform(0.5, 1.0, n)
    return {"name": "hub", "l": l, "u": u, "diag": diag, "upper": upper, "lower": lower,
            "source": rng.uniform(-1, 1, n)}


AMUL_FORMS = {"gather": 0, "explicit": 1, "pattern": 2}


@pytest.fixture(params=sorted(AMUL_FORMS))
def amul_form(request):
    """The product form, set before the test builds its mesh."""
    old = ldu.tune_get(ldu.TUNE_AMUL_SELL)
    ldu.tune_set(ldu.TUNE_AMUL_SELL, AMUL_FORMS[request.param])
    try:
        yield request.param
    finally:
        ldu.tune_set(ldu.TUNE_AMUL_SELL, old)


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
def test_matrix_products_exact(name, amul_form):
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


def test_sliced_rows_layout():
    """Pattern slices where the rows share their offsets (a lexicographic
    cube: every slice), explicit ones on a randomly renumbered mesh, none
    with a row of more than 255 neighbours."""
    old = ldu.tune_get(ldu.TUNE_AMUL_SELL)
    try:
        ldu.tune_set(ldu.TUNE_AMUL_SELL, 2)
        mesh, _ = _fresh(SYSTEMS["cube24"]())
        slices, pat, entries = mesh.sell_info()
        assert slices == 24 ** 3 // 32 and pat == slices and entries == 32 * 6 * slices
        mesh, _ = _fresh(SYSTEMS["perm_lap"]())
        slices, pat, entries = mesh.sell_info()
        assert slices == (9 ** 3 + 31) // 32 and pat < slices
        ldu.tune_set(ldu.TUNE_AMUL_SELL, 1)
        mesh, _ = _fresh(SYSTEMS["cube24"]())
        assert mesh.sell_info()[1] == 0
        mesh, _ = _fresh(SYSTEMS["hub"]())
        assert mesh.sell_info() == (0, 0, 0)
        mesh, _ = _fresh(SYSTEMS["hub255"]())
        assert mesh.sell_info()[:2] == (8, 0)
    finally:
        ldu.tune_set(ldu.TUNE_AMUL_SELL, old)


@pytest.mark.parametrize("name", ["cube24", "cd6", "cycd7", "perm_cd", "hub"])
def test_products_follow_coefficient_updates(name, amul_form):
    """cfx_matrix_update rewrites every copy of the coefficients the products
    read (the sliced rows included)."""
    s = SYSTEMS[name]()
    _, A = _fresh(s)
    n = s["diag"].size
    rng = np.random.default_rng(11)
    s2 = dict(s)
    s2["upper"] = s["upper"] * rng.uniform(0.5, 1.5, s["upper"].size)
    if s.get("lower") is not None:
        s2["lower"] = s["lower"] * rng.uniform(0.5, 1.5, s["lower"].size)
    s2["diag"] = s["diag"] * rng.uniform(1.0, 1.5, n)
    x = cases.uniform(9, n)
    dx, db, dy = dev(x), dev(s["source"]), torch.empty(n, dtype=torch.float64, device="cuda")
    A.Amul(dx, dy)
    A.update(s2["diag"], s2["upper"], s2.get("lower"))
    m2 = orc.Matrix(s2)
    A.Amul(dx, dy)
    np.testing.assert_array_equal(host(dy), m2.amul(x))
    A.residual(dx, db, dy)
    np.testing.assert_array_equal(host(dy), m2.residual(x, s["source"]))


@pytest.mark.parametrize("name", sorted(set(SYSTEMS) - {"hub", "hub255"}))
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


def _colored_gs(s, x, b, sweeps, dt=np.float64):
    """The multicolour Gauss-Seidel the FP32 inner cycles use, on the host in
    precision dt: greedy colours (ascending cells, smallest colour no
    smaller-index neighbour has); per sweep the colours in ascending order,
    each cell from b minus its smaller-coloured neighbours' new values, then
    its larger-coloured neighbours' old values (each group in the reference's
    entry order: losort faces, then owned faces), divided by the diagonal."""
    n = s["diag"].size
    l, u = np.asarray(s["l"]), np.asarray(s["u"])
    upper = np.asarray(s["upper"], dt)
    lower = upper if s.get("lower") is None else np.asarray(s["lower"], dt)
    diag = np.asarray(s["diag"], dt)
    b = np.asarray(b, dt)
    entries = [[] for _ in range(n)]
    for f in np.argsort(u, kind="stable"):  # losort: by neighbour cell, faces in order
        entries[u[f]].append((int(l[f]), lower[f]))
    for f in range(l.size):
        entries[l[f]].append((int(u[f]), upper[f]))
    color = np.full(n, -1)
    for c in range(n):
        taken = {color[nb] for nb, _ in entries[c] if nb < c}
        k = 0
        while k in taken:
            k += 1
        color[c] = k
    x = np.array(x, dt)
    order = np.argsort(color, kind="stable")
    for _ in range(sweeps):
        for c in order:
            acc = b[c]
            for first in (True, False):
                for nb, cf in entries[c]:
                    if (color[nb] < color[c]) == first:
                        acc = acc - cf * x[nb]
            x[c] = acc / diag[c]
    return x


def _colored_ilu(s, b, transpose=False):
    """The multicolour DIC / DILU the FP32 inner solves use, in FP64 on the
    host: the greedy colours of _colored_gs; a cell's forward entries are its
    smaller-coloured neighbours in the Gauss-Seidel entry order (losort faces,
    then owned faces), its backward entries the larger-coloured ones in the
    reverse of that order; each entry's coefficient is the matrix entry of
    the cell's row (of the transpose's row for preconditionT).  Pivots
    d_c = diag_c - sum upper*lower / d_j over the forward entries, rD = 1/d;
    forward w_c = rD_c r_c - sum (rD_c a_cj) w_j, backward
    w_c -= sum (rD_c a_cj) w_j.  Returns (rD, w)."""
    n = s["diag"].size
    l, u = np.asarray(s["l"]), np.asarray(s["u"])
    upper = np.asarray(s["upper"], np.float64)
    lower = upper if s.get("lower") is None else np.asarray(s["lower"], np.float64)
    if transpose:
        upper, lower = lower, upper
    entries = [[] for _ in range(n)]  # (neighbour, a_cj, upper*lower)
    for f in np.argsort(u, kind="stable"):
        entries[u[f]].append((int(l[f]), lower[f], upper[f] * lower[f]))
    for f in range(l.size):
        entries[l[f]].append((int(u[f]), upper[f], upper[f] * lower[f]))
    color = np.full(n, -1)
    for c in range(n):
        taken = {color[nb] for nb, _, _ in entries[c] if nb < c}
        k = 0
        while k in taken:
            k += 1
        color[c] = k
    order = np.argsort(color, kind="stable")
    d = np.array(s["diag"], np.float64)
    for c in order:
        acc = d[c]
        for nb, _, p in entries[c]:
            if color[nb] < color[c]:
                acc = acc - p / d[nb]
        d[c] = acc
    rD = 1.0 / d
    w = np.zeros(n)
    for c in order:
        acc = rD[c] * b[c]
        for nb, a, _ in entries[c]:
            if color[nb] < color[c]:
                acc = acc - (rD[c] * a) * w[nb]
        w[c] = acc
    for c in order[::-1]:
        acc = w[c]
        for nb, a, _ in entries[c][::-1]:
            if color[nb] > color[c]:
                acc = acc - (rD[c] * a) * w[nb]
        w[c] = acc
    return rD, w


@pytest.mark.parametrize("name", ["cube6", "cd6", "perm_lap", "perm_cd", "box", "cycd7"])
def test_multicolour_dic_dilu_exact(name, sweep_form):
    """The multicolour DIC / DILU schedules (CFX_TUNE_COLORED_PRE 3 runs them
    in FP64 too) equal the host restatement bit for bit in every sweep form:
    the pivots, the preconditioner, DILU's preconditionT, and the DIC / DILU
    smoother's sweeps."""
    s = SYSTEMS[name]()
    old = ldu.tune_get(ldu.TUNE_COLORED_PRE)
    ldu.tune_set(ldu.TUNE_COLORED_PRE, 3)
    try:
        _, A = _fresh(s)
        n = s["diag"].size
        b = s["source"]
        db = dev(b)
        rD = torch.empty(n, dtype=torch.float64, device="cuda")
        w = torch.empty(n, dtype=torch.float64, device="cuda")
        kind = "DIC" if A.symmetric() else "DILU"
        want_rD, want_w = _colored_ilu(s, b)
        A.reciprocalD(kind, rD)
        np.testing.assert_array_equal(host(rD), want_rD)
        A.precondition(kind, db, w)
        np.testing.assert_array_equal(host(w), want_w)
        # the smoother: psi += M^-1 (b - A psi), one sweep from psi = 0
        psi = torch.zeros(n, dtype=torch.float64, device="cuda")
        A.smooth(kind, psi, db, 1)
        np.testing.assert_array_equal(host(psi), want_w)
        if kind == "DILU" and s.get("ifCell") is None:
            # preconditionT (PBiCG's transpose sweeps) on the multicolour
            # schedules: PBiCG+DILU still reaches the solution
            dense = np.diag(np.asarray(s["diag"], np.float64))
            dense[s["l"], s["u"]] = s["upper"]
            dense[s["u"], s["l"]] = s["lower"]
            want = np.linalg.solve(dense, b)
            psi = np.zeros(n)
            p = ldu.solve(s, psi, {"solver": "cudaPBiCG", "preconditioner": "DILU", "tolerance": 1e-12,
                                   "relTol": 0, "maxIter": 1000})
            assert p.converged
            assert np.linalg.norm(psi - want) <= 1e-9 * np.linalg.norm(want)
    finally:
        ldu.tune_set(ldu.TUNE_COLORED_PRE, old)


@pytest.mark.parametrize("name", ["cube24", "cd6", "perm_lap", "box"])
def test_fp32_inner_smoothing_exact(name, sweep_form):
    """cfx_diag_smooth_f32: the FP32 inner cycles' multicolour Gauss-Seidel
    on the FP32 coefficient copy equals an FP32 host restatement bit for bit
    in every sweep form, and reports the form it ran in."""
    s = SYSTEMS[name]()
    _, A = _fresh(s)
    n = s["diag"].size
    x = cases.uniform(8, n).astype(np.float32)
    b = s["source"].astype(np.float32)
    for sweeps in (1, 2, 4):
        psi = torch.from_numpy(x.copy()).cuda()
        form = A.smooth_f32("GaussSeidel", psi, torch.from_numpy(b).cuda(), sweeps)
        assert 0 <= form <= 6
        torch.cuda.synchronize()
        np.testing.assert_array_equal(psi.cpu().numpy(), _colored_gs(s, x, b, sweeps, np.float32))


@pytest.mark.parametrize("name", ["cube6", "cd6", "perm_lap", "box"])
def test_multicolour_gauss_seidel_exact(name):
    """The multicolour Gauss-Seidel schedule (CFX_TUNE_COLORED_GS 2 runs it in
    FP64 too) equals the host restatement bit for bit, fused sweeps included."""
    s = SYSTEMS[name]()
    old = ldu.tune_get(ldu.TUNE_COLORED_GS)
    ldu.tune_set(ldu.TUNE_COLORED_GS, 2)
    try:
        _, A = _fresh(s)
        n = s["diag"].size
        x = cases.uniform(8, n)
        b = s["source"]
        for sweeps in (1, 3):
            psi = dev(x)
            A.smooth("GaussSeidel", psi, dev(b), sweeps)
            np.testing.assert_array_equal(host(psi), _colored_gs(s, x, b, sweeps))
    finally:
        ldu.tune_set(ldu.TUNE_COLORED_GS, old)
