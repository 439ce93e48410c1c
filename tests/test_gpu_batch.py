"""Batched solves (cfx_batch_*): many independent systems in one launch, one
CTA per system, checked system by system against the oracle.

* FP64 PCG+DIC: each system's solution within relative L2 1e-10 of the
  oracle's PCG (PCG.C:65-193), iterations within +-1, same solver name and
  initial residual to rounding;
* FP64 PBiCGStab+DILU on asymmetric systems: as the single-system tests
  (iterations within 10% / 4, residual below tolerance);
* FP32-inner / FP64-refined: every system reaches the FP64 residual
  tolerance (checked with the oracle's residual and normFactor), and its
  error against the FP64 solution is bounded;
* a system's result is bit-identical alone and inside a batch, from the
  host and from the resident device vectors, and after autotuning.
"""
import numpy as np
import pytest

from oracle import oracle as orc
from openfoam_dev_gb300 import cases, ldu

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

PATCHES = ("xmin", "xmax", "ymin", "ymax", "zmin", "zmax")
SHAPES = [(8, 8, 8), (12, 6, 5), (5, 17, 9), (20, 7, 3), (9, 9, 14), (4, 4, 30), (16, 16, 6), (3, 11, 25),
          (10, 10, 10), (7, 13, 5), (24, 5, 5), (6, 6, 6)]


def _boxes():
    out = []
    for k, (nx, ny, nz) in enumerate(SHAPES):
        out.append(cases.box(nx, ny, nz, dirichlet=PATCHES[k % 6], seed=100 + k))
    return out


def _concat(systems):
    return np.concatenate([s["source"] for s in systems])


def _split(psi, systems):
    out, o = [], 0
    for s in systems:
        n = s["diag"].size
        out.append(psi[o:o + n])
        o += n
    return out


CTL = {"solver": "cudaPCG", "preconditioner": "DIC", "tolerance": 1e-8, "relTol": 0.0, "maxIter": 2000}


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _residual(s, psi):
    m = orc.Matrix(s)
    r = m.residual(psi, s["source"])
    return np.abs(r).sum() / m.norm_factor(np.zeros_like(psi), s["source"])


def test_batch_fp64_pcg_matches_oracle():
    systems = _boxes()
    bt = ldu.Batch(ldu.default_context(), systems)
    psi = np.zeros(int(bt.offsets[-1]))
    perfs = bt.solve(psi, _concat(systems), CTL)
    for s, x, p in zip(systems, _split(psi, systems), perfs):
        ref = np.zeros_like(s["source"])
        rp = orc.pcg(s, ref, tol=1e-8, max_iter=2000)
        assert p.solverName == "DICPCG"
        assert p.converged and not p.singular
        assert abs(p.nIterations - rp.nIterations) <= 1, (s["name"], p.nIterations, rp.nIterations)
        assert p.initialResidual == pytest.approx(rp.initialResidual, rel=1e-12)
        assert _rel(x, ref) <= 1e-10, s["name"]


def test_batch_mixed_reaches_fp64_tolerance():
    systems = _boxes()
    bt = ldu.Batch(ldu.default_context(), systems)
    src = _concat(systems)
    psi64 = np.zeros(int(bt.offsets[-1]))
    bt.solve(psi64, src, CTL)
    psi = np.zeros_like(psi64)
    perfs = bt.solve(psi, src, dict(CTL, precision="mixed"))
    for s, x, x64, p in zip(systems, _split(psi, systems), _split(psi64, systems), perfs):
        assert p.converged and not p.singular
        assert p.nOuter >= 1
        assert p.finalResidual < 1e-8
        assert _residual(s, x) < 1.5e-8, s["name"]
        # the error of a 1e-8 residual solve, from either precision
        assert _rel(x, x64) <= 1e-5, s["name"]


def test_batch_result_is_the_same_alone_and_in_the_mix():
    systems = _boxes()
    ctx = ldu.default_context()
    for prec in ("FP64", "mixed"):
        ctl = dict(CTL, precision=prec)
        bt = ldu.Batch(ctx, systems)
        psi = np.zeros(int(bt.offsets[-1]))
        bt.solve(psi, _concat(systems), ctl)
        parts = _split(psi, systems)
        for k in (0, 5, len(systems) - 1):
            one = ldu.Batch(ctx, [systems[k]])
            x = np.zeros(systems[k]["diag"].size)
            one.solve(x, systems[k]["source"], ctl)
            np.testing.assert_array_equal(x, parts[k])


class _DeviceArray:
    """A float64 device array owned by the library, seen by torch."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (ptr, False), "version": 2}


def test_batch_device_vectors_and_tuning_give_the_same_result():
    systems = _boxes()
    bt = ldu.Batch(ldu.default_context(), systems)
    src = _concat(systems)
    psi = np.zeros(int(bt.offsets[-1]))
    ctl = dict(CTL, precision="mixed")
    bt.solve(psi, src, ctl)
    n = int(bt.offsets[-1])
    d_psi, d_src = bt.vectors()
    t_psi = torch.as_tensor(_DeviceArray(d_psi, n), device="cuda")
    t_src = torch.as_tensor(_DeviceArray(d_src, n), device="cuda")
    np.testing.assert_array_equal(t_src.cpu().numpy(), src)
    np.testing.assert_array_equal(t_psi.cpu().numpy(), psi)
    t_psi.zero_()
    torch.cuda.synchronize()
    cs, ms = bt.tune(ctl)
    assert cs in (0, 4, 8, 16) and ms > 0
    assert float(t_psi.abs().max()) == 0.0  # restored after tuning
    # the comparison below is with the single-CTA form
    bt.set_groups(0, 0)
    perfs = bt.solve_device(ctl)
    assert all(p.converged for p in perfs)
    np.testing.assert_array_equal(t_psi.cpu().numpy(), psi)


def test_batch_rejects_bad_requests():
    ctx = ldu.default_context()
    s = cases.box(5, 5, 5, seed=3)
    bad = dict(s)
    bad["l"], bad["u"] = s["u"].copy(), s["l"].copy()
    with pytest.raises(ldu.CfxError) as e:
        ldu.Batch(ctx, [s, bad])
    assert e.value.status == -2
    cd = cases.convection_diffusion(cases.box_mesh(6, 5, 4, seed=2), [1.0, 0.2, 0.1], 1e-2)
    cd["source"] = cases.uniform(9, cd["diag"].size)
    bt = ldu.Batch(ctx, [cd])
    with pytest.raises(ldu.FatalError, match="asymmetric matrix solver cudaPCG"):
        bt.solve(np.zeros(cd["diag"].size), cd["source"], CTL)


def test_batch_pbicgstab_dilu_on_asymmetric_systems():
    systems = []
    for k, (nx, ny, nz) in enumerate([(8, 6, 5), (10, 10, 4), (5, 9, 12), (7, 7, 7)]):
        U = np.array([1.0, 0.3 * (k - 1), 0.2])
        sy = cases.convection_diffusion(cases.box_mesh(nx, ny, nz, jitter=0.1, seed=k), U / np.linalg.norm(U), 1e-2)
        sy["source"] = cases.uniform(50 + k, sy["diag"].size)
        systems.append(sy)
    bt = ldu.Batch(ldu.default_context(), systems)
    ctl = {"solver": "cudaPBiCGStab", "preconditioner": "DILU", "tolerance": 1e-9, "relTol": 0.0, "maxIter": 1000}
    for prec in ("FP64", "mixed"):
        psi = np.zeros(int(bt.offsets[-1]))
        perfs = bt.solve(psi, _concat(systems), dict(ctl, precision=prec))
        for s, x, p in zip(systems, _split(psi, systems), perfs):
            assert p.solverName == "DILUPBiCGStab"
            assert p.converged
            assert _residual(s, x) < 1.5e-9
            ref = np.zeros_like(s["source"])
            rp = orc.pbicgstab(s, ref, tol=1e-9, max_iter=1000)
            if prec == "FP64":
                assert abs(p.nIterations - rp.nIterations) <= max(4, rp.nIterations // 10)
                assert p.initialResidual == pytest.approx(rp.initialResidual, rel=1e-12)
            assert _rel(x, ref) <= 1e-5


@pytest.mark.parametrize("cluster", [2, 8, 16])
def test_batch_cluster_form_matches_oracle(cluster):
    """Large systems solved by whole thread-block clusters (phase 1) and the
    rest by single CTAs (phase 2) in one launch."""
    systems = _boxes()
    bt = ldu.Batch(ldu.default_context(), systems)
    big = sorted(s["diag"].size for s in systems)[len(systems) // 2]
    bt.set_groups(cluster, big)
    cs, nbig, _ = bt.groups()
    assert cs == cluster and nbig >= len(systems) // 2
    for prec in ("FP64", "mixed"):
        psi = np.zeros(int(bt.offsets[-1]))
        perfs = bt.solve(psi, _concat(systems), dict(CTL, precision=prec))
        for s, x, p in zip(systems, _split(psi, systems), perfs):
            assert p.converged and not p.singular
            assert _residual(s, x) < 1.5e-8, s["name"]
            if prec == "FP64":
                ref = np.zeros_like(s["source"])
                rp = orc.pcg(s, ref, tol=1e-8, max_iter=2000)
                assert abs(p.nIterations - rp.nIterations) <= 1, (s["name"], p.nIterations, rp.nIterations)
                assert _rel(x, ref) <= 1e-10, s["name"]
        # reproducible bit for bit
        again = np.zeros_like(psi)
        bt.solve(again, _concat(systems), dict(CTL, precision=prec))
        np.testing.assert_array_equal(again, psi)


def test_batch_autotune_keeps_results_within_tolerance():
    systems = _boxes()
    bt = ldu.Batch(ldu.default_context(), systems)
    cs, ms = bt.tune(dict(CTL, precision="mixed"))
    assert cs in (0, 4, 8, 16) and ms > 0
    psi = np.zeros(int(bt.offsets[-1]))
    perfs = bt.solve(psi, _concat(systems), dict(CTL, precision="mixed"))
    for s, x, p in zip(systems, _split(psi, systems), perfs):
        assert p.converged and _residual(s, x) < 1.5e-8
