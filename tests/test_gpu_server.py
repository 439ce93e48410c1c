"""The solve server (cfx_server_*): resident matrices, continuous batching,
HBM admission, cancellation and disconnects, large requests through the
whole-GPU drivers.

* every request's result matches the oracle (FP64: relative L2 1e-10,
  iterations +-1) or reaches the FP64 tolerance (mixed);
* a request's result is bit-identical whether it ran alone or in a launch
  shared with many other requests from several client threads;
* re-solving a resident matrix with a new right-hand side needs no new
  registration and gives the oracle's answer;
* a matrix larger than the HBM budget is refused; requests that do not fit
  wait for space; cancelled and released (disconnected) requests free
  their memory;
* large matrices run alone through cudaGAMG and match the single-system
  driver bit for bit.
"""
import threading

import numpy as np
import pytest

from oracle import oracle as orc
from openfoam_dev_gb300 import cases, ldu

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

PATCHES = ("xmin", "xmax", "ymin", "ymax", "zmin", "zmax")
SHAPES = [(8, 8, 8), (12, 6, 5), (5, 17, 9), (20, 7, 3), (9, 9, 14), (16, 16, 6), (10, 10, 10), (24, 5, 5)]
CTL = {"solver": "cudaPCG", "preconditioner": "DIC", "tolerance": 1e-8, "relTol": 0.0, "maxIter": 2000}


def _boxes():
    return [cases.box(nx, ny, nz, dirichlet=PATCHES[k % 6], seed=300 + k) for k, (nx, ny, nz) in enumerate(SHAPES)]


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _residual(s, psi, src=None):
    m = orc.Matrix(s)
    b = s["source"] if src is None else src
    r = m.residual(psi, b)
    return np.abs(r).sum() / m.norm_factor(np.zeros_like(psi), b)


def test_server_results_match_the_oracle():
    sv = ldu.Server(groupCells=700)  # the larger boxes on 4-CTA clusters
    systems = _boxes()
    mids = [sv.add_matrix(s) for s in systems]
    rids = [sv.submit(m, s["source"], CTL) for m, s in zip(mids, systems)]
    for s, rid in zip(systems, rids):
        psi, p = sv.wait(rid)
        ref = np.zeros_like(s["source"])
        rp = orc.pcg(s, ref, tol=1e-8, max_iter=2000)
        assert p.solverName == "DICPCG" and p.converged
        assert abs(p.nIterations - rp.nIterations) <= 1, s["name"]
        assert _rel(psi, ref) <= 1e-10, s["name"]
    st = sv.stats()
    assert st["completed"] == len(systems) and st["residentMatrices"] == len(systems)
    assert st["batches"] >= 1 and st["p99Ms"] >= st["p50Ms"] > 0
    sv.close()


def test_server_result_is_the_same_alone_and_in_the_mix():
    sv = ldu.Server(groupCells=700)
    systems = _boxes()
    mids = [sv.add_matrix(s) for s in systems]
    for prec in ("FP64", "mixed"):
        ctl = dict(CTL, precision=prec)
        alone = {}
        for k in (0, 3, 5):
            alone[k], _ = sv.wait(sv.submit(mids[k], systems[k]["source"], ctl))
        # many requests from several threads at once
        results = {}

        def client(ks):
            rids = [(k, sv.submit(mids[k], systems[k]["source"], ctl)) for k in ks]
            for k, rid in rids:
                results[k] = sv.wait(rid)[0]

        threads = [threading.Thread(target=client, args=(list(range(t, len(systems), 3)),)) for t in range(3)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        assert len(results) == len(systems)
        for k in alone:
            np.testing.assert_array_equal(results[k], alone[k])
        for k, s in enumerate(systems):
            assert _residual(s, results[k]) < 1.5e-8
    sv.close()


def test_server_resolves_a_resident_matrix_with_new_sources():
    sv = ldu.Server()
    s = cases.box(14, 9, 7, dirichlet="ymin", seed=7)
    mid = sv.add_matrix(s)
    rids = []
    srcs = [cases.uniform(40 + i, s["diag"].size) for i in range(3)]
    for src in srcs:  # three correctors queued at once on one matrix
        rids.append(sv.submit(mid, src, CTL))
    for src, rid in zip(srcs, rids):
        psi, p = sv.wait(rid)
        s2 = dict(s, source=src)
        ref = np.zeros_like(src)
        orc.pcg(s2, ref, tol=1e-8, max_iter=2000)
        assert _rel(psi, ref) <= 1e-10
    assert sv.stats()["residentMatrices"] == 1
    # a warm start: the previous solution as psi0 converges at once
    psi, p = sv.wait(sv.submit(mid, srcs[-1], CTL, psi0=psi))
    assert p.nIterations <= 1
    sv.close()


def test_server_admission_refuses_and_waits():
    s = cases.box(20, 20, 20, seed=5)
    small = ldu.Server(hbmBudget=1 << 20)
    with pytest.raises(ldu.CfxError) as e:
        small.add_matrix(s)
    assert e.value.status == -5
    assert small.stats()["refused"] == 1
    small.close()
    # room for the matrix and one request's vectors: a second request waits
    probe = ldu.Server()
    mid = probe.add_matrix(s)
    matrix_bytes = probe.stats()["hbmInUse"]
    probe.close()
    sv = ldu.Server(hbmBudget=matrix_bytes + 2 * 8 * s["diag"].size + 1024)
    mid = sv.add_matrix(s)
    out = {}

    def client(i):
        out[i] = sv.wait(sv.submit(mid, cases.uniform(60 + i, s["diag"].size), CTL))

    threads = [threading.Thread(target=client, args=(i,)) for i in range(3)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert len(out) == 3 and all(p.converged for _, p in out.values())
    assert sv.stats()["hbmInUse"] == matrix_bytes
    sv.close()


def test_server_cancel_and_release_free_their_memory():
    sv = ldu.Server()
    s = cases.box(12, 12, 12, seed=9)
    mid = sv.add_matrix(s)
    base = sv.stats()["hbmInUse"]
    first = sv.submit(mid, s["source"], CTL)
    second = sv.submit(mid, s["source"], CTL)  # same matrix: queued behind the first
    try:
        sv.cancel(second)
        cancelled = True
    except ldu.CfxError as e:
        assert e.status == -8  # already running or finished
        cancelled = False
    if cancelled:
        with pytest.raises(ldu.CfxError) as e:
            sv.wait(second)
        assert e.value.status == -8
    else:
        sv.wait(second)
    psi, p = sv.wait(first)
    assert p.converged
    # a client that disconnects: released while queued or running
    for _ in range(4):
        sv.release(sv.submit(mid, s["source"], CTL))
    # the server drains; everything released is freed
    done = sv.wait(sv.submit(mid, s["source"], CTL))
    assert done[1].converged
    for _ in range(200):
        st = sv.stats()
        if st["queueDepth"] == 0 and st["running"] == 0 and st["hbmInUse"] == base:
            break
        threading.Event().wait(0.01)
    assert st["hbmInUse"] == base
    sv.remove_matrix(mid)
    assert sv.stats()["hbmInUse"] == 0
    sv.close()


def test_server_large_gamg_matches_the_single_system_driver():
    s = cases.gamg_cube(24, jitter=0.2, seed=3)
    ctl = {"solver": "cudaGAMG", "smoother": "GaussSeidel", "nPreSweeps": 2, "tolerance": 1e-8, "relTol": 0.0}
    sv = ldu.Server(largeCells=10000)
    mid = sv.add_matrix(s, gamg=True)
    for prec in ("FP64", "mixed"):
        c = dict(ctl, precision=prec)
        psi, p = sv.wait(sv.submit(mid, s["source"], c))
        ref = np.zeros_like(s["source"])
        rp = ldu.solve(s, ref, c)
        np.testing.assert_array_equal(psi, ref)
        assert p.nIterations == rp.nIterations and p.solverName == "GAMG"
    assert sv.stats()["largeSolves"] == 2
    sv.close()


def test_server_asymmetric_requests_and_metrics():
    sv = ldu.Server()
    cd = cases.convection_diffusion(cases.box_mesh(9, 7, 6, jitter=0.1, seed=4), [1.0, 0.3, 0.2], 1e-2)
    cd["source"] = cases.uniform(21, cd["diag"].size)
    mid = sv.add_matrix(cd)
    ctl = {"solver": "cudaPBiCGStab", "preconditioner": "DILU", "tolerance": 1e-9, "relTol": 0.0}
    psi, p = sv.wait(sv.submit(mid, cd["source"], ctl))
    assert p.solverName == "DILUPBiCGStab" and p.converged and _residual(cd, psi) < 1.5e-9
    with pytest.raises(ldu.FatalError):
        sv.submit(mid, cd["source"], CTL)  # PCG on an asymmetric matrix
    import json
    m = json.loads(sv.metrics_json())
    for k in ("solvesPerS", "p50Ms", "p99Ms", "queueDepth", "hbmInUse", "hbmBudget"):
        assert k in m
    sv.close()


def test_small_requests_run_between_the_cycles_of_a_large_solve():
    """Continuous batching across kinds: small requests that arrive while a
    large GAMG solve runs are served in the gaps between its V-cycles (the
    large solve yields the GPU to one batch at a time), finish long before
    it, and every result equals the one computed alone."""
    s = cases.gamg_cube(40, jitter=0.2, seed=4)
    gctl = {"solver": "cudaGAMG", "smoother": "GaussSeidel", "nPreSweeps": 2, "tolerance": 1e-10, "relTol": 0.0}
    sv = ldu.Server(largeCells=10000, groupCells=700)
    big = sv.add_matrix(s, gamg=True)
    systems = _boxes()
    mids = [sv.add_matrix(x) for x in systems]
    alone = [sv.wait(sv.submit(m, x["source"], CTL))[0] for m, x in zip(mids, systems)]
    psi_big_alone, p_alone = sv.wait(sv.submit(big, s["source"], gctl))
    sv.reset_stats()
    import time
    rid_big = sv.submit(big, s["source"], gctl)
    t0 = time.perf_counter()
    while sv.stats()["running"] < 1 and time.perf_counter() - t0 < 5.0:
        time.sleep(0.0002)  # the large solve has started
    t_small = []
    rids = [sv.submit(m, x["source"], CTL) for m, x in zip(mids, systems)]
    for k, rid in enumerate(rids):
        psi, p = sv.wait(rid)
        t_small.append(time.perf_counter())
        np.testing.assert_array_equal(psi, alone[k])
    psi_big, p_big = sv.wait(rid_big)
    t_big = time.perf_counter()
    np.testing.assert_array_equal(psi_big, psi_big_alone)
    assert p_big.nIterations == p_alone.nIterations
    st = sv.stats()
    assert st["largeSolves"] == 1 and st["batchedSolves"] == len(systems)
    # the small requests were served inside the large solve, not after it
    assert st["largeYields"] >= 1
    assert max(t_small) <= t_big
    sv.close()


def test_small_requests_do_not_wait_for_a_long_launch():
    """Batch lanes: a small request submitted while a long launch (one
    cluster-sized system) runs starts on an idle lane at once and finishes
    first; both results equal the ones computed alone."""
    long_sys = cases.box(64, 64, 48, dirichlet="xmin", seed=21)
    ctl_long = dict(CTL, tolerance=1e-12)
    sv = ldu.Server(groupCells=100000)
    big = sv.add_matrix(long_sys)
    systems = _boxes()[:4]
    mids = [sv.add_matrix(x) for x in systems]
    alone = [sv.wait(sv.submit(m, x["source"], CTL))[0] for m, x in zip(mids, systems)]
    big_alone, _ = sv.wait(sv.submit(big, long_sys["source"], ctl_long))
    import time
    rid_big = sv.submit(big, long_sys["source"], ctl_long)
    t0 = time.perf_counter()
    while sv.stats()["running"] < 1 and time.perf_counter() - t0 < 5.0:
        time.sleep(0.0002)
    rids = [sv.submit(m, x["source"], CTL) for m, x in zip(mids, systems)]
    done_small = []
    for k, rid in enumerate(rids):
        psi, _ = sv.wait(rid)
        done_small.append(time.perf_counter())
        np.testing.assert_array_equal(psi, alone[k])
    psi_big, _ = sv.wait(rid_big)
    t_big = time.perf_counter()
    np.testing.assert_array_equal(psi_big, big_alone)
    assert max(done_small) < t_big
    st = sv.stats()
    assert st["batches"] >= 2
    sv.close()


def test_a_small_request_completes_before_the_largest_of_its_launch():
    """Per-system completion: with one lane, a small request that shares a
    launch with a large one is handed back as soon as its own system
    finishes (the kernel publishes each system's result), not when the
    launch ends; both results equal the ones computed alone."""
    sv = ldu.Server(lanes=1, groupCells=10 ** 9)
    blocker = cases.box(40, 40, 40, dirichlet="xmin", seed=31)
    big = cases.box(40, 40, 40, dirichlet="ymin", seed=32)
    small = cases.box(8, 8, 8, dirichlet="zmin", seed=33)
    ctl = dict(CTL, tolerance=1e-12)
    m_blk, m_big, m_small = sv.add_matrix(blocker), sv.add_matrix(big), sv.add_matrix(small)
    big_alone, _ = sv.wait(sv.submit(m_big, big["source"], ctl))
    small_alone, _ = sv.wait(sv.submit(m_small, small["source"], ctl))
    import time
    rid_blk = sv.submit(m_blk, blocker["source"], ctl)
    t0 = time.perf_counter()
    while sv.stats()["running"] < 1 and time.perf_counter() - t0 < 5.0:
        time.sleep(0.0002)
    rid_big = sv.submit(m_big, big["source"], ctl)
    rid_small = sv.submit(m_small, small["source"], ctl)
    done = {}

    def waiter(name, rid):
        done[name] = (sv.wait(rid)[0], time.perf_counter())

    ts = [threading.Thread(target=waiter, args=a) for a in (("big", rid_big), ("small", rid_small))]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    sv.wait(rid_blk)
    np.testing.assert_array_equal(done["big"][0], big_alone)
    np.testing.assert_array_equal(done["small"][0], small_alone)
    assert done["small"][1] < done["big"][1]
    sv.close()
