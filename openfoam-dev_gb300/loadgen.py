"""Workload drivers for the batched and serving paths (used by bench.py).

* ``batch_systems``: the batch of independent PCG+DIC Laplacian systems —
  box meshes with cell counts log-uniform in [4096, 500000], per-axis aspect
  ratios U[1,4], Dirichlet on one seeded face of six, source U[-1,1].
* ``bench_batch``: solves/s of one launch over the whole batch (resident
  vectors, CUDA events on the library's stream), the same through the host
  API (pinned psi/source in and psi out), and the one-solve-at-a-time rate
  of the whole-GPU driver on a sample of the same systems.
* ``serve_stream``: a Poisson-arrival stream of requests against a solve
  server — 90% batch-like systems (30% of all requests re-solve a resident
  matrix with a new source, the rest register a matrix from the pool, solve
  and remove it), 10% large jittered-cube GAMG Laplacians — with latency
  percentiles, throughput and the server's own counters.
"""
import math
import threading
import time

import numpy as np

from . import cases, ldu

PCG = {"solver": "cudaPCG", "preconditioner": "DIC", "tolerance": 1e-8, "relTol": 0.0, "maxIter": 2000}
GAMG = {"solver": "cudaGAMG", "smoother": "GaussSeidel", "nPreSweeps": 2, "nPostSweeps": 2,
        "nCellsInCoarsestLevel": 10, "tolerance": 1e-8, "relTol": 0.0, "maxIter": 200}


def batch_systems(count=512, seed=1, lo=4096, hi=500000):
    return [cases.box(nx, ny, nz, dirichlet=f, seed=sd)
            for nx, ny, nz, f, sd in cases.batch_boxes(count, lo=lo, hi=hi, seed=seed)]


class _DeviceArray:
    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (ptr, False), "version": 2}


def bench_batch(ctx, systems, steps=3, warmup=1, precision="mixed", sample=16):
    """Times batched solves of `systems`; returns a dict of the measurements."""
    import torch
    bt = ldu.Batch(ctx, systems)
    N = int(bt.offsets[-1])
    src = np.concatenate([s["source"] for s in systems])
    ctl = dict(PCG, precision=precision)
    d_psi, d_src = bt.vectors()
    t_psi = torch.as_tensor(_DeviceArray(d_psi, N), device="cuda")
    t_src = torch.as_tensor(_DeviceArray(d_src, N), device="cuda")
    t_src.copy_(torch.from_numpy(src))
    stream = torch.cuda.ExternalStream(ctx.stream())
    torch.cuda.synchronize()
    cluster, tune_ms = bt.tune(ctl)
    groups = bt.groups()

    def one():
        with torch.cuda.stream(stream):
            t_psi.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        perfs = bt.solve_device(ctl)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3, perfs

    for _ in range(warmup):
        one()
    l0 = ctx.launch_count()
    times, perfs = [], None
    for _ in range(steps):
        t, perfs = one()
        times.append(t)
    launches = (ctx.launch_count() - l0) / max(steps, 1)
    t_dev = float(np.median(times))
    # host API: pinned psi/source in, psi out
    h_src = torch.from_numpy(src).pin_memory().numpy()
    h_psi = torch.zeros(N, dtype=torch.float64).pin_memory().numpy()
    e2e = []
    for i in range(warmup + steps):
        h_psi[:] = 0.0
        t0 = time.perf_counter()
        bt.solve(h_psi, h_src, ctl)
        if i >= warmup:
            e2e.append(time.perf_counter() - t0)
    t_e2e = float(np.median(e2e))
    its = np.array([p.nIterations for p in perfs])
    # one solve at a time through the whole-GPU driver, on an even sample
    idx = np.linspace(0, len(systems) - 1, min(sample, len(systems))).astype(int)
    t_one = 0.0
    n_sample = 0
    for i in idx:
        s = systems[i]
        x = np.zeros(s["diag"].size)
        ldu.solve(s, x, ctl)  # warm: schedules, graphs
        x[:] = 0.0
        t0 = time.perf_counter()
        ldu.solve(s, x, ctl)
        t_one += time.perf_counter() - t0
        n_sample += s["diag"].size
        s.pop("_cfx", None)
    a, b = bt.timings()
    out = {
        "systems": len(systems), "cells": N, "precision": precision, "launch_s": t_dev,
        "solves_per_s": len(systems) / t_dev, "e2e_s": t_e2e, "e2e_solves_per_s": len(systems) / t_e2e,
        "h2d_bytes": 16 * N, "d2h_bytes": 8 * N, "kernel_launches_per_step": launches,
        "converged": bool(all(p.converged for p in perfs)),
        "max_final_residual": float(max(p.finalResidual for p in perfs)),
        "iterations_mean": float(its.mean()), "iterations_max": int(its.max()),
        "cluster_size": groups[0], "systems_on_clusters": groups[1], "tune_ms": tune_ms,
        "mean_concurrent_systems": float((b - a).sum() / max(b.max(), 1e-9)),
        "one_at_a_time_solves_per_s": len(idx) / t_one,
        "one_at_a_time_sample": f"{len(idx)} systems evenly spaced in the batch ({n_sample} cells), "
                                f"whole-GPU cudaPCG, {precision}",
    }
    out["speedup_vs_one_at_a_time"] = out["solves_per_s"] / out["one_at_a_time_solves_per_s"]
    bt.close()
    return out


def _pct(v, q):
    v = sorted(v)
    if not v:
        return None
    return float(v[min(len(v) - 1, max(0, math.ceil(q * len(v)) - 1))])


class ServeMix:
    """The request mix: a pool of batch-like systems, a set of them kept
    resident, and one large GAMG system kept resident."""

    def __init__(self, server, pool, large, resident=16, seed=1):
        self.server = server
        self.pool = pool
        self.large = large
        self.rng = np.random.default_rng(seed)
        self.lock = threading.Lock()
        self.large_mid = server.add_matrix(large, gamg=True) if large is not None else None
        self.resident = [(i, server.add_matrix(pool[i])) for i in range(min(resident, len(pool)))]

    def draw(self, large_frac=0.1, resident_frac=0.3):
        with self.lock:
            u = self.rng.random()
            seed = int(self.rng.integers(1 << 30))
            if self.large_mid is not None and u < large_frac:
                return ("large", None, seed)
            if u < large_frac + resident_frac:
                return ("resident", self.resident[int(self.rng.integers(len(self.resident)))], seed)
            return ("new", int(self.rng.integers(len(self.pool))), seed)

    def run(self, req, precision, phases=None):
        """One client request; returns (kind, latency_s, converged).  phases
        (a dict, optional) receives the seconds spent registering, solving
        (submit to the end of wait) and removing."""
        kind, what, seed = req
        t0 = time.perf_counter()
        sv = self.server
        ph = {} if phases is None else phases
        if kind == "large":
            src = cases.uniform(seed, self.large["diag"].size)
            t1 = time.perf_counter()
            _, p = sv.wait(sv.submit(self.large_mid, src, dict(GAMG, precision=precision)))
            ph["solve"] = time.perf_counter() - t1
        elif kind == "resident":
            i, mid = what
            src = cases.uniform(seed, self.pool[i]["diag"].size)
            t1 = time.perf_counter()
            _, p = sv.wait(sv.submit(mid, src, dict(PCG, precision=precision)))
            ph["solve"] = time.perf_counter() - t1
        else:
            s = self.pool[what]
            mid = sv.add_matrix(s)
            t1 = time.perf_counter()
            ph["add"] = t1 - t0
            try:
                _, p = sv.wait(sv.submit(mid, s["source"], dict(PCG, precision=precision)))
            finally:
                t2 = time.perf_counter()
                ph["solve"] = t2 - t1
                sv.remove_matrix(mid)
                ph["remove"] = time.perf_counter() - t2
        return kind, time.perf_counter() - t0, bool(p.converged)


def serve_unloaded(mix, count, precision, seed=7):
    """Requests of the mix one at a time (no queueing): their latencies."""
    rng = np.random.default_rng(seed)
    lat = {"all": []}
    kinds = []
    for _ in range(count):
        req = mix.draw()
        kinds.append(req[0])
        k, t, ok = mix.run(req, precision)
        lat["all"].append(t)
        lat.setdefault(k, []).append(t)
    del rng
    return {"requests": count, "p50_ms": 1e3 * _pct(lat["all"], 0.5), "p99_ms": 1e3 * _pct(lat["all"], 0.99),
            "by_kind_p50_ms": {k: 1e3 * _pct(v, 0.5) for k, v in lat.items() if k != "all"},
            "by_kind_p99_ms": {k: 1e3 * _pct(v, 0.99) for k, v in lat.items() if k != "all"},
            "by_kind_n": {k: len(v) for k, v in lat.items() if k != "all"}}


def per_kind_ratio(stream, unloaded):
    """Each request kind's p99 under load over its p99 one at a time (and
    over its median one at a time), and the worst of the first."""
    out = {}
    for k, v in stream["by_kind"].items():
        u99 = unloaded["by_kind_p99_ms"].get(k)
        u50 = unloaded["by_kind_p50_ms"].get(k)
        out[k] = {"p99_over_unloaded_p99": v["p99_ms"] / u99 if u99 else None,
                  "p99_over_unloaded_p50": v["p99_ms"] / u50 if u50 else None}
    worst = [r["p99_over_unloaded_p99"] for r in out.values() if r["p99_over_unloaded_p99"] is not None]
    return out, (max(worst) if worst else None)


def serve_stream(mix, rate, duration, precision, seed=11, clients=64):
    """Poisson arrivals at `rate` requests/s for `duration` s, each request
    handled by a client thread (register / submit / wait / remove)."""
    from concurrent.futures import ThreadPoolExecutor
    rng = np.random.default_rng(seed)
    arrivals = []
    t = 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        arrivals.append(t)
    reqs = [mix.draw() for _ in arrivals]
    mix.server.reset_stats()
    results = []
    lock = threading.Lock()
    start = time.perf_counter()

    phases = {}

    def handle(i):
        # latency from the scheduled arrival (includes any client-side delay)
        t_begin = time.perf_counter()
        ph = {}
        k, _, ok = mix.run(reqs[i], precision, ph)
        done = time.perf_counter()
        ph["client_wait"] = t_begin - (start + arrivals[i])
        with lock:
            results.append((k, done - (start + arrivals[i]), ok, done))
            for name, v in ph.items():
                phases.setdefault(k, {}).setdefault(name, []).append(v)

    with ThreadPoolExecutor(max_workers=clients) as ex:
        futs = []
        for i, a in enumerate(arrivals):
            delay = start + a - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            futs.append(ex.submit(handle, i))
        for f in futs:
            f.result()
    end = max(r[3] for r in results) if results else time.perf_counter()
    lat = [r[1] for r in results]
    by = {}
    for k, t_, _, _ in results:
        by.setdefault(k, []).append(t_)
    st = mix.server.stats()
    return {"rate_offered": rate, "duration_s": duration, "requests": len(results),
            "solves_per_s": len(results) / (end - start), "p50_ms": 1e3 * _pct(lat, 0.5),
            "p99_ms": 1e3 * _pct(lat, 0.99), "max_ms": 1e3 * max(lat),
            "by_kind": {k: {"n": len(v), "p50_ms": 1e3 * _pct(v, 0.5), "p99_ms": 1e3 * _pct(v, 0.99)}
                        for k, v in by.items()},
            "converged": all(r[2] for r in results),
            # where the time goes, per kind: p99 of each phase of the client's request
            "phases_p99_ms": {k: {n: 1e3 * _pct(v, 0.99) for n, v in d.items()} for k, d in phases.items()},
            "server": {k: st[k] for k in ("batches", "batchedSolves", "largeSolves", "largeYields", "hbmInUse",
                                          "hbmBudget", "refused", "failed", "queueP50Ms", "queueP99Ms",
                                          "runP50Ms", "runP99Ms")}}
