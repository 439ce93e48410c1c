#!/usr/bin/env python3
"""Benchmark of the lduMatrix solver path on one GB300 (or N replicas).

Workload (the headline configuration): cudaGAMG with faceAreaPair
agglomeration, GaussSeidel smoother, nPreSweeps 2, nPostSweeps 2,
nCellsInCoarsestLevel 10, tolerance 1e-8, relTol 0, on the Laplacian of a
256^3 hex cube (16.8M cells) with vertices jittered by U[-0.2h, 0.2h], Dirichlet
T=0 on x=0, source U[-1,1] (seeded, synthetic).

One step is one complete solve from psi = 0 to the 1e-8 residual.  The
headline value is the FP32-inner / FP64-refined solve's time-to-1e-8; the
plain FP64 solve is timed too (fp64_time_s, mixed_speedup).  Device timing uses
CUDA events on the library's stream with the system resident in HBM (its
arrays are larger than the 129 MB L2, so no flush is needed).  e2e times the
reference-facing call a plugin makes per solve: coefficient upload, psi and
source host->device from pinned memory, the solve, psi device->host.

--impl reference times the C restatement of the reference solver (oracle/,
bit-exact with the reference built from its sources, compiled with the
reference's own optimisation flags) on the host cores: every step is one
complete serial solve from psi = 0 to 1e-8, the steps run concurrently, one
process per host core.  Its inputs are the same seeded arrays, written to a
file by a separate generator process, so the timed processes load only the
oracle.

Parity: oracle processes started before the first GPU call solve the same
systems (256^3 GAMG, 64^3 PCG+DIC, 128^3 PBiCGStab+DILU) to 1e-8, then on to
1e-12; the line states each GPU solution's relative L2 error against both.

Multi-GPU: replicas only (one independent system per rank, no collective on
the data path); launch with torchrun, value = max over ranks.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

import __graft_entry__ as ge  # noqa: E402

METRIC = "time-to-1e-8 (FP32-refined vs FP64) of cudaGAMG"
TOL = 1e-8
GAMG = {"solver": "cudaGAMG", "tolerance": TOL, "relTol": 0.0, "smoother": "GaussSeidel",
        "nPreSweeps": 2, "nPostSweeps": 2, "nCellsInCoarsestLevel": 10, "maxIter": 200}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=256, help="cube cells per axis")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--kernel-only", choices=["gs", "level1", "gs32", "level1_32", "solves", "amul"], default=None,
                    help="profiling: gs = the finest level's fused 2-sweep Gauss-Seidel alone, level1 = the "
                         "first agglomerated level's, gs32 / level1_32 = the same levels' FP32 inner-cycle "
                         "smoothing (multicolour order), solves = one FP64 and one mixed headline solve inside "
                         "the NVTX ranges 'profiled_fp64' / 'profiled_mixed' (after one warm-up solve of each), "
                         "amul = Amul on the finest level, FP64 then FP32 (warmup + steps launches each)")
    ap.add_argument("--form", choices=["default", "grid", "flow"], default="default",
                    help="profiling modes: the sweep form of the levels larger than one CTA")
    ap.add_argument("--write-case", default=None, help=argparse.SUPPRESS)
    ap.add_argument("--workload", choices=["all", "gamg", "batch", "serve"], default="all",
                    help="all: the GAMG headline line with the batch and serving measurements added")
    ap.add_argument("--batch-count", type=int, default=512)
    ap.add_argument("--serve-duration", type=float, default=60.0,
                    help="seconds of Poisson arrivals of the serving stream, per precision")
    ap.add_argument("--serve-rate", type=float, default=0.0,
                    help="requests/s of the serving stream (0: the largest rate of the sweep at which every "
                         "request kind's p99 stays within 2x its unloaded p99)")
    ap.add_argument("--serve-sweep-duration", type=float, default=10.0,
                    help="seconds per rate of the sweep that picks the serving rate (0: no sweep)")
    ap.add_argument("--serve-large", type=int, default=200, help="cells per axis of the large GAMG requests")
    return ap.parse_args()


def dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as tdist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        tdist.init_process_group("gloo", rank=rank, world_size=world)
        pg = tdist
    return rank, world, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def reduce_max(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def workload(n):
    """The configuration both arms report (identical dicts)."""
    return {"workload": f"cudaGAMG faceAreaPair GaussSeidel nPre2/nPost2, Laplacian of a {n}^3 cube jittered "
                        f"+-20%, Dirichlet x=0, tolerance 1e-8 relTol 0",
            "n_cells": n ** 3, "n_faces": 3 * n * n * (n - 1), "solve": "psi=0 to residual 1e-8",
            "seed": 1, "l2": "inputs larger than L2 (no flush): the resident system is several GB"}


# ------------------------------------------------------------ oracle (CPU) legs
# These run in processes started with the spawn method before the first GPU
# call.  They load the oracle built with the reference's optimisation flags
# (CFX_ORACLE_TIMED=1; bit-identical results to the build the tests pin).

GAMG_ORACLE = dict(smoother="GaussSeidel", nPreSweeps=2, nPostSweeps=2)


def _oracle_case(kind, n, seed):
    ge.load_package()
    from openfoam_dev_gb300 import cases
    if kind == "gamg":
        return cases.gamg_cube(n, jitter=0.2, seed=seed)
    if kind == "pcg":
        return cases.pcg_cube(n, seed=seed)
    return cases.bicgstab_cube(n, seed=seed)


def _oracle_solve(kind, s, psi, tol, agg=None, max_iter=None):
    from oracle import oracle as orc
    if kind == "gamg":
        return orc.gamg(s, psi, agg, tol=tol, rel_tol=0.0, max_iter=max_iter or 200, **GAMG_ORACLE)
    if kind == "pcg":
        return orc.pcg(s, psi, tol=tol, rel_tol=0.0, max_iter=max_iter or 2000, precond="DIC")
    return orc.pbicgstab(s, psi, tol=tol, rel_tol=0.0, max_iter=max_iter or 2000, precond="DILU")


def oracle_job(kind, n, seed, outdir):
    """One configuration in the oracle (serial): the solve from psi = 0 to
    1e-8, timed (GAMG: the agglomeration, cached per mesh as the reference
    caches it, timed apart), then continued from that psi to 1e-12 (the FP64
    truth every result is measured against).  Both solutions are written to
    outdir; the statistics are returned."""
    os.environ["CFX_ORACLE_TIMED"] = "1"
    from oracle import oracle as orc
    s = _oracle_case(kind, n, seed)
    agg, t_agg = None, 0.0
    if kind == "gamg":
        t0 = time.perf_counter()
        agg = orc.Agglomeration(s, n_coarsest=10)
        t_agg = time.perf_counter() - t0
    psi = np.zeros_like(s["source"])
    t0 = time.perf_counter()
    p = _oracle_solve(kind, s, psi, 1e-8, agg)
    t = time.perf_counter() - t0
    np.save(os.path.join(outdir, f"{kind}{n}_psi8.npy"), psi)
    psi12 = psi.copy()
    q = _oracle_solve(kind, s, psi12, 1e-12, agg, max_iter=4000)
    np.save(os.path.join(outdir, f"{kind}{n}_psi12.npy"), psi12)
    return {"kind": kind, "n": n, "seed": seed, "s": t, "iterations": p.nIterations,
            "final_residual": p.finalResidual, "converged": bool(p.converged), "agglomeration_s": t_agg,
            "truth_iterations": q.nIterations, "truth_final_residual": q.finalResidual,
            "truth_converged": bool(q.converged)}


def _rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def parity_of(job, outdir, psi_fp64, it_fp64, psi_mixed=None):
    """The GPU solutions against the oracle's: FP64 against its 1e-8 solve
    (the drop-in bar: rel L2 <= 1e-10, iterations +-1) and both precisions
    against its 1e-12 solution (the error each result states)."""
    p8 = np.load(os.path.join(outdir, f"{job['kind']}{job['n']}_psi8.npy"))
    p12 = np.load(os.path.join(outdir, f"{job['kind']}{job['n']}_psi12.npy"))
    out = {"oracle_iterations": job["iterations"], "fp64_iterations": it_fp64,
           "fp64_vs_oracle_1e-8_rel_l2": _rel_l2(psi_fp64, p8),
           "fp64_vs_truth_1e-12_rel_l2": _rel_l2(psi_fp64, p12),
           "oracle_1e-8_vs_truth_rel_l2": _rel_l2(p8, p12),
           "truth": f"oracle FP64 continued to {job['truth_final_residual']:.2e} "
                    f"({job['truth_iterations']} more iterations)"}
    if psi_mixed is not None:
        out["mixed_vs_truth_1e-12_rel_l2"] = _rel_l2(psi_mixed, p12)
    out["fp64_drop_in_ok"] = bool(out["fp64_vs_oracle_1e-8_rel_l2"] <= 1e-10 and
                                  abs(it_fp64 - job["iterations"]) <= 1)
    return out


def write_case(path, n, seed=1):
    """The headline system (256^3 jittered Laplacian) as the oracle takes it,
    with its faceAreaPair weights: written by a separate process so that the
    timed reference processes load the oracle only."""
    os.environ["CFX_ORACLE_TIMED"] = "1"
    from oracle import oracle as orc
    s = _oracle_case("gamg", n, seed)
    w = orc.face_area_pair_weights(s["Sf"])
    np.savez(path, l=s["l"], u=s["u"], diag=s["diag"], upper=s["upper"], source=s["source"], weights=w)


def reference_step(path, i):
    """One step of the reference arm: one complete serial solve of the case
    file's system from psi = 0 to 1e-8 (coarse-level set-up included, the
    cached agglomeration not), timed in this process."""
    os.environ["CFX_ORACLE_TIMED"] = "1"
    from oracle import oracle as orc
    z = np.load(path)
    s = {k: z[k] for k in ("l", "u", "diag", "upper", "source")}
    s["lower"] = None
    agg = orc.Agglomeration(s, weights=z["weights"], n_coarsest=10)
    psi = np.zeros_like(s["source"])
    t0 = time.perf_counter()
    p = _oracle_solve("gamg", s, psi, 1e-8, agg)
    t = time.perf_counter() - t0
    return {"step": i, "s": t, "iterations": p.nIterations, "final_residual": p.finalResidual,
            "converged": bool(p.converged)}


def _mem_available():
    try:
        with open("/proc/meminfo") as fh:
            for line in fh:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) * 1024
    except OSError:
        pass
    return 0


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def run_reference(args, rank, world, pg):
    """The reference arm: the oracle (the reference's solver restated,
    bit-exact with its own build, compiled with its optimisation flags) on
    the host cores.  Every step is one complete serial solve of the headline
    system to 1e-8, timed directly; the warm-up and timed steps run
    concurrently, one process per host core (as many as the host memory
    holds), so the run ends within minutes.  Rank 0 alone runs it."""
    if rank != 0:
        return 0
    import multiprocessing as mp
    import shutil
    import tempfile
    tmp = tempfile.mkdtemp(prefix="cfx_ref_")
    try:
        path = os.path.join(tmp, "case.npz")
        t0 = time.perf_counter()
        subprocess.run([sys.executable, os.path.abspath(__file__), "--write-case", path, "--n", str(args.n)],
                       check=True)
        t_case = time.perf_counter() - t0
        case_bytes = os.path.getsize(path)
        cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
        # a solve holds the case, the agglomeration and coarse levels and its
        # vectors: 4.3x the case file measured at 128^3; budget 5x per process
        # and at most half the free host memory
        per_proc = 5 * case_bytes
        fit = max(1, int(0.5 * _mem_available() // per_proc)) if _mem_available() else 1
        nsteps = args.warmup + args.steps
        procs = max(1, min(cores, nsteps, fit))
        ctx = mp.get_context("spawn")
        t0 = time.perf_counter()
        with ctx.Pool(procs) as pool:
            res = pool.starmap(reference_step, [(path, i) for i in range(nsteps)])
        wall = time.perf_counter() - t0
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    timed = [r for r in res if r["step"] >= args.warmup]
    v = statistics.median(r["s"] for r in timed)
    sample = (f"oracle/ldu_oracle.c GAMG (serial C restatement of GAMGSolver, bit-exact with the reference "
              f"built from source; -O3 with the reference's flags): each of the {nsteps} steps is one complete "
              f"solve from psi=0 to 1e-8 at {args.n}^3, run {procs} at a time on {cores} host cores "
              f"(value = median of the {len(timed)} timed steps; {wall:.0f} s wall); the reference is serial "
              f"(no MPI on this host)")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": v * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": workload(args.n),
            "cpu_baseline": {"value": v, "unit": "s", "cores": procs, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "detail": {"steps": res, "case_write_s": t_case, "concurrent_processes": procs,
                       "wall_s": wall, "min_s": min(r["s"] for r in timed), "max_s": max(r["s"] for r in timed),
                       "iterations": sorted({r["iterations"] for r in res}),
                       "converged": all(r["converged"] for r in res)}}
    print(json.dumps(line), flush=True)
    return 0


def gs_sweeps(level):
    """Gauss-Seidel sweeps of a V-cycle smoothing on a level (0 = the mesh):
    nFinestSweeps 2 on the finest; nPre/PostSweeps 2 plus one per coarser
    level, at most 4 (GAMGSolver.C:70-80, GAMGSolverSolve.C)."""
    return 2 if level == 0 else min(2 + (level - 1), 4)


def gs_bytes(N, F, s=8):
    """Algorithmic bytes of one Gauss-Seidel sweep: 7sN + sF + 4F + 4N."""
    return 7 * s * N + s * F + 4 * F + 4 * N


# GB300's FP64 rate: 1.25 TFLOP/s nominal counting a fused multiply-add as
# two, i.e. 0.625e12 FP64 instructions/s.  The products here are not
# contracted (the reference's rounding), so every multiply and every add is
# one FP64 instruction.
FP64_OPS_PEAK = 0.625e12


def fp64_ops(kernel, N, F):
    """FP64 instructions of one Amul (diag*x, then a multiply and an add per
    off-diagonal entry: 2F entries) or residual (b - diag*x, then a multiply
    and a subtract per entry)."""
    base = kernel.split("_")[0]
    return (N if base == "amul" else 2 * N) + 2 * 2 * F


def level_sweeps(ctx, mesh, A, N, F, ev_time, local, smem_cells):
    """Every GAMG level's smoothing timed alone (FP64, the V-cycle's sweep
    count): each coarse level's matrix, assembled on the device, read back
    and swept through its own cfx_smooth, CUDA events on the library's
    stream.  Returns one row per level with its algorithmic bytes and GB/s."""
    import torch
    from openfoam_dev_gb300 import ldu
    rows = []
    nc_prev, nf_prev = N, F
    levels = [(0, N, F, None, None)]
    for i in range(mesh.n_levels()):
        _, _, _, nc, ncf, cl, cu = mesh.level(i, nc_prev, nf_prev)
        levels.append((i + 1, nc, ncf, cl, cu))
        nc_prev, nf_prev = nc, ncf
    rng = np.random.default_rng(7)
    for lv, nc, ncf, cl, cu in levels:
        S = gs_sweeps(lv)
        if lv == 0:
            Al, ml = A, None
        else:
            d, up, _ = A.coarse(lv, nc, ncf)
            ml = ldu.LduMesh(ctx, nc, cl, cu)
            Al = ldu.LduMatrix(ml, d, up)
        b = torch.from_numpy(rng.uniform(-1, 1, nc)).to(f"cuda:{local}")
        x = torch.zeros_like(b)
        t = ev_time(lambda: Al.smooth("GaussSeidel", x, b, S))
        by = S * gs_bytes(nc, ncf)
        # the form the library picks: one CTA when the vector fits its shared
        # memory, else the dataflow form for the hexahedral finest level (at
        # most 8 entries per slot) and the level-counter grid for the
        # agglomerated levels (more entries per slot)
        form = ("one CTA, vector in shared memory" if nc <= smem_cells
                else "dataflow" if lv == 0 else "persistent grid")
        rows.append({"level": lv, "cells": nc, "faces": ncf, "sweeps": S, "s": t, "algorithmic_bytes": by,
                     "GB_s": by / t / 1e9, "form": form})
        if ml is not None:
            Al.close()
            ml.close()
    return rows


FORM_NAMES = {0: "one CTA, vector in shared memory", 1: "cluster, distributed shared memory",
              2: "one CTA, vector in global memory", 3: "cluster, global memory", 4: "persistent grid",
              5: "dataflow", 6: "one launch per level"}


def level_sweeps_f32(ctx, mesh, A, N, F, ev_time, local):
    """Every GAMG level's smoothing as the FP32 inner cycles of the mixed
    solve apply it (multicolour Gauss-Seidel on the FP32 coefficient copy,
    the V-cycle's sweep count), each level's matrix alone through
    cfx_diag_smooth_f32, CUDA events on the library's stream.  Algorithmic
    bytes with 4-byte values: 7sN + sF + 4F + 4N per sweep, s = 4."""
    import torch
    from openfoam_dev_gb300 import ldu
    rows = []
    nc_prev, nf_prev = N, F
    levels = [(0, N, F, None, None)]
    for i in range(mesh.n_levels()):
        _, _, _, nc, ncf, cl, cu = mesh.level(i, nc_prev, nf_prev)
        levels.append((i + 1, nc, ncf, cl, cu))
        nc_prev, nf_prev = nc, ncf
    rng = np.random.default_rng(7)
    for lv, nc, ncf, cl, cu in levels:
        S = gs_sweeps(lv)
        if lv == 0:
            Al, ml = A, None
        else:
            d, up, _ = A.coarse(lv, nc, ncf)
            ml = ldu.LduMesh(ctx, nc, cl, cu)
            Al = ldu.LduMatrix(ml, d, up)
        b = torch.from_numpy(rng.uniform(-1, 1, nc).astype(np.float32)).to(f"cuda:{local}")
        x = torch.zeros_like(b)
        form = Al.smooth_f32("GaussSeidel", x, b, S)
        t = ev_time(lambda: Al.smooth_f32("GaussSeidel", x, b, S))
        by = S * gs_bytes(nc, ncf, s=4)
        rows.append({"level": lv, "cells": nc, "faces": ncf, "sweeps": S, "s": t, "algorithmic_bytes": by,
                     "GB_s": by / t / 1e9, "form": FORM_NAMES.get(form, str(form))})
        if ml is not None:
            Al.close()
            ml.close()
    return rows


def run_ours(args, rank, world, local, pg):
    # the oracle legs start first, in spawned processes, before any GPU call
    cpu = not args.no_cpu_baseline and world == 1 and rank == 0
    pool, jobs, outdir = None, {}, None
    if cpu:
        import multiprocessing as mp
        import tempfile
        outdir = tempfile.mkdtemp(prefix="cfx_oracle_")
        pool = mp.get_context("spawn").Pool(2)
        jobs["gamg"] = pool.apply_async(oracle_job, ("gamg", args.n, 1, outdir))
        jobs["pcg"] = pool.apply_async(oracle_job, ("pcg", 64, 1, outdir))
        jobs["bicgstab"] = pool.apply_async(oracle_job, ("bicgstab", 128, 1, outdir))
    import torch
    torch.cuda.set_device(local)
    ge.load_package()
    from openfoam_dev_gb300 import cases, ldu
    n = args.n
    s = cases.gamg_cube(n, jitter=0.2, seed=1 + rank)
    ctx = ldu.Context(local)
    mesh = ldu.LduMesh(ctx, s["diag"].size, s["l"], s["u"])
    A = ldu.LduMatrix(mesh, s["diag"], s["upper"])
    mesh.agglomerate(Sf=s["Sf"], nCellsInCoarsestLevel=10)
    stream = torch.cuda.ExternalStream(ctx.stream())
    N, F = s["diag"].size, s["l"].size
    d_src = torch.from_numpy(s["source"]).to(f"cuda:{local}")
    d_psi = torch.zeros_like(d_src)
    torch.cuda.synchronize()
    mixed = ldu.solver_new("T", A, dict(GAMG, precision="mixed"))
    fp64 = ldu.solver_new("T", A, dict(GAMG, precision="FP64"))

    def device_solve(solver):
        with torch.cuda.stream(stream):
            d_psi.zero_()
        return solver.solve(d_psi, d_src)

    def timed(solver, steps):
        evs = []
        perf = None
        for _ in range(steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            perf = device_solve(solver)
            e1.record(stream)
            evs.append((e0, e1))
        torch.cuda.synchronize()
        return [a.elapsed_time(b) / 1e3 for a, b in evs], perf

    for _ in range(args.warmup):
        device_solve(mixed)
        device_solve(fp64)
    torch.cuda.synchronize()

    barrier(pg)
    torch.cuda.synchronize()
    launches0 = ctx.launch_count()
    with Clocks(local) as clk:
        t_mixed, p_mixed = timed(mixed, args.steps)
    launches = ctx.launch_count() - launches0
    torch.cuda.synchronize()
    psi_mixed = d_psi.cpu().numpy()
    barrier(pg)
    t_fp64, p_fp64 = timed(fp64, args.steps)
    psi_fp64 = d_psi.cpu().numpy()
    barrier(pg)

    # e2e: what a plugin does per fvMatrix::solve, host buffers (pinned)
    pin = lambda a: torch.from_numpy(a).pin_memory().numpy()  # noqa: E731
    h_diag, h_upper, h_src = pin(s["diag"]), pin(s["upper"]), pin(s["source"])
    h_psi = torch.zeros(N, dtype=torch.float64).pin_memory().numpy()
    e2e = []
    for i in range(args.warmup + args.steps):
        h_psi[:] = 0.0
        t0 = time.perf_counter()
        A.update(h_diag, h_upper)
        mixed.solve(h_psi, h_src)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            e2e.append(dt)

    def ev_time(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        out = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            out.append((e0, e1))
        torch.cuda.synchronize()
        return statistics.median([a.elapsed_time(b) / 1e3 for a, b in out])

    # every level's smoothing alone (FP64): the dominant kernels by device
    # time are the Gauss-Seidel sweeps of the agglomerated levels
    smem_cells = ldu.tune_get(ldu.TUNE_SMEM_BYTES) // 8
    levels = level_sweeps(ctx, mesh, A, N, F, ev_time, local, smem_cells)
    # the mixed solve's smoothing (FP32 inner cycles): its dominant kernel
    levels32 = level_sweeps_f32(ctx, mesh, A, N, F, ev_time, local)

    # the streaming kernels of the path (HBM-bound, no level chain), FP64 at
    # the same size, each timed alone: Amul (3sN + 2sF), residual
    # (4sN + 2sF); rows read from the sliced ELL copy (the default) and,
    # for comparison, through the losort/owner gathers
    d_b = d_src.clone()
    d_y = torch.empty_like(d_src)
    streaming = {
        "amul": (ev_time(lambda: A.Amul(d_b, d_y)), 3 * 8 * N + 8 * F + 8 * F),
        "residual": (ev_time(lambda: A.residual(d_b, d_src, d_y)), 4 * 8 * N + 8 * F + 8 * F),
    }
    sell_was = ldu.tune_get(ldu.TUNE_AMUL_SELL)
    ldu.tune_set(ldu.TUNE_AMUL_SELL, 0)
    try:
        streaming["amul_gather"] = (ev_time(lambda: A.Amul(d_b, d_y)), 3 * 8 * N + 8 * F + 8 * F)
        streaming["residual_gather"] = (ev_time(lambda: A.residual(d_b, d_src, d_y)), 4 * 8 * N + 8 * F + 8 * F)
    finally:
        ldu.tune_set(ldu.TUNE_AMUL_SELL, sell_was)

    assembly = fvm_assembly_measure(ctx, ev_time, stream, local) if world == 1 else None
    krylov, krylov_psi = krylov_configs(ctx, stream, local) if world == 1 else (None, None)

    tm = reduce_max(pg, statistics.median(t_mixed))
    t64 = reduce_max(pg, statistics.median(t_fp64))
    te = reduce_max(pg, statistics.median(e2e))
    if rank != 0:
        return 0
    peaks = {}
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as fh:
            peaks = json.load(fh)
    except OSError:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    # roofline: the kernel with the largest share of the headline (mixed)
    # solve's device time, sweep_level_k<float>: the FP32 multicolour
    # Gauss-Seidel smoothing of the levels that run one launch per DAG level;
    # bytes and time summed over those levels' smoothings = average bytes per
    # smoothing / average smoothing time
    dom = [r for r in levels32 if r["form"] == FORM_NAMES[6]]
    dom_bytes = sum(r["algorithmic_bytes"] for r in dom)
    dom_time = sum(r["s"] for r in dom)
    achieved = dom_bytes / dom_time / 1e9 if dom else 0.0
    # the same for the FP64 solve's dominant kernels (the agglomerated
    # levels' persistent-grid sweeps)
    dom64 = [r for r in levels if r["level"] > 0 and r["form"] == "persistent grid"]
    dom64_bytes = sum(r["algorithmic_bytes"] for r in dom64)
    dom64_time = sum(r["s"] for r in dom64)
    cycle_sweeps = 2 * sum(r["s"] for r in levels)  # pre and post smoothing per V-cycle
    traffic = traffic64 = None
    try:
        with open(os.path.join(REPO, "profiles", "traffic.json")) as fh:
            tr = json.load(fh)
        per_byte = tr.get("gs_level_f32_dram_per_algorithmic_byte")
        if per_byte and dom:
            traffic = per_byte * dom_bytes / len(dom)
        per_byte64 = tr.get("gs_coarse_dram_per_algorithmic_byte")
        if per_byte64 and dom64:
            traffic64 = per_byte64 * dom64_bytes / len(dom64)
    except (OSError, ValueError):
        pass
    for r in levels + levels32:
        r["frac"] = r["GB_s"] / peak
    line = {"metric": METRIC, "value": tm, "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tm * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32-inner/f64-refined", "data": "synthetic (seeded)",
            "config": workload(n), "parallelism": "replicas" if world > 1 else "1 GPU",
            "fp64_time_s": t64, "mixed_speedup": t64 / tm,
            "recommended_precision": "mixed" if t64 / tm > 1.0 else "FP64", "v_cycles_mixed": p_mixed.nIterations,
            "v_cycles_fp64": p_fp64.nIterations, "final_residual_mixed": p_mixed.finalResidual,
            "final_residual_fp64": p_fp64.finalResidual,
            "e2e": {"value": te, "unit": "s", "h2d_bytes_per_step": 8 * (N + F) + 16 * N,
                    "d2h_bytes_per_step": 8 * N},
            "gpu_launches": int(launches),
            "streaming_kernels": {k: {"s": t, "algorithmic_bytes": b, "GB_s": b / t / 1e9, "frac": b / t / 1e9 / peak,
                                      "fp64_ops": fp64_ops(k, N, F),
                                      "fp64_Gops_s": fp64_ops(k, N, F) / t / 1e9,
                                      "fp64_pipe_frac": fp64_ops(k, N, F) / t / FP64_OPS_PEAK}
                                  for k, (t, b) in streaming.items()},
            "roofline": {"bound": "hbm",
                         "kernel": "sweep_level_k<float>: the FP32 inner cycles' multicolour Gauss-Seidel "
                                   "smoothing, one launch per DAG level "
                                   f"(levels {', '.join(str(r['level']) for r in dom)}, the V-cycle's sweep counts; "
                                   "bytes and time per level smoothing)" if dom else "none",
                         "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "algorithmic_bytes_per_launch": dom_bytes / max(len(dom), 1),
                         "launch_s": dom_time / max(len(dom), 1), "launches": len(dom),
                         "peak_source": "measured" if "hbm_gbs" in peaks else "fallback"},
            "roofline_fp64": {"bound": "hbm",
                              "kernel": "sweep_grid_k<double>: the FP64 solve's Gauss-Seidel sweeps of the "
                                        "agglomerated levels, persistent grid form (levels "
                                        f"{dom64[0]['level']}-{dom64[-1]['level']})" if dom64 else "none",
                              "achieved": dom64_bytes / dom64_time / 1e9 if dom64 else 0.0, "peak": peak,
                              "unit": "GB/s",
                              "frac": dom64_bytes / dom64_time / 1e9 / peak if dom64 else 0.0,
                              "traffic": traffic64,
                              "algorithmic_bytes_per_launch": dom64_bytes / max(len(dom64), 1),
                              "launch_s": dom64_time / max(len(dom64), 1), "launches": len(dom64)},
            "gamg_levels_fp64": levels,
            "gamg_levels_f32_inner": levels32,
            "v_cycle_fp64_s": t64 / max(p_fp64.nIterations, 1),
            "v_cycle_smoothing_fp64_s": cycle_sweeps,
            "clocks": clk.summary()}
    if assembly:
        assembly["frac"] = assembly["GB_s"] / peak
        line["assembly"] = assembly
    if krylov:
        for v in krylov.values():
            v["FP64"]["frac"] = v["FP64"]["GB_s"] / peak
        line["krylov"] = krylov
    if cpu:
        res = {k: j.get() for k, j in jobs.items()}
        pool.close()
        pool.join()
        g = res["gamg"]
        line["parity"] = parity_of(g, outdir, psi_fp64, p_fp64.nIterations, psi_mixed)
        line["cpu_baseline"] = {
            "value": g["s"], "unit": "s", "cores": 1, "kind": "port",
            "sample": f"oracle GAMG (serial C restatement of GAMGSolver, bit-exact with the reference build, "
                      f"-O3 with the reference's flags) at {n}^3: one complete solve from psi=0 to 1e-8 "
                      f"({g['iterations']} V-cycles), timed directly, agglomeration ({g['agglomeration_s']:.1f} s, "
                      f"cached per mesh as in the reference) excluded",
            "detail": g}
        if krylov:
            for name, key in (("pcg_dic_64", "pcg"), ("pbicgstab_dilu_128", "bicgstab")):
                r = res[key]
                k = krylov[name]
                k["parity"] = parity_of(r, outdir, krylov_psi[name]["FP64"], k["FP64"]["iterations"],
                                        krylov_psi[name]["mixed"])
                k["cpu_baseline"] = {"value": r["s"], "unit": "s", "cores": 1, "kind": "port",
                                     "iterations": r["iterations"],
                                     "sample": "oracle, one complete solve to 1e-8, timed directly"}
                k["speedup_fp64_vs_cpu"] = r["s"] / k["FP64"]["s"]
        import shutil
        shutil.rmtree(outdir, ignore_errors=True)
    if world == 1 and args.workload == "all":
        line.update(run_batch_serve(args, local, True, True))
    print(json.dumps(line), flush=True)
    return 0


def krylov_configs(ctx, stream, local, reps=3):
    """The Krylov configurations: PCG+DIC on the uniform 64^3 cube and
    PBiCGStab+DILU on the 128^3 jittered, permuted-then-CM-renumbered upwind
    system, each to 1e-8 in FP64 and FP32-inner/FP64-refined, resident
    vectors, CUDA events on the library's stream (median of reps).  GB/s:
    the per-iteration algorithmic bytes (PCG+DIC 23sN + 3sF + 24F,
    PBiCGStab+DILU 41sN + 8sF + 56F, s = 8) times the iterations, over the
    solve time.  Returns the measurements and each precision's solution
    (host arrays, for the parity against the oracle)."""
    import torch
    from openfoam_dev_gb300 import cases, ldu
    out, sols = {}, {}
    for name, s, ctl, per_iter in (
            ("pcg_dic_64", cases.pcg_cube(64, seed=1),
             {"solver": "cudaPCG", "preconditioner": "DIC", "tolerance": 1e-8, "relTol": 0, "maxIter": 2000},
             lambda N, F: 23 * 8 * N + 3 * 8 * F + 24 * F),
            ("pbicgstab_dilu_128", cases.bicgstab_cube(128, seed=1),
             {"solver": "cudaPBiCGStab", "preconditioner": "DILU", "tolerance": 1e-8, "relTol": 0,
              "maxIter": 2000},
             lambda N, F: 41 * 8 * N + 8 * 8 * F + 56 * F)):
        mesh = ldu.LduMesh(ctx, s["diag"].size, s["l"], s["u"])
        A = ldu.LduMatrix(mesh, s["diag"], s["upper"], s.get("lower"))
        N, F = s["diag"].size, s["l"].size
        src = torch.from_numpy(s["source"]).to(f"cuda:{local}")
        psi = torch.zeros_like(src)
        res = {"cells": N, "faces": F, "bytes_per_iteration": per_iter(N, F)}
        sols[name] = {}
        for prec in ("FP64", "mixed"):
            sol = ldu.solver_new("x", A, dict(ctl, precision=prec))
            ts, perf = [], None
            for r in range(reps + 1):
                with torch.cuda.stream(stream):
                    psi.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                perf = sol.solve(psi, src)
                e1.record(stream)
                torch.cuda.synchronize()
                if r:
                    ts.append(e0.elapsed_time(e1) / 1e3)
            t = statistics.median(ts)
            sols[name][prec] = psi.cpu().numpy()
            res[prec] = {"s": t, "iterations": perf.nIterations, "final_residual": perf.finalResidual,
                         "converged": bool(perf.converged)}
            if prec == "FP64":
                res[prec]["GB_s"] = per_iter(N, F) * perf.nIterations / t / 1e9
        res["mixed_speedup"] = res["FP64"]["s"] / res["mixed"]["s"]
        # the precision a drop-in user should pick for this solver: both
        # reach the tolerance, so the faster one
        res["recommended_precision"] = "mixed" if res["mixed_speedup"] > 1.0 else "FP64"
        out[name] = res
        A.close()
        mesh.close()
    return out, sols


def fvm_assembly_measure(ctx, ev_time, stream, local, n=128):
    """Device-side assembly of a transport equation (ddt + upwind div -
    laplacian(face gamma) == su) on an n^3 jittered box, against the host
    upload of the same coefficients that it replaces (pinned buffers)."""
    import torch
    from openfoam_dev_gb300 import cases, ldu
    m = cases.box_mesh(n, n, n, jitter=0.2, seed=3)
    g = cases.fv_geometry(m)
    nI, nB, N = m["nInternalFaces"], g["bCell"].size, m["nCells"]
    mesh = ldu.LduMesh(ctx, N, m["owner"][:nI], m["neighbour"])
    mesh.fv_geometry(g["magSf"], g["deltaCoeffs"], g["V"], g["bCell"], g["magSfB"], g["deltaCoeffsB"],
                     weights=g["weights"])
    rng = np.random.default_rng(5)
    dev = lambda a, t=torch.float64: torch.as_tensor(a, device=f"cuda:{local}").to(t)  # noqa: E731
    f = dict(psi0=dev(rng.uniform(-1, 1, N)), phi=dev(rng.uniform(-1, 1, nI)), phiB=dev(rng.uniform(-1, 1, nB)),
             gamma=dev(rng.uniform(0.01, 0.1, nI)), gammaB=dev(rng.uniform(0.01, 0.1, nB)),
             bcType=dev(np.ones(nB, np.int32), torch.int32), bcValue=dev(rng.uniform(-1, 1, nB)),
             su=dev(rng.uniform(-1, 1, N)))
    A = ldu.LduMatrix.empty(mesh, symmetric=False)
    src = torch.empty(N, dtype=torch.float64, device=f"cuda:{local}")
    t_asm = ev_time(lambda: A.assemble(src, rDeltaT=10.0, lapSign=-1, div="upwind", **f))
    # the upload a plugin does instead: diag, upper, lower and the source
    pin = lambda a: torch.from_numpy(a).pin_memory().numpy()  # noqa: E731
    h = [pin(rng.uniform(-1, 1, N)), pin(rng.uniform(-1, 1, nI)), pin(rng.uniform(-1, 1, nI))]
    h_src = torch.from_numpy(rng.uniform(-1, 1, N)).pin_memory()

    def upload():
        A.update(*h)
        with torch.cuda.stream(stream):
            src.copy_(h_src, non_blocking=True)

    t_up = ev_time(upload)
    # algorithmic bytes: per internal face phi, gamma, magSf, deltaCoeffs in,
    # upper, lower out, l/u; per cell V, psi0, su in, diag, source out, the
    # two addressing offsets; per boundary face phiB, gammaB, magSfB,
    # deltaCoeffsB, bcValue, bcType, cell
    alg = 8 * 6 * nI + 4 * 2 * nI + 8 * 5 * N + 4 * 2 * N + (8 * 5 + 4 + 4) * nB
    A.close()
    mesh.close()
    return {"workload": f"fvm::ddt + fvm::div(phi) upwind - fvm::laplacian(face gamma) == su, {n}^3 jittered box, "
                        f"fixedValue patches ({N} cells, {nI} internal faces)",
            "s": t_asm, "algorithmic_bytes": alg, "GB_s": alg / t_asm / 1e9,
            "host_upload_s": t_up, "upload_bytes": 8 * (N + 2 * nI) + 8 * N,
            "speedup_vs_upload": t_up / t_asm}


def cpu_batch_sample(count, seed=1, per_core=2):
    """Oracle PCG+DIC (serial C restatement) on an even sample of the batch,
    one process per host core: solves/s of the host cores."""
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    k = min(count, per_core * cores)
    idx = [int(round(i * (count - 1) / max(k - 1, 1))) for i in range(k)]
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        res = pool.starmap(_cpu_batch_one, [(seed, count, i) for i in idx])
    wall = time.perf_counter() - t0
    return {"value": k / wall, "unit": "solves/s", "cores": cores, "kind": "port",
            "sample": f"{k} of the {count} systems (evenly spaced), oracle PCG+DIC FP64 to 1e-8, one process per "
                      f"core; {wall:.1f} s wall, {sum(r[1] for r in res):.1f} s of CPU work",
            "converged": all(r[0] for r in res)}


def _cpu_batch_one(seed, count, i):
    ge.load_package()
    from oracle import oracle as orc
    from openfoam_dev_gb300 import cases
    nx, ny, nz, f, sd = cases.batch_boxes(count, seed=seed)[i]
    s = cases.box(nx, ny, nz, dirichlet=f, seed=sd)
    x = np.zeros(s["diag"].size)
    t0 = time.process_time()
    p = orc.pcg(s, x, tol=1e-8, max_iter=2000)
    return bool(p.converged), time.process_time() - t0


def run_batch_serve(args, local, want_batch, want_serve):
    """The batched (512 independent systems) and serving measurements."""
    import torch
    ge.load_package()
    from openfoam_dev_gb300 import cases, ldu, loadgen
    out = {}
    ctx = ldu.Context(local)
    if want_batch:
        systems = loadgen.batch_systems(args.batch_count, seed=1)
        b = {"workload": f"{args.batch_count} independent PCG+DIC Laplacian box systems (cells log-uniform in "
                         f"[4096, 500000], aspect U[1,4], Dirichlet on one seeded face), tolerance 1e-8, one "
                         f"persistent launch, autotuned packing"}
        for prec in ("mixed", "FP64"):
            b[prec] = loadgen.bench_batch(ctx, systems, steps=args.steps, warmup=1, precision=prec)
        del systems
        if not args.no_cpu_baseline:
            b["cpu_baseline"] = cpu_batch_sample(args.batch_count)
        out["batch"] = b
    if want_serve:
        pool = loadgen.batch_systems(64, seed=5)
        large = cases.gamg_cube(args.serve_large, jitter=0.2, seed=9)
        sv = ldu.Server(ctx)
        mix = loadgen.ServeMix(sv, pool, large, resident=16, seed=3)
        srv = {"workload": f"Poisson arrivals: 90% batch-like systems (30% of all requests re-solve one of 16 "
                           f"resident matrices with a new source; the rest register one of 64 pool systems, "
                           f"solve, remove), 10% GAMG on a {args.serve_large}^3 jittered cube "
                           f"({args.serve_large ** 3} cells, resident); HBM budget "
                           f"{sv.config.hbmBudget / 1e9:.0f} GB"}
        for prec in ("mixed", "FP64"):
            mix.run(mix.draw(), prec)  # warm the drivers
            mix.run(("large", None, 1), prec)
            un = loadgen.serve_unloaded(mix, 48, prec)
            t_large = un["by_kind_p50_ms"].get("large", 1000.0) / 1e3
            t_small = un["by_kind_p50_ms"].get("resident", 10.0) / 1e3
            # requests/s the GPU could take if nothing overlapped
            capacity = 1.0 / (0.1 * t_large + 0.9 * t_small)
            r = {"unloaded": un, "capacity_estimate_per_s": capacity}
            rate = args.serve_rate
            if not rate:
                rate = 0.3 * capacity
                if args.serve_sweep_duration > 0:
                    sweep = []
                    for f in (0.3, 0.5, 0.7):
                        q = loadgen.serve_stream(mix, f * capacity, args.serve_sweep_duration, prec)
                        q["by_kind_ratio"], q["worst_kind_p99_over_unloaded_p99"] = loadgen.per_kind_ratio(q, un)
                        sweep.append(q)
                        if q["worst_kind_p99_over_unloaded_p99"] is not None and \
                                q["worst_kind_p99_over_unloaded_p99"] <= 2.0:
                            rate = f * capacity
                    r["sweep"] = sweep
            # the long stream; a 10 s sweep window sees few tail requests, so
            # when the long stream misses the 2x target at the chosen rate it
            # runs once more at 0.7x that rate (both kept)
            attempts = []
            for _ in range(2):
                q = loadgen.serve_stream(mix, rate, args.serve_duration, prec)
                q["by_kind_ratio"], q["worst_kind_p99_over_unloaded_p99"] = loadgen.per_kind_ratio(q, un)
                q["p99_over_unloaded_p99_all"] = q["p99_ms"] / un["p99_ms"]
                attempts.append(q)
                w = q["worst_kind_p99_over_unloaded_p99"]
                if args.serve_rate or w is None or w <= 2.0:
                    break
                rate *= 0.7
            r["stream"] = attempts[-1]
            if len(attempts) > 1:
                r["stream_attempts"] = attempts[:-1]
            r["sustained_solves_per_s"] = attempts[-1]["solves_per_s"]
            srv[prec] = r
        sv.close()
        out["serve"] = srv
    ctx.close()
    torch.cuda.synchronize()
    return out


def run_kernel_only(args):
    """One Gauss-Seidel smoothing alone, warmup + steps times (for profiling
    under ncu): gs = the finest level's fused 2 sweeps, level1 = the first
    agglomerated level's (the persistent grid form, the V-cycle's 2 sweeps);
    gs32 / level1_32 = the same levels' FP32 inner-cycle smoothing
    (multicolour order, one launch per DAG level)."""
    import torch
    ge.load_package()
    from openfoam_dev_gb300 import cases, ldu
    if args.form != "default":
        ldu.tune_set(ldu.TUNE_FLOW, int(args.form == "flow"))
    s = cases.gamg_cube(args.n, jitter=0.2, seed=1)
    mesh, A = ldu.system_matrix(s)
    N, F = s["diag"].size, s["l"].size
    if args.kernel_only == "solves":
        mesh.agglomerate(Sf=s["Sf"], nCellsInCoarsestLevel=10)
        d_src = torch.from_numpy(s["source"]).cuda()
        d_psi = torch.zeros_like(d_src)
        torch.cuda.synchronize()
        sol = {p: ldu.solver_new("T", A, dict(GAMG, precision=p)) for p in ("FP64", "mixed")}
        out = {}
        # the second solve of each precision runs inside the NVTX range
        # profiled_fp64 / profiled_mixed (ncu --nvtx-include selects one)
        for prof in (False, True):
            for p in ("FP64", "mixed"):
                d_psi.zero_()
                torch.cuda.synchronize()
                if prof:
                    torch.cuda.nvtx.range_push("profiled_" + p.lower())
                t0 = time.perf_counter()
                perf = sol[p].solve(d_psi, d_src)
                torch.cuda.synchronize()
                out[p] = {"s": time.perf_counter() - t0, "v_cycles": perf.nIterations}
                if prof:
                    torch.cuda.nvtx.range_pop()
        print(json.dumps({"kernel": "solves", "n": args.n, **out}), flush=True)
        return 0
    if args.kernel_only == "amul":
        # cfx_amul and cfx_residual run in FP64 (the FP32 copies of the
        # coefficients are reached only inside mixed-precision solves)
        d_b = torch.from_numpy(np.random.default_rng(7).uniform(-1, 1, N)).cuda()
        d_y = torch.empty_like(d_b)
        torch.cuda.synchronize()
        t = {}
        for name, fn in (("amul", lambda: A.Amul(d_b, d_y)), ("residual", lambda: A.residual(d_b, d_b, d_y))):
            ts = []
            for i in range(args.warmup + args.steps):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                fn()
                torch.cuda.synchronize()
                if i >= args.warmup:
                    ts.append(time.perf_counter() - t0)
            t[name] = statistics.median(ts)
        print(json.dumps({"kernel": "amul", "n": args.n, "cells": N, "faces": F, **t}), flush=True)
        return 0
    if args.kernel_only in ("level1", "level1_32"):
        mesh.agglomerate(Sf=s["Sf"], nCellsInCoarsestLevel=10)
        _, _, _, nc, ncf, cl, cu = mesh.level(0, N, F)
        d, up, _ = A.coarse(1, nc, ncf)
        mesh = ldu.LduMesh(mesh.ctx, nc, cl, cu)
        A = ldu.LduMatrix(mesh, d, up)
        N, F = nc, ncf
    f32 = args.kernel_only.endswith("32")
    d_b = torch.from_numpy(np.random.default_rng(7).uniform(-1, 1, N)).cuda()
    if f32:
        d_b = d_b.float()
    d_x = torch.zeros_like(d_b)
    torch.cuda.synchronize()
    t = []
    form = None
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if f32:
            form = A.smooth_f32("GaussSeidel", d_x, d_b, 2)
        else:
            A.smooth("GaussSeidel", d_x, d_b, 2)
        torch.cuda.synchronize()
        if i >= args.warmup:
            t.append(time.perf_counter() - t0)
    print(json.dumps({"kernel": args.kernel_only, "n": args.n, "cells": N, "faces": F,
                      "algorithmic_bytes": 2 * gs_bytes(N, F, s=4 if f32 else 8), "s": statistics.median(t),
                      "form": FORM_NAMES.get(form) if f32 else None}), flush=True)
    return 0


def main():
    args = parse()
    if args.write_case:
        write_case(args.write_case, args.n)
        return 0
    if args.kernel_only:
        return run_kernel_only(args)
    rank, world, local, pg = dist()
    if args.impl == "ours" and args.workload in ("batch", "serve"):
        import torch
        torch.cuda.set_device(local)
        extra = run_batch_serve(args, local, args.workload == "batch", args.workload == "serve")
        print(json.dumps(dict(extra, workload=args.workload)), flush=True)
        return 0
    if args.impl == "reference":
        rc = run_reference(args, rank, world, pg)
    else:
        rc = run_ours(args, rank, world, local, pg)
    if pg is not None:
        pg.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
