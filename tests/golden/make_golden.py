"""Write the golden fixtures of tests/golden/ from the reference itself.

Run in a container where the OpenFOAM-dev sources are mounted and
``python oracle/build_ref.py`` has built oracle/_ref (libOpenFOAM.so and the
harness).  Every fixture is produced by the reference's own code:

* geom_*.npz   polyMesh face areas/centres and cell centres/volumes of a
               jittered hex box (primitiveMesh geometry)
* ops_*.npz    lduMatrix::Amul/Tmul/residual/sumA, normFactor, gSum*, the
               DIC/DILU reciprocal diagonals and preconditioners, the
               GaussSeidel, symGaussSeidel, DIC, DILU, DICGaussSeidel and
               DILUGaussSeidel smoothers, lduAddressing losort/ownerStart
* solve_*.npz  lduMatrix::solver::New(...)->solve for PCG, PBiCGStab, GAMG
               (with the agglomeration levels and coarse matrices) and
               smoothSolver with each smoother of the run-time table
* fvm_*.npz    finiteVolume's fvm::ddt + fvm::div +/- fvm::laplacian == su
               on a jittered hex box (oracle/fv_harness, linked against the
               reference's libfiniteVolume): the inputs (in_*), the geometry
               the schemes used, and the diag/upper/lower/source handed to
               the solver
* fvsolve_*.npz  fvMatrix::solve of those equations on a larger box (GAMG
               with faceAreaPair on the fvMesh, PCG with GAMG, PCG, PBiCGStab,
               smoothSolver): psi, the solver performance, GAMG's levels and
               a digest of the assembled matrix
* fvcyc_*.npz  fvMatrix::solve with a cyclic patch pair (the reference's own
               cyclicPolyPatch / cyclicFvPatchField, GAMG's cyclicGAMGInterface):
               the lduMatrix and interfaces the solver received and its results

Inputs are regenerated by the tests from the stored case parameters with
openfoam-dev_gb300/cases.py; their checksums are stored to catch drift.

Usage:  python tests/golden/make_golden.py
        (flux_fvsolve.npz alone, on the machine that made the fvsolve
        fixtures: python tests/golden/make_golden.py --fvsolve-inputs;
        some fvcyc_*.npz alone: python tests/golden/make_golden.py --fvcyc NAME...)
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

sys.path.insert(0, os.path.dirname(HERE))
import __graft_entry__ as ge  # noqa: E402

ge.load_package()
from openfoam_dev_gb300 import cases  # noqa: E402
from oracle import oracle as orc  # noqa: E402
from oracle import reference as ref  # noqa: E402
import golden_cases as gc  # noqa: E402

# Case specs: (kind, params).  Shared with tests/golden_cases.py via JSON.
SYSTEMS = {
    "cube6": ("pcg_cube", dict(n=6, seed=2)),
    "cube12": ("pcg_cube", dict(n=12, seed=2)),
    "jcube7": ("gamg_cube", dict(n=7, jitter=0.3, seed=3)),
    "jcube14": ("gamg_cube", dict(n=14, jitter=0.2, seed=5)),
    "jcube16": ("gamg_cube", dict(n=16, jitter=0.2, seed=9)),
    "cd6": ("bicgstab_cube", dict(n=6, seed=4)),
    "cd10": ("bicgstab_cube", dict(n=10, seed=4)),
    "box": ("box", dict(nx=9, ny=5, nz=13, dirichlet="zmax", seed=11)),
    # periodic in x: a cyclic interface pair (symmetric / upwind asymmetric)
    "cyc7": ("cyclic_cube", dict(n=7, jitter=0.2, seed=6)),
    "cycd7": ("cyclic_cube", dict(n=7, jitter=0.1, seed=8, U=[1.0, 0.4, 0.2], gamma=0.05)),
}

SOLVES = {
    "pcg_dic": ("cube12", dict(solver="PCG", preconditioner="DIC", tolerance=1e-8, relTol=0.0, maxIter=2000)),
    "pcg_diag": ("cube12", dict(solver="PCG", preconditioner="diagonal", tolerance=1e-8, relTol=0.0)),
    "pcg_none": ("box", dict(solver="PCG", preconditioner="none", tolerance=1e-7, relTol=0.0)),
    "pcg_reltol": ("jcube14", dict(solver="PCG", preconditioner="DIC", tolerance=0.0, relTol=1e-3)),
    "pcg_maxiter": ("jcube14", dict(solver="PCG", preconditioner="DIC", tolerance=1e-12, relTol=0.0, maxIter=7)),
    "pcg_miniter": ("cube6", dict(solver="PCG", preconditioner="DIC", tolerance=1.0, relTol=0.0, minIter=3)),
    "bicgstab_dilu": ("cd10", dict(solver="PBiCGStab", preconditioner="DILU", tolerance=1e-8, relTol=0.0,
                                   maxIter=2000)),
    "bicgstab_sym": ("jcube14", dict(solver="PBiCGStab", preconditioner="DIC", tolerance=1e-8, relTol=0.0)),
    "gamg_gs": ("jcube14", dict(solver="GAMG", smoother="GaussSeidel", tolerance=1e-8, relTol=0.0,
                                nCellsInCoarsestLevel=10)),
    "gamg_gs_pre": ("jcube16", dict(solver="GAMG", smoother="GaussSeidel", nPreSweeps=2, nPostSweeps=2,
                                    tolerance=1e-8, relTol=0.0, nCellsInCoarsestLevel=10)),
    "gamg_dic": ("jcube14", dict(solver="GAMG", smoother="DIC", tolerance=1e-8, relTol=0.0)),
    "gamg_box": ("box", dict(solver="GAMG", smoother="GaussSeidel", nPreSweeps=1, tolerance=1e-9, relTol=0.0,
                             nCellsInCoarsestLevel=4)),
    "smooth_gs": ("cube12", dict(solver="smoothSolver", smoother="GaussSeidel", tolerance=1e-6, relTol=0.0,
                                 maxIter=5000)),
    "smooth_symgs": ("jcube14", dict(solver="smoothSolver", smoother="symGaussSeidel", nSweeps=2,
                                     tolerance=1e-7, relTol=0.0, maxIter=5000)),
    "smooth_dic": ("cube12", dict(solver="smoothSolver", smoother="DIC", tolerance=1e-7, relTol=0.0,
                                  maxIter=5000)),
    "smooth_dicgs": ("jcube14", dict(solver="smoothSolver", smoother="DICGaussSeidel", tolerance=1e-7,
                                     relTol=0.0, maxIter=5000)),
    "smooth_dilu": ("cd10", dict(solver="smoothSolver", smoother="DILU", tolerance=1e-9, relTol=0.0)),
    "smooth_dilugs": ("cd10", dict(solver="smoothSolver", smoother="DILUGaussSeidel", nSweeps=2, tolerance=1e-9,
                                   relTol=0.0)),
    "smooth_symgs_asym": ("cd10", dict(solver="smoothSolver", smoother="symGaussSeidel", tolerance=1e-9,
                                       relTol=0.0)),
    "smooth_fixed": ("box", dict(solver="smoothSolver", smoother="symGaussSeidel", nSweeps=-5)),
    "smooth_maxiter": ("box", dict(solver="smoothSolver", smoother="GaussSeidel", nSweeps=3, tolerance=1e-12,
                                   relTol=0.0, maxIter=7)),
    "smooth_reltol": ("jcube14", dict(solver="smoothSolver", smoother="DICGaussSeidel", tolerance=0.0,
                                      relTol=1e-2)),
    "pcg_gamg": ("jcube16", dict(solver="PCG", tolerance=1e-8, relTol=0.0,
                                 preconditioner=dict(preconditioner="GAMG", smoother="GaussSeidel", nVcycles=2,
                                                     nCellsInCoarsestLevel=10))),
    "pcg_gamg_dicgs": ("jcube14", dict(solver="PCG", tolerance=1e-9, relTol=0.0,
                                       preconditioner=dict(preconditioner="GAMG", smoother="DICGaussSeidel",
                                                           nVcycles=1, nPreSweeps=1, tolerance=1e-4))),
    "gamg_interp": ("jcube14", dict(solver="GAMG", smoother="GaussSeidel", interpolateCorrection=True,
                                    tolerance=1e-8, relTol=0.0)),
    "gamg_interp_pre": ("jcube16", dict(solver="GAMG", smoother="DICGaussSeidel", nPreSweeps=2,
                                        interpolateCorrection=True, tolerance=1e-9, relTol=0.0)),
    "gamg_interp_asym": ("cd10", dict(solver="GAMG", smoother="GaussSeidel", nPreSweeps=1,
                                      interpolateCorrection=True, tolerance=1e-9, relTol=0.0)),
    "gamg_direct": ("jcube14", dict(solver="GAMG", smoother="GaussSeidel", directSolveCoarsest=True,
                                    tolerance=1e-8, relTol=0.0)),
    "gamg_direct_big": ("jcube16", dict(solver="GAMG", smoother="DIC", directSolveCoarsest=True,
                                        nCellsInCoarsestLevel=60, tolerance=1e-9, relTol=0.0)),
    "gamg_direct_asym": ("cd10", dict(solver="GAMG", smoother="GaussSeidel", directSolveCoarsest=True,
                                      tolerance=1e-9, relTol=0.0)),
    "pcg_fdic": ("jcube14", dict(solver="PCG", preconditioner="FDIC", tolerance=1e-9, relTol=0.0)),
    "bicgstab_fdic": ("cube6", dict(solver="PBiCGStab", preconditioner="FDIC", tolerance=1e-9, relTol=0.0)),
    "smooth_fdic": ("cube12", dict(solver="smoothSolver", smoother="FDIC", nSweeps=2, tolerance=1e-7,
                                   relTol=0.0, maxIter=5000)),
    "smooth_nbgs_asym": ("cd10", dict(solver="smoothSolver", smoother="nonBlockingGaussSeidel", tolerance=1e-9,
                                      relTol=0.0)),
    "gamg_nbgs": ("jcube14", dict(solver="GAMG", smoother="nonBlockingGaussSeidel", nPreSweeps=1,
                                  tolerance=1e-8, relTol=0.0)),
    "gamg_fdic": ("jcube16", dict(solver="GAMG", smoother="FDIC", tolerance=1e-9, relTol=0.0)),
    "pbicg_dilu": ("cd10", dict(solver="PBiCG", preconditioner="DILU", tolerance=1e-9, relTol=0.0,
                                maxIter=2000)),
    "pbicg_diagonal": ("cd6", dict(solver="PBiCG", preconditioner="diagonal", tolerance=1e-8, relTol=0.0,
                                   maxIter=2000)),
    "pbicg_none_reltol": ("cd6", dict(solver="PBiCG", preconditioner="none", tolerance=0.0, relTol=1e-4)),
    "pcg_cyc": ("cyc7", dict(solver="PCG", preconditioner="DIC", tolerance=1e-10, relTol=0.0)),
    "pcg_cyc_diagonal": ("cyc7", dict(solver="PCG", preconditioner="diagonal", tolerance=1e-9, relTol=0.0)),
    "bicgstab_cyc": ("cycd7", dict(solver="PBiCGStab", preconditioner="DILU", tolerance=1e-10, relTol=0.0)),
    "pbicg_cyc": ("cycd7", dict(solver="PBiCG", preconditioner="DILU", tolerance=1e-10, relTol=0.0)),
    "smooth_cyc_gs": ("cyc7", dict(solver="smoothSolver", smoother="GaussSeidel", nSweeps=2, tolerance=1e-7,
                                   relTol=0.0, maxIter=5000)),
    "smooth_cyc_symgs": ("cycd7", dict(solver="smoothSolver", smoother="symGaussSeidel", tolerance=1e-9,
                                       relTol=0.0)),
    "smooth_cyc_dic": ("cyc7", dict(solver="smoothSolver", smoother="DIC", tolerance=1e-7, relTol=0.0,
                                    maxIter=5000)),
    "smooth_cyc_dilugs": ("cycd7", dict(solver="smoothSolver", smoother="DILUGaussSeidel", tolerance=1e-9,
                                        relTol=0.0)),
    "pcg_gamg_direct": ("jcube14", dict(solver="PCG", tolerance=1e-9, relTol=0.0,
                                        preconditioner=dict(preconditioner="GAMG", smoother="GaussSeidel",
                                                            directSolveCoarsest=True,
                                                            interpolateCorrection=True))),
}


# fvMatrix assembly cases: psi's patch conditions on the 6 box patches
# (0 zeroGradient, 1 fixedValue, 2 fixedGradient) and the terms of each.
FVM_MESH = dict(nx=7, ny=6, nz=5, jitter=0.25, seed=3)
FVM_PATCH_BC = [1, 0, 2, 1, 0, 2]
FVM = {
    # scalarTransportFoam: ddt + div(phi,T) - laplacian(DT,T) == su
    "transport_upwind": dict(deltaT=0.01, div="upwind", lapSign=-1, gammaUniform=0.05, su=True),
    "transport_linear_face_gamma": dict(deltaT=0.02, div="linear", lapSign=-1, gamma=True),
    # pressure equation: laplacian(rAU, p) == div(phiHbyA)
    "pressure": dict(lapSign=1, gamma=True, su=True),
    "minus_laplacian": dict(lapSign=-1, gammaUniform=0.7),
    # laplacianFoam: ddt(T) - laplacian(DT,T)
    "ddt_laplacian": dict(deltaT=0.005, lapSign=-1, gammaUniform=0.3),
    "div_only": dict(div="upwind"),
    "ddt_div": dict(deltaT=0.01, div="linear"),
}
# fvMatrix::solve of some of those equations on a 14x12x10 box
FVSOLVE = dict(mesh=dict(nx=14, ny=12, nz=10, jitter=0.25, seed=5), seed=13, patchBC=FVM_PATCH_BC, cases={
    "pressure_gamg": ("pressure", dict(solver="GAMG", smoother="GaussSeidel", tolerance=1e-9, relTol=0.0)),
    "pressure_gamg_dic": ("pressure", dict(solver="GAMG", smoother="DIC", nPreSweeps=1, tolerance=1e-9,
                                           relTol=0.0)),
    "pressure_pcg_gamg": ("pressure", dict(solver="PCG", tolerance=1e-9, relTol=0.0,
                                           preconditioner=dict(preconditioner="GAMG", smoother="GaussSeidel"))),
    "ddt_laplacian_pcg": ("ddt_laplacian", dict(solver="PCG", preconditioner="DIC", tolerance=1e-10,
                                                relTol=0.0)),
    "transport_pbicgstab": ("transport_upwind", dict(solver="PBiCGStab", preconditioner="DILU",
                                                     tolerance=1e-10, relTol=0.0)),
    "transport_smooth": ("transport_upwind", dict(solver="smoothSolver", smoother="symGaussSeidel",
                                                  tolerance=1e-9, relTol=0.0)),
})


def fvm_cases():
    m = cases.box_mesh(**FVM_MESH)
    inp = gc.fvm_inputs(m)
    nI = m["nInternalFaces"]
    for name, spec in FVM.items():
        kw = gc.fvm_ref_kwargs(spec, inp, FVM_PATCH_BC)
        r = ref.fvm(m, **kw)
        out = {k: v for k, v in r.items() if not isinstance(v, str)}
        ins = {"in_" + k: np.asarray(v) for k, v in kw.items() if k not in ("div",)}
        ins["in_div"] = np.frombuffer(kw.get("div", "none").encode(), np.uint8)
        np.savez_compressed(os.path.join(HERE, f"fvm_{name}.npz"), l=m["owner"][:nI], u=m["neighbour"],
                            patchStart=m["patchStart"], **ins, **out)
        print(name, float(np.abs(out["diag"]).sum()), float(np.abs(out["source"]).sum()))


def write_fvsolve_inputs(inp):
    """The face flux the fvsolve cases are assembled from, as computed here:
    Sf.U goes through the host BLAS, whose rounding is machine-dependent, so
    the tests read these bits instead of recomputing them."""
    np.savez_compressed(os.path.join(HERE, "flux_fvsolve.npz"), phi=np.concatenate([inp["phi"], inp["phiB"]]))


def fvsolve_cases():
    """The equation assembled and solved by fvMatrix::solve on a larger
    jittered box: psi, the solver performance and GAMG's levels (faceAreaPair
    on the fvMesh's own Sf); the assembled matrix is kept as a digest."""
    m = cases.box_mesh(**FVSOLVE["mesh"])
    inp = gc.fvm_inputs(m, seed=FVSOLVE["seed"])
    write_fvsolve_inputs(inp)
    for name, (eq, ctl) in FVSOLVE["cases"].items():
        kw = gc.fvm_ref_kwargs(FVM[eq], inp, FVSOLVE["patchBC"])
        r = ref.fvm(m, solve=ctl, **kw)
        out = {k: v for k, v in r.items() if not isinstance(v, str)}
        for k in ("diag", "upper", "lower", "source", "magSf", "deltaCoeffs", "weights", "V", "bCell", "magSfB",
                  "deltaCoeffsB"):
            out.pop(k, None)
        out["matrixDigest"] = np.frombuffer(gc.matrix_digest(r["diag"], r["upper"], r.get("lower"),
                                                             r["source"]).encode(), np.uint8)
        out["solverName"] = np.frombuffer(r["solverName"].encode(), np.uint8)
        np.savez_compressed(os.path.join(HERE, f"fvsolve_{name}.npz"), **out)
        print(name, r["solverName"], int(r["nIterations"][0]), float(r["finalResidual"][0]))


# fvMatrix::solve with a cyclic pair (x periodic, patches 0 and 1) on a box
# whose xmin and xmax points match: the lduMatrix, the interfaces and the
# reference's solve (psi, performance, GAMG levels)
FVCYC = dict(mesh=dict(nx=10, ny=9, nz=8, jitter=0.25, seed=4, periodic_x=True), seed=21,
             patchBC=[3, 3, 1, 0, 2, 0], cases={
    "laplacian_pcg": (dict(lapSign=-1, gammaUniform=0.6, su=True),
                      dict(solver="PCG", preconditioner="DIC", tolerance=1e-10, relTol=0.0)),
    "laplacian_gamg": (dict(lapSign=-1, gammaUniform=0.6, su=True),
                       dict(solver="GAMG", smoother="GaussSeidel", tolerance=1e-9, relTol=0.0)),
    "laplacian_gamg_dic": (dict(lapSign=-1, gammaUniform=0.6, su=True),
                           dict(solver="GAMG", smoother="DIC", nPreSweeps=1, tolerance=1e-9, relTol=0.0)),
    "laplacian_pcg_gamg": (dict(lapSign=-1, gammaUniform=0.6, su=True),
                           dict(solver="PCG", tolerance=1e-9, relTol=0.0,
                                preconditioner=dict(preconditioner="GAMG", smoother="GaussSeidel"))),
    "transport_gamg": (dict(deltaT=0.004, div="upwind", lapSign=-1, gamma=True, su=True),
                       dict(solver="GAMG", smoother="GaussSeidel", tolerance=1e-10, relTol=0.0)),
    "transport_pbicgstab": (dict(deltaT=0.004, div="upwind", lapSign=-1, gamma=True, su=True),
                            dict(solver="PBiCGStab", preconditioner="DILU", tolerance=1e-10, relTol=0.0)),
    "transport_pbicg": (dict(deltaT=0.004, div="upwind", lapSign=-1, gamma=True, su=True),
                        dict(solver="PBiCG", preconditioner="DILU", tolerance=1e-10, relTol=0.0)),
    "transport_smooth": (dict(deltaT=0.004, div="upwind", lapSign=-1, gamma=True, su=True),
                         dict(solver="smoothSolver", smoother="symGaussSeidel", tolerance=1e-9, relTol=0.0)),
    # the direct coarsest-level solve with the cyclic interfaces in its dense matrix
    "laplacian_gamg_direct": (dict(lapSign=-1, gammaUniform=0.6, su=True),
                              dict(solver="GAMG", smoother="GaussSeidel", directSolveCoarsest=True,
                                   tolerance=1e-9, relTol=0.0)),
    "transport_gamg_direct": (dict(deltaT=0.004, div="upwind", lapSign=-1, gamma=True, su=True),
                              dict(solver="GAMG", smoother="GaussSeidel", directSolveCoarsest=True,
                                   tolerance=1e-10, relTol=0.0)),
})


def fvcyc_cases(only=None):
    m = cases.box_mesh(**FVCYC["mesh"])
    inp = gc.fvcyc_inputs(m, FVCYC["seed"])
    nI = m["nInternalFaces"]
    for name, (eq, ctl) in FVCYC["cases"].items():
        if only and name not in only:
            continue
        kw = gc.fvm_ref_kwargs(eq, inp, FVCYC["patchBC"])
        r = ref.fvm(m, solve=ctl, **kw)
        # the geometry stays: the device assembly of the cyclic patches is
        # checked against the same arrays (patchStart: the patches' first
        # faces); so do the fluxes the harness was given (Sf.U is a BLAS
        # product whose rounding differs between machines)
        out = {k: v for k, v in r.items() if not isinstance(v, str)}
        out["solverName"] = np.frombuffer(r["solverName"].encode(), np.uint8)
        np.savez_compressed(os.path.join(HERE, f"fvcyc_{name}.npz"), l=m["owner"][:nI], u=m["neighbour"],
                            patchStart=m["patchStart"], in_phi=inp["phi"], in_phiB=inp["phiB"], **out)
        print(name, r["solverName"], int(r["nIterations"][0]), float(r["finalResidual"][0]))


def build(kind, params):
    return getattr(cases, kind)(**params)


def checksum(s):
    h = hashlib.sha256()
    for k in ("l", "u", "diag", "upper", "lower", "source"):
        if s.get(k) is not None:
            h.update(np.ascontiguousarray(s[k]).tobytes())
    return h.hexdigest()


def main():
    if not ref.available():
        print("reference harness not built (python oracle/build_ref.py) or sources absent")
        return 1
    specs = {"systems": SYSTEMS, "solves": SOLVES}
    if ref.fv_available():
        specs["fvm"] = dict(mesh=FVM_MESH, patchBC=FVM_PATCH_BC, cases=FVM)
        specs["fvsolve"] = FVSOLVE
        specs["fvcyc"] = FVCYC
    with open(os.path.join(HERE, "specs.json"), "w") as fh:
        json.dump(specs, fh, indent=1, sort_keys=True)
    if len(sys.argv) > 2 and sys.argv[1] == "--fvcyc":
        # only the named cyclic fvMatrix::solve fixtures (the others kept)
        if not ref.fv_available():
            print("fv_harness not built (python oracle/build_ref_fv.py)")
            return 1
        fvcyc_cases(only=set(sys.argv[2:]))
        return 0

    # geometry of a jittered box
    m = cases.box_mesh(5, 6, 7, jitter=0.3, seed=11)
    g = ref.geometry(m)
    np.savez_compressed(os.path.join(HERE, "geom_box567.npz"), nx=5, ny=6, nz=7, jitter=0.3, seed=11,
                        **{k: g[k] for k in ("Sf", "Cf", "magSf", "C", "V")})

    sums = {}
    for name in ("cube6", "jcube7", "cd6", "box", "cyc7", "cycd7"):
        s = build(*SYSTEMS[name])
        sums[name] = checksum(s)
        x = cases.uniform(99, s["diag"].size)
        r = ref.ops(s, x, s["source"])
        r = {k: v for k, v in r.items() if not isinstance(v, str)}
        np.savez_compressed(os.path.join(HERE, f"ops_{name}.npz"), x=x, **r)

    for name, (sysname, ctl) in SOLVES.items():
        s = build(*SYSTEMS[sysname])
        sums[sysname] = checksum(s)
        pre = ctl.get("preconditioner")
        gamg_pre = isinstance(pre, dict) and pre.get("preconditioner") == "GAMG"
        w = orc.face_area_pair_weights(s["Sf"]) if ctl["solver"] == "GAMG" or gamg_pre else None
        r = ref.solve(s, ctl, weights=w)
        out = {k: v for k, v in r.items() if not isinstance(v, str)}
        out["solverName"] = np.frombuffer(r["solverName"].encode(), np.uint8)
        np.savez_compressed(os.path.join(HERE, f"solve_{name}.npz"), **out)
        print(name, r["solverName"], int(r["nIterations"][0]), float(r["finalResidual"][0]))

    if ref.fv_available():
        fvm_cases()
        fvsolve_cases()
        fvcyc_cases()
    elif len(sys.argv) > 1 and sys.argv[1] == "--fvsolve-inputs":
        m = cases.box_mesh(**FVSOLVE["mesh"])
        write_fvsolve_inputs(gc.fvm_inputs(m, seed=FVSOLVE["seed"]))
    else:
        print("fv_harness not built (python oracle/build_ref_fv.py): fvm_*.npz kept")

    with open(os.path.join(HERE, "checksums.json"), "w") as fh:
        json.dump(sums, fh, indent=1, sort_keys=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
