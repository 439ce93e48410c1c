"""Run the reference's own solver code (oracle/_ref/ref_harness) on a system.

TEST INFRASTRUCTURE ONLY, and only where the reference sources are mounted
(the harness links oracle/_ref/libOpenFOAM.so built by build_ref.py).  Used
to pin the C oracle and to write the golden fixtures in tests/golden/.
"""
import os
import subprocess
import tempfile

import numpy as np

from . import records
from .refpath import REF_ROOT

HERE = os.path.dirname(os.path.abspath(__file__))
HARNESS = os.path.join(HERE, "_ref", "ref_harness")


def available():
    return os.path.exists(HARNESS) and os.path.isdir(os.path.join(REF_ROOT, "etc"))


def run(recs):
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.rec"), os.path.join(td, "out.rec")
        records.write(fin, recs)
        env = dict(os.environ, WM_PROJECT_DIR=REF_ROOT, WM_PROJECT="OpenFOAM",
                   WM_PROJECT_VERSION="dev", CFX_HARNESS_ROOT=td)
        os.makedirs(os.path.join(td, "cfxcase"), exist_ok=True)
        r = subprocess.run([HARNESS, fin, fout], env=env, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference harness failed:\n" + r.stdout[-3000:] + r.stderr[-3000:])
        return records.read(fout)


def _ldu(s):
    d = dict(l=s["l"], u=s["u"], diag=s["diag"], upper=s["upper"])
    if s.get("lower") is not None:
        d["lower"] = s["lower"]
    if s.get("ifCell") is not None:  # coupled (cyclic) interfaces
        for k in ("ifSize", "ifCell", "ifNbr", "ifBou", "ifInt"):
            d[k] = s[k]
    return d


def geometry(mesh):
    return run(dict(mode="geom", points=mesh["points"], faces=mesh["faces"], owner=mesh["owner"],
                    neighbour=mesh["neighbour"], patchStart=mesh["patchStart"]))


def ops(s, x, b):
    return run(dict(mode="ops", x=x, b=b, **_ldu(s)))


def dict_text(ctl):
    parts = []
    for k, v in ctl.items():
        if isinstance(v, dict):
            parts.append(f"{k} {dict_text(v)}")
            continue
        if isinstance(v, bool):
            v = "true" if v else "false"
        elif isinstance(v, float):
            v = repr(v)
        parts.append(f"{k} {v};")
    return "{ " + " ".join(parts) + " }"


def solve(s, ctl, psi0=None, weights=None):
    recs = dict(mode="solve", source=s["source"],
                psi=np.zeros_like(s["source"]) if psi0 is None else psi0,
                dict=dict_text(ctl), **_ldu(s))
    if weights is not None:
        recs["weights"] = weights
    return run(recs)


PLUGIN = os.path.join(HERE, "_ref", "libcudaLduSolvers_OpenFOAM.so")


def plugin_available():
    return os.path.exists(PLUGIN) and available()


def plugin_solve(s, ctl, library=PLUGIN, psi0=None):
    """The reference's run-time loading path: libs.open(library), then
    lduMatrix::solver::New with the dictionary and solve; returns the
    records (loaded, type, psi and performance, or the FatalError message
    as "fatal")."""
    recs = dict(mode="plugin", source=s["source"],
                psi=np.zeros_like(s["source"]) if psi0 is None else psi0,
                dict=dict_text(ctl), library=library or "", **_ldu(s))
    return run(recs)


FV_HARNESS = os.path.join(HERE, "_ref", "fv_harness")

_FOAM_HEADER = "FoamFile\n{\n    format ascii;\n    class dictionary;\n    object %s;\n}\n"


def fv_available():
    return os.path.exists(FV_HARNESS) and available()


def _fv_case(td, div):
    """system/ of the case fv_harness runs in: Euler, Gauss <div> for
    div(phi,T), Gauss linear uncorrected for the Laplacian (the face-normal
    gradient without the non-orthogonal correction, as the device assembly
    has it)."""
    sysdir = os.path.join(td, "cfxcase", "system")
    os.makedirs(sysdir, exist_ok=True)
    files = {
        "fvSchemes": ("ddtSchemes { default Euler; }\n"
                      "gradSchemes { default Gauss linear; }\n"
                      "divSchemes { default none; div(phi,T) Gauss %s; }\n"
                      "laplacianSchemes { default Gauss linear uncorrected; }\n"
                      "interpolationSchemes { default linear; }\n"
                      "snGradSchemes { default uncorrected; }\n" % div),
        "fvSolution": "solvers { }\n",
        "controlDict": ("application none;\nstartFrom startTime;\nstartTime 0;\nstopAt endTime;\n"
                        "endTime 1;\ndeltaT 1;\nwriteControl timeStep;\nwriteInterval 1;\n"),
    }
    for name, body in files.items():
        with open(os.path.join(sysdir, name), "w") as fh:
            fh.write(_FOAM_HEADER % name + body)


def fvm(mesh, patchBC, bcValue, deltaT=None, psi0=None, phi=None, phiB=None, div="upwind", lapSign=0,
        gamma=None, gammaB=None, gammaUniform=None, su=None, solve=None):
    """The reference's fvm::ddt(T) + fvm::div(phi, T) +/- fvm::laplacian(gamma, T)
    == su on a hex mesh, each term optional (fv_harness): the diag (with
    addBoundaryDiag), upper, lower (when asymmetric) and source (with
    addBoundarySource) the solver receives, and the geometry the schemes used.
    patchBC per patch: 0 zeroGradient, 1 fixedValue, 2 fixedGradient; bcValue
    per boundary face (value or gradient).  With solve (a solver control
    dict) the harness then runs fvMatrix::solve with it from psi0 (or zero)
    and adds psi, the solver performance and GAMG's agglomeration levels."""
    recs = dict(points=mesh["points"], faces=mesh["faces"], owner=mesh["owner"], neighbour=mesh["neighbour"],
                patchStart=mesh["patchStart"], patchBC=np.asarray(patchBC, np.int32),
                bcValue=np.asarray(bcValue, np.float64))
    if deltaT is not None:
        recs["deltaT"] = np.array([deltaT], np.float64)
    opt = dict(psi0=psi0, phi=phi, phiB=phiB, gamma=gamma, gammaB=gammaB, su=su)
    recs.update({k: np.asarray(v, np.float64) for k, v in opt.items() if v is not None})
    if gammaUniform is not None:
        recs["gammaUniform"] = np.array([gammaUniform], np.float64)
    if lapSign:
        recs["lapSign"] = np.array([lapSign], np.int32)
    if solve is not None:
        recs["dict"] = dict_text(solve)
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.rec"), os.path.join(td, "out.rec")
        records.write(fin, recs)
        _fv_case(td, div)
        env = dict(os.environ, WM_PROJECT_DIR=REF_ROOT, WM_PROJECT="OpenFOAM",
                   WM_PROJECT_VERSION="dev", CFX_HARNESS_ROOT=td)
        r = subprocess.run([FV_HARNESS, fin, fout], env=env, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("fv harness failed:\n" + r.stdout[-3000:] + r.stderr[-3000:])
        return records.read(fout)
