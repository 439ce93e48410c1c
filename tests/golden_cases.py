"""Access to the golden fixtures written by tests/golden/make_golden.py."""
import hashlib
import json
import os

import numpy as np

from openfoam_dev_gb300 import cases

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

with open(os.path.join(GOLDEN, "specs.json")) as fh:
    SPECS = json.load(fh)
with open(os.path.join(GOLDEN, "checksums.json")) as fh:
    CHECKSUMS = json.load(fh)


def checksum(s):
    h = hashlib.sha256()
    for k in ("l", "u", "diag", "upper", "lower", "source"):
        if s.get(k) is not None:
            h.update(np.ascontiguousarray(s[k]).tobytes())
    return h.hexdigest()


def system(name):
    kind, params = SPECS["systems"][name]
    return getattr(cases, kind)(**params)


def load(fname):
    with np.load(os.path.join(GOLDEN, fname)) as z:
        return {k: z[k] for k in z.files}


def solve_case(name):
    sysname, ctl = SPECS["solves"][name]
    g = load(f"solve_{name}.npz")
    g["solverName"] = bytes(g["solverName"]).decode()
    return system(sysname), dict(ctl), g


def gamg_kwargs(ctl):
    keys = ("smoother", "nPreSweeps", "nPostSweeps", "nFinestSweeps", "maxPreSweeps", "maxPostSweeps",
            "nCellsInCoarsestLevel", "interpolateCorrection", "directSolveCoarsest")
    return {k: ctl[k] for k in keys if k in ctl}


FVM_GEOMETRY_KEYS = ("magSf", "deltaCoeffs", "weights", "V", "bCell", "magSfB", "deltaCoeffsB")


def fvm_names():
    return sorted(f[4:-4] for f in os.listdir(GOLDEN) if f.startswith("fvm_") and f.endswith(".npz"))


def fvm_case(name):
    """One fvMatrix assembly fixture: (l, u, the reference's geometry, the
    assembly terms in the oracle's/device's argument form, the reference's
    diag/upper/lower/source).  rDeltaT = 1/deltaT as EulerDdtScheme forms
    it; the per-patch condition is expanded to one per boundary face."""
    g = load(f"fvm_{name}.npz")
    geom = {k: g[k] for k in FVM_GEOMETRY_KEYS}
    bcType = np.repeat(g["in_patchBC"], np.diff(g["patchStart"])).astype(np.int32)
    assert bcType.size == g["in_bcValue"].size
    div = bytes(g["in_div"]).decode()
    terms = dict(rDeltaT=1.0 / float(g["in_deltaT"]) if "in_deltaT" in g else 0.0,
                 div="upwind" if div == "none" else div,
                 lapSign=int(g["in_lapSign"]), bcType=bcType, bcValue=g["in_bcValue"])
    for k in ("psi0", "phi", "phiB", "su", "gammaB"):
        if "in_" + k in g:
            terms[k] = g["in_" + k]
    if "in_gamma" in g:
        terms["gamma"] = g["in_gamma"]
    elif "in_gammaUniform" in g:
        terms["gamma"] = float(g["in_gammaUniform"])
    ref = dict(diag=g["diag"], upper=g["upper"], lower=g.get("lower"), source=g["source"])
    return g["l"], g["u"], geom, terms, ref
