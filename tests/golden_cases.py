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
