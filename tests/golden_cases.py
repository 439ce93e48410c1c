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


def fvm_inputs(mesh, seed=11):
    """Seeded fields on the mesh: psi's boundary values/gradients, the old
    value, a flux phi = Sf.U + noise, a face diffusivity and a source."""
    rng = np.random.default_rng(seed)
    nI, nF, nC = mesh["nInternalFaces"], mesh["nFaces"], mesh["V"].size
    Sf = mesh["Sf"].reshape(nF, 3)
    phi = Sf @ np.array([0.8, -0.35, 0.2]) + 0.05 * rng.uniform(-1, 1, nF) * mesh["magSf"]
    gam = rng.uniform(0.2, 1.5, nF)
    return dict(bcValue=rng.uniform(-2, 2, nF - nI), psi0=rng.uniform(-1, 1, nC), phi=phi[:nI], phiB=phi[nI:],
                gamma=gam[:nI], gammaB=gam[nI:], su=rng.uniform(-3, 3, nC))


def fvm_ref_kwargs(spec, inp, patchBC):
    """An equation spec's arguments to the reference harness (oracle.reference.fvm)."""
    kw = dict(patchBC=patchBC, bcValue=inp["bcValue"], lapSign=spec.get("lapSign", 0))
    if "deltaT" in spec:
        kw.update(deltaT=spec["deltaT"], psi0=inp["psi0"])
    if "div" in spec:
        kw.update(phi=inp["phi"], phiB=inp["phiB"], div=spec["div"])
    if spec.get("gamma"):
        kw.update(gamma=inp["gamma"], gammaB=inp["gammaB"])
    elif "gammaUniform" in spec:
        kw.update(gammaUniform=spec["gammaUniform"])
    if spec.get("su"):
        kw.update(su=inp["su"])
    return kw


def fvm_terms(spec, inp, bcType):
    """The same equation in the oracle's / device's assembly arguments."""
    t = dict(rDeltaT=1.0 / spec["deltaT"] if "deltaT" in spec else 0.0, div=spec.get("div", "upwind"),
             lapSign=spec.get("lapSign", 0), bcType=bcType, bcValue=inp["bcValue"])
    if "deltaT" in spec:
        t["psi0"] = inp["psi0"]
    if "div" in spec:
        t.update(phi=inp["phi"], phiB=inp["phiB"])
    if spec.get("gamma"):
        t.update(gamma=inp["gamma"], gammaB=inp["gammaB"])
    elif "gammaUniform" in spec:
        t["gamma"] = spec["gammaUniform"]
    if spec.get("su"):
        t["su"] = inp["su"]
    return t


def matrix_digest(diag, upper, lower, source):
    h = hashlib.sha256()
    for a in (diag, upper, lower, source):
        if a is not None:
            h.update(np.ascontiguousarray(a, np.float64).tobytes())
    return h.hexdigest()


def fvsolve_names():
    return sorted(f[8:-4] for f in os.listdir(GOLDEN) if f.startswith("fvsolve_") and f.endswith(".npz"))


def fvsolve_case(name):
    """One fvMatrix::solve fixture: (mesh, the equation's assembly terms,
    the solver controls, the reference's results)."""
    spec = SPECS["fvsolve"]
    eq, ctl = spec["cases"][name]
    m = cases.box_mesh(**spec["mesh"])
    nI = m["nInternalFaces"]
    inp = fvm_inputs(m, seed=spec["seed"])
    # the flux as the reference received it: Sf.U goes through the host's
    # BLAS, whose rounding differs between machines (x86-64 and aarch64), so
    # the bits the fixtures were made from are stored beside them
    phi = load("flux_fvsolve.npz")["phi"]
    inp["phi"], inp["phiB"] = phi[:nI].copy(), phi[nI:].copy()
    bcType = np.repeat(np.asarray(spec["patchBC"], np.int32), np.diff(m["patchStart"])).astype(np.int32)
    g = load(f"fvsolve_{name}.npz")
    g["solverName"] = bytes(g["solverName"]).decode()
    g["matrixDigest"] = bytes(g["matrixDigest"]).decode()
    m["Sf_internal"] = m["Sf"][: 3 * nI].reshape(nI, 3).copy()
    return m, fvm_terms(SPECS["fvm"]["cases"][eq], inp, bcType), dict(ctl), g


def fvcyc_inputs(mesh, seed):
    """fvm_inputs with the cyclic pair's face values made periodic: the flux
    through an xmax face is minus that through its xmin partner, and both
    carry the same diffusivity."""
    inp = fvm_inputs(mesh, seed=seed)
    nI, ps = mesh["nInternalFaces"], mesh["patchStart"]
    a = slice(ps[0] - nI, ps[1] - nI)
    b = slice(ps[1] - nI, ps[2] - nI)
    inp["phiB"][b] = -inp["phiB"][a]
    inp["gammaB"][b] = inp["gammaB"][a]
    return inp


def fvcyc_names():
    return sorted(f[6:-4] for f in os.listdir(GOLDEN) if f.startswith("fvcyc_") and f.endswith(".npz"))


def fvcyc_assembly_case(name):
    """One cyclic fvMatrix fixture as an assembly case: (l, u, the
    reference's geometry (the cyclic faces' deltaCoeffsB the snGrad
    scheme's), the terms with the cyclic pair as bcType 3, and the
    reference's diag/upper/lower/source and interfaceBou/IntCoeffs)."""
    eq, _ = SPECS["fvcyc"]["cases"][name]
    g = load(f"fvcyc_{name}.npz")
    m = cases.box_mesh(**SPECS["fvcyc"]["mesh"])
    inp = fvcyc_inputs(m, SPECS["fvcyc"]["seed"])
    inp["phi"], inp["phiB"] = g["in_phi"], g["in_phiB"]  # the fluxes the reference was given
    bcType = np.repeat(np.asarray(SPECS["fvcyc"]["patchBC"], np.int32), np.diff(g["patchStart"])).astype(np.int32)
    geom = {k: g[k] for k in FVM_GEOMETRY_KEYS}
    ref = dict(diag=g["diag"], upper=g["upper"], lower=g.get("lower"), source=g["source"], ifBou=g["ifBou"],
               ifInt=g["ifInt"], ifSize=g["ifSize"], ifCell=g["ifCell"], ifNbr=g["ifNbr"])
    return g["l"], g["u"], geom, fvm_terms(eq, inp, bcType), ref


def fvcyc_case(name):
    """(the lduMatrix system with its cyclic interfaces as the solver
    received it, the starting psi, the solver controls, the reference's
    results)."""
    eq, ctl = SPECS["fvcyc"]["cases"][name]
    g = load(f"fvcyc_{name}.npz")
    g["solverName"] = bytes(g["solverName"]).decode()
    # the harness lists the cyclic patches in pairs (xmin, xmax): each
    # other's partner (cyclicLduInterface::nbrPatchIndex)
    nbr_patch = np.arange(len(g["ifSize"]), dtype=np.int32) ^ 1
    s = dict(l=g["l"], u=g["u"], diag=g["diag"], upper=g["upper"], lower=g.get("lower"), source=g["source"],
             ifSize=g["ifSize"], ifCell=g["ifCell"], ifNbr=g["ifNbr"], ifBou=g["ifBou"], ifInt=g["ifInt"],
             ifNbrPatch=nbr_patch)
    m = cases.box_mesh(**SPECS["fvcyc"]["mesh"])
    nI = m["nInternalFaces"]
    s["Sf"] = m["Sf"][: 3 * nI].reshape(nI, 3).copy()  # faceAreaPair weights
    psi0 = fvcyc_inputs(m, SPECS["fvcyc"]["seed"])["psi0"] if "deltaT" in eq else None
    return s, psi0, dict(ctl), g
