"""Device-side finite-volume assembly (cfx_fvm_assemble) against the oracle.

The device writes the lduMatrix and source that fvMatrix::solveSegregated
hands to the solver for fvm::ddt + fvm::div +/- fvm::laplacian == su; every
coefficient must equal the oracle's restatement bit for bit (the same
products and sums in the reference's order), for the term combinations a
PISO/PIMPLE step assembles, on a jittered mesh with fixedValue,
zeroGradient and fixedGradient patches.  Re-assembly with new fluxes
replaces the resident coefficients (no stale packs), and an assembled
system solves to the same answer as the same system uploaded from the host.
"""
import numpy as np
import pytest

from oracle import oracle as orc
from openfoam_dev_gb300 import cases, ldu

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _setup(seed=3, shape=(9, 8, 7)):
    m = cases.box_mesh(*shape, jitter=0.25, seed=seed)
    g = cases.fv_geometry(m)
    nI, nB, nC = m["nInternalFaces"], g["bCell"].size, m["nCells"]
    rng = np.random.default_rng(seed)
    ps = m["patchStart"]
    bcType = np.zeros(nB, np.int32)
    for p, t in enumerate((1, 0, 2, 1, 0, 2)):  # xmin fixedValue, xmax zeroGradient, ymin fixedGradient, ...
        bcType[ps[p] - nI:ps[p + 1] - nI] = t
    f = dict(psi0=rng.uniform(-1, 1, nC), phi=rng.uniform(-1, 1, nI), phiB=rng.uniform(-1, 1, nB),
             gamma=rng.uniform(0.01, 0.1, nI), gammaB=rng.uniform(0.01, 0.1, nB), bcType=bcType,
             bcValue=rng.uniform(-1, 1, nB), su=rng.uniform(-1, 1, nC))
    mesh = ldu.LduMesh(ldu.default_context(), nC, m["owner"][:nI], m["neighbour"])
    mesh.fv_geometry(g["magSf"], g["deltaCoeffs"], g["V"], g["bCell"], g["magSfB"], g["deltaCoeffsB"],
                     weights=g["weights"])
    return m, g, f, mesh


def _dev(a, dtype=torch.float64):
    return None if a is None else torch.as_tensor(np.ascontiguousarray(a), device="cuda").to(dtype)


CASES = {
    # scalarTransportFoam: ddt(T) + div(phi,T) - laplacian(DT,T) == su
    "transport_upwind": dict(rDeltaT=50.0, psi0=True, phi=True, div="upwind", lapSign=-1, gamma=0.05, su=True),
    "transport_linear_face_gamma": dict(rDeltaT=20.0, psi0=True, phi=True, div="linear", lapSign=-1,
                                        gamma="face"),
    # the pressure equation: laplacian(rAU, p) == div(phiHbyA)
    "pressure": dict(lapSign=1, gamma="face", su=True),
    "minus_laplacian": dict(lapSign=-1, gamma=0.3),
    "ddt_laplacian": dict(rDeltaT=10.0, psi0=True, lapSign=-1, gamma=0.02, su=True),
    "div_only": dict(phi=True, div="upwind"),
    "ddt_div": dict(rDeltaT=5.0, psi0=True, phi=True, div="linear"),
}


def _terms(case, f, dev):
    kw = dict(rDeltaT=case.get("rDeltaT", 0.0), div=case.get("div", "upwind"), lapSign=case.get("lapSign", 0),
              bcType=f["bcType"], bcValue=f["bcValue"])
    if case.get("psi0"):
        kw["psi0"] = f["psi0"]
    if case.get("phi"):
        kw["phi"], kw["phiB"] = f["phi"], f["phiB"]
    if case.get("su"):
        kw["su"] = f["su"]
    gam = case.get("gamma", 1.0)
    if gam == "face":
        kw["gamma"], kw["gammaB"] = f["gamma"], f["gammaB"]
    else:
        kw["gamma"] = gam
    if dev:
        kw = {k: (_dev(v, torch.int32 if k == "bcType" else torch.float64) if isinstance(v, np.ndarray) else v)
              for k, v in kw.items()}
    return kw


@pytest.mark.parametrize("name", sorted(CASES))
def test_assembly_bit_exact_against_the_oracle(name):
    m, g, f, mesh = _setup()
    case = CASES[name]
    nI = m["nInternalFaces"]
    d, up, lo, src = orc.fvm_assemble(m["owner"][:nI], m["neighbour"], g, **_terms(case, f, dev=False))
    A = ldu.LduMatrix.empty(mesh, symmetric=lo is None)
    source = torch.empty(m["nCells"], dtype=torch.float64, device="cuda")
    A.assemble(source, **_terms(case, f, dev=True))
    torch.cuda.synchronize()
    got_d, got_u, got_l = A.coarse(0, m["nCells"], nI)
    np.testing.assert_array_equal(got_d, d)
    np.testing.assert_array_equal(got_u, up)
    if lo is not None:
        np.testing.assert_array_equal(got_l, lo)
    np.testing.assert_array_equal(source.cpu().numpy(), src)


def test_reassembly_replaces_coefficients_and_solves_like_an_upload():
    m, g, f, mesh = _setup(seed=5)
    nI, n = m["nInternalFaces"], m["nCells"]
    case = CASES["transport_upwind"]
    A = ldu.LduMatrix.empty(mesh, symmetric=False)
    source = torch.empty(n, dtype=torch.float64, device="cuda")
    ctl = {"solver": "cudaPBiCGStab", "preconditioner": "DILU", "tolerance": 1e-10, "relTol": 0}
    A.assemble(source, **_terms(case, f, dev=True))
    psi = torch.zeros(n, dtype=torch.float64, device="cuda")
    ldu.solver_new("T", A, ctl).solve(psi, source)  # packs built for the first coefficients
    f2 = dict(f, phi=-f["phi"] * 0.5, phiB=-f["phiB"] * 0.5)  # the next corrector's fluxes
    A.assemble(source, **_terms(case, f2, dev=True))
    psi = torch.zeros(n, dtype=torch.float64, device="cuda")
    p1 = ldu.solver_new("T", A, ctl).solve(psi, source)
    d, up, lo, src = orc.fvm_assemble(m["owner"][:nI], m["neighbour"], g, **_terms(case, f2, dev=False))
    B = ldu.LduMatrix(mesh, d, up, lo)
    x = np.zeros(n)
    p2 = ldu.solver_new("T", B, ctl).solve(x, src)
    assert p1.converged and p1.nIterations == p2.nIterations
    np.testing.assert_array_equal(psi.cpu().numpy(), x)


def test_assembly_errors():
    m, g, f, mesh = _setup(seed=7, shape=(4, 3, 3))
    n = m["nCells"]
    source = torch.empty(n, dtype=torch.float64, device="cuda")
    S = ldu.LduMatrix.empty(mesh, symmetric=True)
    with pytest.raises(ldu.CfxError):  # a div term needs an asymmetric matrix
        S.assemble(source, **_terms(CASES["div_only"], f, dev=True))
    with pytest.raises(ldu.CfxError):  # no term
        S.assemble(source, bcType=_dev(f["bcType"], torch.int32), bcValue=_dev(f["bcValue"]))
    other = ldu.LduMesh(ldu.default_context(), n, m["owner"][:m["nInternalFaces"]], m["neighbour"])
    with pytest.raises(ldu.CfxError):  # no geometry
        ldu.LduMatrix.empty(other, symmetric=True).assemble(source, **_terms(CASES["minus_laplacian"], f, dev=True))


def _cyclic_names():
    from golden_cases import fvcyc_names
    return fvcyc_names()


@pytest.mark.parametrize("name", _cyclic_names())
def test_cyclic_assembly_matches_the_reference(name):
    """A cyclic patch pair assembled on the device (CFX_BC_CYCLIC): the
    lduMatrix and source equal the reference's fvMatrix bit for bit, and the
    interface coefficients written by the assembly give the reference's A x
    and A^T x (interfaceBouCoeffs in Amul, interfaceIntCoeffs in Tmul)."""
    from golden_cases import fvcyc_assembly_case
    l, u, geom, terms, ref = fvcyc_assembly_case(name)
    n, nI = geom["V"].size, l.size
    mesh = ldu.LduMesh(ldu.default_context(), n, l, u)
    mesh.set_interfaces(ref["ifSize"], ref["ifCell"], ref["ifNbr"],
                        np.arange(len(ref["ifSize"]), dtype=np.int32) ^ 1)
    mesh.fv_geometry(geom["magSf"], geom["deltaCoeffs"], geom["V"], geom["bCell"], geom["magSfB"],
                     geom["deltaCoeffsB"], weights=geom["weights"])
    A = ldu.LduMatrix.empty(mesh, symmetric=ref["lower"] is None)
    source = torch.empty(n, dtype=torch.float64, device="cuda")
    dev = {k: (_dev(v, torch.int32 if k == "bcType" else torch.float64) if isinstance(v, np.ndarray) else v)
           for k, v in terms.items()}
    A.assemble(source, **dev)
    torch.cuda.synchronize()
    got_d, got_u, got_l = A.coarse(0, n, nI)
    np.testing.assert_array_equal(got_d, ref["diag"])
    np.testing.assert_array_equal(got_u, ref["upper"])
    if ref["lower"] is not None:
        np.testing.assert_array_equal(got_l, ref["lower"])
    np.testing.assert_array_equal(source.cpu().numpy(), ref["source"])
    s = dict(l=l, u=u, diag=ref["diag"], upper=ref["upper"], lower=ref["lower"], ifSize=ref["ifSize"],
             ifCell=ref["ifCell"], ifNbr=ref["ifNbr"], ifBou=ref["ifBou"], ifInt=ref["ifInt"])
    om = orc.Matrix(s)
    x = cases.uniform(5, n)
    dx, dy = _dev(x), torch.empty(n, dtype=torch.float64, device="cuda")
    A.Amul(dx, dy)
    np.testing.assert_array_equal(dy.cpu().numpy(), om.amul(x))
    A.Tmul(dx, dy)
    np.testing.assert_array_equal(dy.cpu().numpy(), om.tmul(x))


def test_cyclic_faces_must_be_the_interfaces():
    from golden_cases import fvcyc_assembly_case
    l, u, geom, terms, ref = fvcyc_assembly_case("laplacian_pcg")
    n = geom["V"].size
    mesh = ldu.LduMesh(ldu.default_context(), n, l, u)
    # one patch's faces only: the assembly finds twice as many cyclic faces
    k = int(ref["ifSize"][0])
    mesh.set_interfaces(ref["ifSize"][:1], ref["ifCell"][:k], ref["ifNbr"][:k])
    mesh.fv_geometry(geom["magSf"], geom["deltaCoeffs"], geom["V"], geom["bCell"], geom["magSfB"],
                     geom["deltaCoeffsB"], weights=geom["weights"])
    A = ldu.LduMatrix.empty(mesh, symmetric=True)
    source = torch.empty(n, dtype=torch.float64, device="cuda")
    dev = {k2: (_dev(v, torch.int32 if k2 == "bcType" else torch.float64) if isinstance(v, np.ndarray) else v)
           for k2, v in terms.items()}
    with pytest.raises(ldu.CfxError, match="cyclic"):
        A.assemble(source, **dev)
