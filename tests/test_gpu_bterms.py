"""Boundary terms on the device (Robin c*u*v into the matrix, Neumann g*v into the linear
form, on labelled boundary edges and faces) against FreeFEM's outputs and the oracle, through
the C ABI.  Same bars as the volume path: pattern bit-exact, values within 1e-12 relative per
entry, right-hand side within 1e-12 of its largest entry, solution within 1e-9 relative."""
import numpy as np
import pytest

import ffgpu
import ffo
from ffgpu.fespace import FESpace
from golden_cases import BT_CASES, bt_case, value_errors

pytestmark = pytest.mark.gpu

VAL_TOL = 1e-12
SOL_TOL = 1e-9


@pytest.fixture(scope="module", autouse=True)
def _lib_built():
    from ffgpu.build import build
    build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    ffgpu.context(0)
    yield


def device_varf(c, tgv=1e30):
    spec = c["spec"]
    adj_elem, _ = ffo.boundary_adjacency(c["Th"])
    terms = [ffgpu.BoundaryTerm(labels=lab, robin=r) for lab, r in spec["robin"]]
    for lab, g in spec["neumann"]:
        terms.append(ffgpu.BoundaryTerm(labels=lab, g=c["gk_elem"][adj_elem] if isinstance(g, str) else g))
    if c["kind"] == "P2vec":
        return ffgpu.varf_elasticity(E=1.0, nu=0.3, f=(0.0, 0.0, -1.0), on=spec["on"], tgv=tgv, bterms=terms)
    return ffgpu.varf_diffusion(f=1.0, on=spec["on"], tgv=tgv, bterms=terms)


@pytest.mark.parametrize("name", list(BT_CASES))
def test_boundary_terms_against_freefem(name):
    c = bt_case(name)
    d, sc = c["d"], c["sc"]
    Vh = FESpace(c["Th"], c["kind"], c["dof"])
    a = device_varf(c)
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(a, Vh, eps=1e-10, rhs_out=b)
    rp, cl, v = A.csr()
    I = np.repeat(np.arange(Vh.ndof), np.diff(rp))
    assert np.array_equal(I, d["I"]) and np.array_equal(cl, d["J"]), "pattern differs"
    assert value_errors(v, d["C"], rp).max() <= VAL_TOL
    assert np.abs(b - d["b"]).max() <= VAL_TOL * np.abs(d["b"]).max()
    u = A.solve(b)
    assert np.linalg.norm(u - d["u"]) <= SOL_TOL * np.linalg.norm(d["u"])
    assert abs(A.stats.iterations - int(sc["nit"])) <= 2
    # a(0,Vh) alone equals the linear form assembled with the matrix, bit for bit
    assert np.array_equal(ffgpu.rhs(a, A.space), b)


@pytest.mark.parametrize("tgv", [-1.0, -2.0, -3.0])
def test_boundary_terms_with_tgv_variants_against_oracle(tgv):
    """Robin rows on Dirichlet boundaries: the tgv < 0 variants zero rows/columns after the
    boundary terms, as HashMatrix::SetBC does after AssembleBilinearForm."""
    c = bt_case("bt_p1sq_6x5")
    Th, spec = c["Th"], c["spec"]
    Vh = FESpace(Th, "P1")
    adj = ffo.boundary_adjacency(Th)
    Ao = ffo.assemble(Th, Vh)
    for lab, r in spec["robin"]:
        ffo.bterm(Th, Vh, lab, robin=r, A=Ao, adj=adj)
    bo = ffo.rhs(Th, Vh, f=1.0)
    for lab, g in spec["neumann"]:
        ffo.bterm(Th, Vh, lab, g=c["gk_elem"][adj[0]] if isinstance(g, str) else g, b=bo, adj=adj)
    ffo.setbc(Ao, bo, Vh.on(spec["on"]), tgv=tgv)
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(device_varf(c, tgv=tgv), Vh, eps=1e-10, rhs_out=b, solver="GMRES")
    rpo, clo, vo = Ao.csr()
    rp, cl, v = A.csr()
    assert np.array_equal(rp, rpo) and np.array_equal(cl, clo)
    assert value_errors(v, vo, rpo).max() <= VAL_TOL
    assert np.abs(b - bo).max() <= VAL_TOL * np.abs(bo).max()


def test_boundary_terms_whole_boundary_and_per_element_robin():
    """labels = () takes every boundary element; a Robin coefficient per boundary element."""
    from ffgpu import mesh
    Th = mesh.cube(3, 2, 2)
    Vh = FESpace(Th, "P2")
    rng = np.random.default_rng(3)
    rob = rng.uniform(0.5, 1.5, Th.nbe)
    adj = ffo.boundary_adjacency(Th)
    Ao = ffo.assemble(Th, Vh)
    ffo.bterm(Th, Vh, (), robin=rob, A=Ao, adj=adj)
    bo = ffo.rhs(Th, Vh, f=0.0)
    ffo.bterm(Th, Vh, (), g=2.0, b=bo, adj=adj)
    a = ffgpu.varf_diffusion(f=0.0, bterms=[ffgpu.BoundaryTerm(robin=rob, g=2.0)])
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(a, Vh, eps=1e-10, rhs_out=b)
    rpo, clo, vo = Ao.csr()
    rp, cl, v = A.csr()
    assert np.array_equal(cl, clo)
    assert value_errors(v, vo, rpo).max() <= VAL_TOL
    assert np.abs(b - bo).max() <= VAL_TOL * np.abs(bo).max()
    # pure Robin problem (no Dirichlet rows): SPD, solvable by CG
    u = A.solve(b)
    uo, it, r, _ = ffo.cg(Ao, bo, eps=1e-10)
    assert np.linalg.norm(u - uo) <= SOL_TOL * np.linalg.norm(uo)
