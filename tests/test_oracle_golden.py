"""The oracle (C restatement of FreeFEM's path) against FreeFEM's own outputs.

Golden fixtures were produced by the FreeFEM 4.15 interpreter (tests/golden/make_golden.py).
Scalar problems reproduce FreeFEM bit for bit; elasticity within 1e-13 per entry."""
import numpy as np
import pytest

import ffo
from ffgpu import mesh
from ffgpu.fespace import FESpace
from golden_cases import MATRIX_CASES, case, load, value_errors


def oracle_system(c):
    Th = c["Th"]
    Vh = FESpace(Th, c["kind"], c.get("dof"))
    A = ffo.assemble(Th, Vh, form=c["form"], kappa=c["kappa"], quad=c["quad"], mass=c.get("mass", 0.0))
    b = ffo.rhs(Th, Vh, f=c["f"], quad=c["quad"])
    on = Vh.on(c["labels"], c["components"])
    ffo.setbc(A, b, on)
    return Vh, A, b, on


@pytest.mark.parametrize("name", MATRIX_CASES)
def test_mesh_and_numbering(name):
    c = case(name)
    d = c["d"]
    Th = c["Th"]
    assert np.array_equal(Th.coords, d["coords"])
    assert np.array_equal(Th.elems, d["elems"])
    assert np.array_equal(Th.belems, d["belems"])
    assert np.array_equal(Th.blabel, d["blabel"])
    Vh = FESpace(Th, c["kind"], c.get("dof"))
    assert np.array_equal(Vh.dof, d["dof"])


@pytest.mark.parametrize("name", MATRIX_CASES)
def test_oracle_matrix_rhs_solution(name):
    c = case(name)
    d, sc = c["d"], c["sc"]
    Vh, A, b, on = oracle_system(c)
    rp, cl, v = A.csr()
    I = np.repeat(np.arange(Vh.ndof), np.diff(rp))
    # pattern: bit-exact
    assert np.array_equal(I, d["I"]) and np.array_equal(cl, d["J"])
    # values: 1e-12 relative per entry (floor 1e-3 x row scale)
    assert value_errors(v, d["C"], rp).max() <= 1e-12
    assert np.abs(b - d["b"]).max() <= 1e-12 * np.abs(d["b"]).max()
    if c["solver"] == "CG":
        x, it, r, _ = ffo.cg(A, b, eps=c["eps"])
    else:
        x, it, r, _ = ffo.fgmres(A, b, eps=c["eps"])
    assert r >= 1
    assert np.linalg.norm(x - d["u"]) <= 1e-9 * np.linalg.norm(d["u"])
    assert it == int(sc["nit"])


def test_oracle_scalar_cases_bit_exact():
    for name in ["p1sq_n16", "p1sqk_n8_jit", "p1cubek_n4", "p2cube_n2", "p2cubem_n2", "p2sqm_n4"]:
        c = case(name)
        d = c["d"]
        Vh, A, b, on = oracle_system(c)
        rp, cl, v = A.csr()
        assert np.array_equal(v, d["C"]), name
        assert np.array_equal(b, d["b"]), name
        x, it, r, _ = ffo.cg(A, b, eps=1e-10)
        assert np.array_equal(x, d["u"]), name


def test_first_encounter_numbering_matches_oracle():
    Th = mesh.cube(3, 2, 2)
    Vh = FESpace(Th, "P2")
    tab, cnt = ffo.number_nodes(Th)
    assert cnt == Vh.ndof
    assert np.array_equal(tab, Vh.nodes)


def test_known_answer_laplace_umax():
    """square(256)-shaped probe answers recorded from FreeFEM: umax and ||u|| at n=16 (fixture)."""
    d, sc = load("p1sq_n16")
    c = case("p1sq_n16")
    Vh, A, b, on = oracle_system(c)
    x, it, r, _ = ffo.cg(A, b, eps=1e-10)
    assert abs(x.max() - sc["umax"]) <= 1e-12 * sc["umax"]
    assert abs(np.linalg.norm(x) - sc["l2"]) <= 1e-12 * sc["l2"]


@pytest.mark.skipif(ffo.reflib() is None, reason="oracle/_ref (FreeFEM's own HashMatrix/CG) not built here")
@pytest.mark.parametrize("name", ["p1sq_n16", "p1sqk_n8_jit", "p1cubek_n4", "p2el_n2", "p1sq_n12_gmres"])
def test_oracle_against_freefem_hashmatrix_and_cg(name):
    """Feed the oracle's element contributions to FreeFEM's own HashMatrix and CG/fgmres."""
    c = case(name)
    Th = c["Th"]
    Vh = FESpace(Th, c["kind"], c.get("dof"))
    I, J, V = ffo.element_contributions(Th, Vh, form=c["form"], kappa=c["kappa"], quad=c["quad"])
    R = ffo.RefHashMatrix(Vh.ndof, I, J, V)
    A = ffo.assemble(Th, Vh, form=c["form"], kappa=c["kappa"], quad=c["quad"], mass=c.get("mass", 0.0))
    b = ffo.rhs(Th, Vh, f=c["f"], quad=c["quad"])
    on = Vh.on(c["labels"], c["components"])
    R.setbc(on)
    ffo.setbc(A, b, on)
    # same insertion order, same values
    Ir, Jr, Vr = R.coo()
    Io, Jo, Vo = A.coo()
    assert np.array_equal(Ir, Io) and np.array_equal(Jr, Jo) and np.array_equal(Vr, Vo)
    if c["solver"] == "CG":
        xr, itr, rr = R.cg(b)
        xo, ito, ro, _ = ffo.cg(A, b)
    else:
        xr, itr, rr = R.fgmres(b)
        xo, ito, ro, _ = ffo.fgmres(A, b)
    assert itr == ito and rr >= 1 and ro >= 1
    assert np.array_equal(xr, xo)
    # transpose solve too
    if c["solver"] == "CG":
        xr, itr, _ = R.cg(b, trans=True)
        xo, ito, _, _ = ffo.cg(A, b, trans=True)
        assert itr == ito and np.array_equal(xr, xo)
    # sorted CSR last: FreeFEM's CSR() converts the matrix out of its COO (hash) state
    rpr, clr, vr = R.csr()
    rpo, clo, vo = A.csr()
    assert np.array_equal(rpr, rpo) and np.array_equal(clr, clo) and np.array_equal(vr, vo)


def test_adjoint_fixture_consistency():
    """FreeFEM's FP64 adjoint fixture: forward/adjoint oracle solves reproduce it."""
    d, sc = load("adj_p1_n8")
    Th = mesh.square(8)
    Vh = FESpace(Th, "P1")
    A = ffo.assemble(Th, Vh, kappa=d["in_kappa"])
    b = ffo.rhs(Th, Vh, f=d["in_f"])
    on = Vh.on((1, 2, 3, 4))
    ffo.setbc(A, b, on)
    rp, cl, v = A.csr()
    assert value_errors(v, d["C"], rp).max() <= 1e-12
    assert np.abs(b - d["b"]).max() <= 1e-12 * np.abs(d["b"]).max()
    u, it, r, _ = ffo.cg(A, b, eps=1e-14)
    assert np.linalg.norm(u - d["u"]) <= 1e-10 * np.linalg.norm(d["u"])
    M = ffo.assemble(Th, Vh, mass=1.0, c_stiff=0.0)
    rr = u - d["in_uobs"]
    Mr = M.matmul(rr)
    L = 0.5 * rr @ Mr
    assert abs(L - sc["loss"]) <= 1e-10 * abs(sc["loss"])
    lam, it, r, _ = ffo.cg(A, Mr, eps=1e-14, trans=True)
    assert np.linalg.norm(lam - d["g_lam"]) <= 1e-8 * np.linalg.norm(d["g_lam"])


@pytest.mark.parametrize("tag,tgv,solver", [("m1", -1.0, "GMRES"), ("m2", -2.0, "CG"), ("m3", -3.0, "GMRES"),
                                            ("p", 1e30, "CG")])
def test_oracle_tgv_variants(tag, tgv, solver):
    """on(1,2,3,4, u=x) with tgv = -1, -2, -3 and 1e30 against FreeFEM."""
    d, sc = load("p1sq_n6_tgv" + tag)
    Th = mesh.square(6)
    Vh = FESpace(Th, "P1")
    A = ffo.assemble(Th, Vh, quad="qf2pT")
    b = ffo.rhs(Th, Vh, f=1.0, quad="qf2pT")
    on = Vh.on((1, 2, 3, 4))
    ffo.setbc(A, b, on, g=Th.coords[:, 0].copy(), tgv=tgv)
    rp, cl, v = A.csr()
    assert np.array_equal(np.repeat(np.arange(Vh.ndof), np.diff(rp)), d["I"]) and np.array_equal(cl, d["J"])
    assert value_errors(v, d["C"], rp).max() <= 1e-12
    assert np.abs(b - d["b"]).max() <= 1e-12 * np.abs(d["b"]).max()
    if solver == "CG":
        x, it, r, _ = ffo.cg(A, b, eps=1e-12, tgv=tgv)
    else:
        x, it, r, _ = ffo.fgmres(A, b, eps=1e-12, tgv=tgv)
    assert np.linalg.norm(x - d["u"]) <= 1e-9 * np.linalg.norm(d["u"])
    assert it == int(sc["nit"])
