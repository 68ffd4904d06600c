"""Boundary terms (Robin c*u*v and Neumann g*v on labelled boundary edges/faces) of the oracle
against FreeFEM's outputs (tests/golden/bt_*.npz)."""
import numpy as np
import pytest

import ffo
from ffgpu.fespace import FESpace
from golden_cases import BT_CASES, bt_case, value_errors


def oracle_bt_system(c):
    Th, spec = c["Th"], c["spec"]
    Vh = FESpace(Th, c["kind"], c["dof"])
    el = c["kind"] == "P2vec"
    adj = ffo.boundary_adjacency(Th)
    A = ffo.assemble(Th, Vh, form="elasticity" if el else "diffusion")
    for labels, cr in spec["robin"]:
        ffo.bterm(Th, Vh, labels, robin=cr, A=A, adj=adj)
    b = ffo.rhs(Th, Vh, f=(0.0, 0.0, -1.0) if el else 1.0)
    for labels, g in spec["neumann"]:
        gv = c["gk_elem"][adj[0]] if isinstance(g, str) else g
        ffo.bterm(Th, Vh, labels, g=gv, b=b, adj=adj)
    on = Vh.on(spec["on"])
    ffo.setbc(A, b, on)
    return Vh, A, b


@pytest.mark.parametrize("name", list(BT_CASES))
def test_boundary_adjacency_matches_mesh(name):
    c = bt_case(name)
    Th, d = c["Th"], c["d"]
    assert np.array_equal(Th.belems, d["belems"]) and np.array_equal(Th.blabel, d["blabel"])
    e, f = ffo.boundary_adjacency(Th)
    faces = [[1, 2], [2, 0], [0, 1]] if Th.dim == 2 else [[3, 2, 1], [0, 2, 3], [3, 1, 0], [0, 1, 2]]
    got = np.sort(Th.elems[e[:, None], np.asarray(faces)[f]], axis=1)
    assert np.array_equal(got, np.sort(Th.belems, axis=1))


@pytest.mark.parametrize("name", list(BT_CASES))
def test_oracle_boundary_terms(name):
    c = bt_case(name)
    d, sc = c["d"], c["sc"]
    Vh, A, b = oracle_bt_system(c)
    rp, cl, v = A.csr()
    I = np.repeat(np.arange(Vh.ndof), np.diff(rp))
    assert np.array_equal(I, d["I"]) and np.array_equal(cl, d["J"])
    assert value_errors(v, d["C"], rp).max() <= 1e-12
    assert np.abs(b - d["b"]).max() <= 1e-12 * np.abs(d["b"]).max()
    x, it, r, _ = ffo.cg(A, b, eps=1e-10)
    assert np.linalg.norm(x - d["u"]) <= 1e-9 * np.linalg.norm(d["u"])
    assert it == int(sc["nit"])


def test_oracle_boundary_terms_scalar_bit_exact():
    for name in ["bt_p1sq_6x5", "bt_p2sq_5x4", "bt_p1cube_3x3x2", "bt_p2cube_2x2x2"]:
        c = bt_case(name)
        Vh, A, b = oracle_bt_system(c)
        rp, cl, v = A.csr()
        assert np.array_equal(v, c["d"]["C"]), name
        assert np.array_equal(b, c["d"]["b"]), name
