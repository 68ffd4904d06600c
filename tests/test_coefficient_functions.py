"""Matrix coefficients that are functions of the point: int(Th)(c(x,y[,z]) * u * v) and
int(Th)(k(x,y[,z]) * grad u . grad v).

FreeFEM takes them at the points of the form's rule (Element_Op, problem.cpp:6063-6160,
6337-6437).  The fixtures ``mq_*`` hold FreeFEM's matrix, b and solution of
-div grad u + c u = 1 for four mass coefficients, ``kq_*`` those of -div(k grad u) = 1 for
three stiffness coefficients (P1 and P2, squares and cubes); the oracle and the device
(``ffgpu_varf.mass_qp``, ``stiff_qp``) reproduce the pattern exactly and the values within 1e-12.
"""
import numpy as np
import pytest

import ffgpu
import ffo
from ffgpu import mesh
from ffgpu.fespace import FESpace
from golden_cases import load, value_errors

CASES = {
    "mq_sq_p1": ("P1", lambda x, y: 1 + x * y, (1,)),
    "mq_sq_p2": ("P2", lambda x, y: np.exp(x + y), (1, 2)),
    "mq_cube_p1": ("P1", lambda x, y, z: 1 + z * x, (1,)),
    "mq_cube_p2": ("P2", lambda x, y, z: 2 + np.cos(x) * y, (1,)),
    "kq_sq_p1": ("P1", lambda x, y: 1 + x * x * y, (1, 3)),
    "kq_sq_p2": ("P2", lambda x, y: np.exp(x - y), (1, 2)),
    "kq_cube_p2": ("P2", lambda x, y, z: 1 + x * y * z, (1, 2)),
}


def coefs(name, c):
    """(kappa, mass) keyword values of the case's coefficient function."""
    return (c, 0.0) if name.startswith("kq_") else (None, c)


def space(name):
    d, sc = load(name)
    dim = d["coords"].shape[1]
    Th = mesh.Mesh(dim, d["coords"], d["elems"], d["belems"], d["blabel"], d["vlabel"])
    Vh = FESpace(Th, CASES[name][0])
    assert np.array_equal(Vh.dof, d["dof"])
    return d, sc, Th, Vh


def check(d, sc, rp, cl, v, b, u, it):
    I = np.repeat(np.arange(rp.size - 1), np.diff(rp))
    assert np.array_equal(I, d["I"]) and np.array_equal(cl, d["J"])
    assert value_errors(v, d["C"], rp).max() <= 1e-12
    assert np.abs(b - d["b"]).max() <= 1e-12 * np.abs(d["b"]).max()
    assert np.linalg.norm(u - d["u"]) <= 1e-9 * np.linalg.norm(d["u"])
    assert abs(it - int(sc["nit"])) <= 2


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_coefficient_function_equals_freefem(name):
    d, sc, Th, Vh = space(name)
    _, c, labels = CASES[name]
    kappa, mass = coefs(name, c)
    A = ffo.assemble(Th, Vh, kappa=kappa, mass=mass)
    b = ffo.rhs(Th, Vh, f=1.0)
    ffo.setbc(A, b, Vh.on(labels))
    rp, cl, v = A.csr()
    u, it, _, _ = ffo.cg(A, b, eps=1e-12)
    check(d, sc, rp, cl, v, b, u, it)


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_device_coefficient_function_equals_freefem(name):
    from ffgpu.build import build
    build()
    d, sc, Th, Vh = space(name)
    _, c, labels = CASES[name]
    kappa, mass = coefs(name, c)
    a = ffgpu.varf_diffusion(kappa=kappa, c_mass=mass, f=1.0, on=labels)
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(a, Vh, eps=1e-12, rhs_out=b)
    rp, cl, v = A.csr()
    u = A.solve(b)
    check(d, sc, rp, cl, v, b, u, A.stats.iterations)


def test_varf_carries_every_function_at_one_rule():
    """The C varf of a form with several functions holds them all, at one rule (host only)."""
    Vh = FESpace(mesh.square(3), "P2")
    a = ffgpu.varf_diffusion(kappa=lambda x, y: 1 + x, c_mass=lambda x, y: 2 + y, f=lambda x, y: x * y)
    v = a.c_varf(Vh)
    assert v.nqp == 7 and v.stiff_qp and v.mass_qp and v.f_qp and v.qp_lambda and v.qp_weight
    assert not v.kappa and v.c_mass == 0.0


def test_constant_kappa_and_kappa_shape():
    """A constant kappa is part of c_stiff (no per-element array crosses); a P0 array must
    have one value per element (host only)."""
    Vh = FESpace(mesh.square(3), "P1")
    v = ffgpu.varf_diffusion(kappa=2.5, c_stiff=2.0).c_varf(Vh)
    assert not v.kappa and v.c_stiff == 5.0
    v = ffgpu.varf_diffusion(kappa=np.full(Vh.Th.nt, 2.5)).c_varf(Vh)
    assert v.kappa and v.c_stiff == 1.0
    with pytest.raises(ValueError):
        ffgpu.varf_diffusion(kappa=np.ones(5)).c_varf(Vh)


def _materials():
    d, sc = load("p2elmat_2x2x1")
    Th = mesh.Mesh(3, d["coords"], d["elems"], d["belems"], d["blabel"], d["vlabel"])
    Vh = FESpace(Th, "P2vec")
    assert np.array_equal(Vh.dof, d["dof"])
    return d, sc, Th, Vh, d["in_E"], d["in_nu"]


def test_oracle_elasticity_with_materials_equals_freefem():
    """[P2,P2,P2] elasticity with E and nu per element (two materials, P0 Lame coefficients)."""
    d, sc, Th, Vh, E, nu = _materials()
    A = ffo.assemble(Th, Vh, form="elasticity", E=E, nu=nu)
    b = ffo.rhs(Th, Vh, f=(0.0, 0.0, -1.0))
    ffo.setbc(A, b, Vh.on((4,)))
    rp, cl, v = A.csr()
    u, it, _, _ = ffo.cg(A, b, eps=1e-10)
    check(d, sc, rp, cl, v, b, u, it)


@pytest.mark.gpu
def test_device_elasticity_with_materials_equals_freefem():
    from ffgpu.build import build
    build()
    d, sc, Th, Vh, E, nu = _materials()
    a = ffgpu.varf_elasticity(E=E, nu=nu, f=(0.0, 0.0, -1.0), on=(4,))
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(a, Vh, eps=1e-10, rhs_out=b)
    rp, cl, v = A.csr()
    u = A.solve(b)
    check(d, sc, rp, cl, v, b, u, A.stats.iterations)
