"""Sources that are functions of the coordinates: int(Th)(f(x,y[,z]) * v).

FreeFEM takes such a source at the points of the form's quadrature rule (Element_rhs,
problem.cpp:7839-7911, 7917-7990).  The fixtures ``src_*`` hold FreeFEM's b = a(0,Vh) for six
sources (P1 and P2 on squares and cubes, the qf2pT rule, a [P2,P2,P2] load); the oracle and
the device (``ffgpu_varf.f_qp``) reproduce them within 1e-12 of max |b| (the values of f at
the points agree with FreeFEM's to rounding, the sums run in another order).
"""
import numpy as np
import pytest

import ffgpu
import ffo
from ffgpu import mesh
from ffgpu.fespace import FESpace
from golden_cases import load

TOL = 1e-12

CASES = {
    "src_sq_p1": ("P1", lambda x, y: np.sin(3 * x) * np.cos(2 * y) + x * y, None),
    "src_sq_p1_qf2": ("P1", lambda x, y: np.exp(x) * (1 + y * y), "qf2pT"),
    "src_sq_p2": ("P2", lambda x, y: np.exp(x) * y - np.cos(5 * y), None),
    "src_cube_p1": ("P1", lambda x, y, z: x * y * z + np.sin(2 * z), None),
    "src_cube_p2": ("P2", lambda x, y, z: np.cos(x + 2 * y) * z, None),
    "src_cube_el": ("P2vec", lambda x, y, z: (x, y * z, -1 + x * x), None),
}


def space(name):
    d, _ = load(name)
    kind = CASES[name][0]
    dim = d["coords"].shape[1]
    Th = mesh.Mesh(dim, d["coords"], d["elems"], d["belems"], d["blabel"], d["vlabel"])
    Vh = FESpace(Th, kind)
    assert np.array_equal(Vh.dof, d["dof"])          # FreeFEM's numbering, P2 in 2D included
    return d, Th, Vh


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_source_function_equals_freefem(name):
    d, Th, Vh = space(name)
    _, f, quad = CASES[name]
    b = ffo.rhs(Th, Vh, f=f, quad=quad)
    assert np.max(np.abs(b - d["b"])) <= TOL * np.max(np.abs(d["b"]))


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_device_source_function_equals_freefem(name):
    from ffgpu.build import build
    build()
    d, Th, Vh = space(name)
    kind, f, quad = CASES[name]
    if kind == "P2vec":
        a = ffgpu.varf_elasticity(f=f, quad=quad)
    else:
        a = ffgpu.varf_diffusion(f=f, quad=quad)
    b = ffgpu.rhs(a, Vh)
    assert np.max(np.abs(b - d["b"])) <= TOL * np.max(np.abs(d["b"]))
    # the same source through the fused matrix + linear form pass
    b2 = np.empty(Vh.ndof)
    ffgpu.matrix(a, Vh, rhs_out=b2)
    assert np.max(np.abs(b2 - d["b"])) <= TOL * np.max(np.abs(d["b"]))
