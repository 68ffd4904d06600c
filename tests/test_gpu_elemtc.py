"""P2 element matrices on the tensor cores (ffgpu_elemtc.cu) against the FP64 path.

The tensor-core path forms every element matrix as the exact integer product of the reference
tensor M with the elements' features rounded to 53-bit fixed point, so it agrees with the FP64
evaluation (FFGPU_ELEM_TC=0: the rank-structured P2 factorisation inside the row gather) to
rounding: entries within 1e-14 of their row's largest entry.  Patterns are the same (the
pattern pass does not depend on the values), the matrices symmetric to rounding, and the
FreeFEM fixtures (tests/test_gpu_parity.py) run through this path by default.
"""
import os

import numpy as np
import pytest

import ffgpu
import ffo
from ffgpu import mesh
from ffgpu.fespace import FESpace

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib_built():
    from ffgpu.build import build
    build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    ffgpu.context(0)
    yield


def _assemble(a, Vh, tc):
    old = os.environ.get("FFGPU_ELEM_TC")
    os.environ["FFGPU_ELEM_TC"] = "1" if tc else "0"
    try:
        b = np.empty(Vh.ndof)
        A = ffgpu.matrix(a, Vh, rhs_out=b)
        return A.csr(), b
    finally:
        if old is None:
            del os.environ["FFGPU_ELEM_TC"]
        else:
            os.environ["FFGPU_ELEM_TC"] = old


def _rows_close(c1, c2, tol):
    rp, cl, v1 = c1
    rp2, cl2, v2 = c2
    assert np.array_equal(rp, rp2) and np.array_equal(cl, cl2)
    row = np.repeat(np.arange(rp.size - 1), np.diff(rp))
    scale = np.maximum.reduceat(np.abs(v2), rp[:-1])
    err = np.abs(v1 - v2) / scale[row]
    return float(err.max())


def _case(name):
    rng = np.random.Generator(np.random.PCG64(11))
    if name == "square12_p2":
        Th = mesh.square(12)
        Vh = FESpace(Th, "P2")
        return Vh, ffgpu.varf_diffusion(kappa=np.exp(rng.standard_normal(Th.nt)), f=1.0, on=(1, 2, 3, 4))
    if name == "jittered_p2":
        Th = mesh.jittered_square(20, 0.25, rng)
        Vh = FESpace(Th, "P2")
        return Vh, ffgpu.varf_diffusion(kappa=2.5, f=1.0, on=(1, 2))
    if name == "cube4_p2_mass":
        Th = mesh.cube(4)
        Vh = FESpace(Th, "P2")
        return Vh, ffgpu.varf_diffusion(kappa=np.exp(rng.standard_normal(Th.nt)), c_mass=3.0, f=1.0,
                                        on=(1, 2, 3, 4, 5, 6))
    if name == "cube4_elasticity":
        Th = mesh.cube(4)
        Vh = FESpace(Th, "P2vec")
        return Vh, ffgpu.varf_elasticity(E=1.0, nu=0.3, on=(4,))
    if name == "cube5_two_materials":
        Th = mesh.cube(5)
        Vh = FESpace(Th, "P2vec")
        E = np.where(rng.random(Th.nt) < 0.5, 1.0, 20.0)
        nu = np.where(rng.random(Th.nt) < 0.5, 0.3, 0.45)
        return Vh, ffgpu.varf_elasticity(E=E, nu=nu, on=(4,))
    if name == "distorted_cube3_elasticity":
        Th = mesh.cube(3)
        X = Th.coords + 0.08 * rng.uniform(-1, 1, Th.coords.shape) * (Th.coords * (1 - Th.coords) > 0)
        Th = mesh.movemesh(Th, X)
        Vh = FESpace(Th, "P2vec")
        return Vh, ffgpu.varf_elasticity(E=3.0, nu=0.25, on=(4, 2))
    raise KeyError(name)


@pytest.mark.parametrize("name", ["square12_p2", "jittered_p2", "cube4_p2_mass", "cube4_elasticity",
                                  "cube5_two_materials", "distorted_cube3_elasticity"])
def test_tensor_core_elements_match_fp64(name):
    Vh, a = _case(name)
    c_tc, b_tc = _assemble(a, Vh, True)
    c_64, b_64 = _assemble(a, Vh, False)
    assert _rows_close(c_tc, c_64, 1e-14) <= 1e-14
    assert np.array_equal(b_tc, b_64)          # the linear form does not go through the tensor cores
    # symmetric to rounding (the element matrices are exactly symmetric; rows i and j sum
    # their shared elements in different association orders)
    rp, cl, v = c_tc
    n = rp.size - 1
    row = np.repeat(np.arange(n), np.diff(rp))
    key = row.astype(np.int64) * n + cl
    tkey = cl.astype(np.int64) * n + row
    order = np.argsort(key)
    pos = np.searchsorted(key[order], tkey)
    scale = np.maximum.reduceat(np.abs(np.where(np.abs(v) < 1e29, v, 0.0)), rp[:-1])
    assert np.all(np.abs(v - v[order][pos]) <= 1e-14 * scale[row])


def test_tensor_core_elements_against_oracle_solution():
    """[P2]^3 elasticity on cube(4): the tensor-core matrix solves to the oracle's solution."""
    Th = mesh.cube(4)
    Vh = FESpace(Th, "P2vec")
    Ao = ffo.assemble(Th, Vh, form="elasticity")
    bo = ffo.rhs(Th, Vh, f=(0.0, 0.0, -1.0))
    ffo.setbc(Ao, bo, Vh.on((4,)))
    uo, ito, _, _ = ffo.cg(Ao, bo, eps=1e-12)
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(ffgpu.varf_elasticity(on=(4,)), Vh, eps=1e-12, rhs_out=b)
    u = A.solve(b)
    assert np.linalg.norm(u - uo) <= 1e-9 * np.linalg.norm(uo)
    assert abs(A.stats.iterations - ito) <= 2
