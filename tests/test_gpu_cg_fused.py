"""The two-kernel CG iteration of small scalar systems (cg_kca_sell + K_b storing C G).

H' = gamma H - C G is formed where the SpMV gathers it, so an iteration is two kernels instead of
three.  The direction update has the same roundings as the three-kernel path's K_c, the rows sum
in the same order; only the dot products (G, H) are summed in another order.  Bars: solutions
within 1e-12 of the three-kernel path (FFGPU_CG_FUSE=0) and within 1e-9 of the oracle, iteration
counts within 1 and 2; the host-driven loop gives the graph's bits; two launches per iteration.
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


def _problem(name):
    rng = np.random.Generator(np.random.PCG64(5))
    Th = {"square64": mesh.square(64), "square40_p2": mesh.square(40), "cube10": mesh.cube(10)}[name]
    Vh = FESpace(Th, "P2" if name.endswith("p2") else "P1")
    kappa = np.exp(rng.standard_normal(Th.nt))
    on = (1, 2, 3, 4) if Th.dim == 2 else (1, 2, 3, 4, 5, 6)
    Ao = ffo.assemble(Th, Vh, kappa=kappa)
    bo = ffo.rhs(Th, Vh, f=1.0)
    ffo.setbc(Ao, bo, Vh.on(on))
    return Vh, ffgpu.varf_diffusion(kappa=kappa, f=1.0, on=on), Ao, bo


def _solve(A, b, env=None, **kw):
    old = {k: os.environ.get(k) for k in (env or {})}
    os.environ.update(env or {})
    try:
        A.solve(b, **kw)                     # setup, tuning, graph
        l0 = ffgpu.kernel_launches()
        u = A.solve(b, **kw)
        return u, ffgpu.kernel_launches() - l0, A.stats.iterations
    finally:
        for k, v in old.items():
            if v is None:
                del os.environ[k]
            else:
                os.environ[k] = v


@pytest.mark.parametrize("name", ["square64", "square40_p2", "cube10"])
@pytest.mark.parametrize("trans", [False, True])
def test_fused_iteration_against_three_kernels_and_oracle(name, trans):
    Vh, a, Ao, bo = _problem(name)
    c = np.random.Generator(np.random.PCG64(2)).standard_normal(Vh.ndof) if trans else None
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(a, Vh, eps=1e-10, rhs_out=b)
    rhs = c if trans else b
    uf, lf, itf = _solve(A, rhs, trans=trans)
    u3, l3, it3 = _solve(A, rhs, env={"FFGPU_CG_FUSE": "0"}, trans=trans)
    assert np.linalg.norm(uf - u3) <= 1e-12 * np.linalg.norm(u3)
    assert abs(itf - it3) <= 1
    assert lf <= 2 * itf + 24 and l3 >= 3 * it3, (lf, itf, l3, it3)
    uo, ito, _, _ = ffo.cg(Ao, rhs, eps=1e-10, trans=trans)
    assert np.linalg.norm(uf - uo) <= 1e-9 * np.linalg.norm(uo)
    assert abs(itf - ito) <= 2
    # the host-driven loop launches the same kernels: same bits
    uh, _, _ = _solve(A, rhs, env={"FFGPU_CG_GRAPH": "0"}, trans=trans)
    assert np.array_equal(uh, uf)
    # reproducible
    assert np.array_equal(A.solve(rhs, trans=trans), uf)
