"""The CG loop of small scalar systems in one thread-block cluster (ffgpu_cluster.cu).

The path is opt-in (FFGPU_CLUSTER_CG=1: on GB300 the FP64 work of an iteration needs more SMs
than one cluster has, so the three-kernel graph is faster); with it, systems of up to
8 x 9216 rows take it (a rule on the sizes, not on timings).  Same bars as the other CG tests: solution within 1e-9 of the oracle (FreeFEM's
ConjugueGradient restated), iteration counts within 2; against the regular three-kernel
path (a fixed SpMV layout selects it) the rows sum in the same order, so only the dot
products' order differs: solutions within 1e-12, iterations within 1.
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
    os.environ["FFGPU_CLUSTER_CG"] = "1"
    yield
    del os.environ["FFGPU_CLUSTER_CG"]


def _problem(Th, kind="P1", seed=1):
    Vh = FESpace(Th, kind)
    kappa = np.exp(np.random.Generator(np.random.PCG64(seed)).standard_normal(Th.nt))
    on = (1, 2, 3, 4) if Th.dim == 2 else (1, 2, 3, 4, 5, 6)
    Ao = ffo.assemble(Th, Vh, kappa=kappa)
    bo = ffo.rhs(Th, Vh, f=1.0)
    ffo.setbc(Ao, bo, Vh.on(on))
    return Vh, ffgpu.varf_diffusion(kappa=kappa, f=1.0, on=on), Ao, bo


def _solve_counting(A, b, **kw):
    l0 = ffgpu.kernel_launches()
    u = A.solve(b, **kw)
    return u, ffgpu.kernel_launches() - l0


@pytest.mark.parametrize("case", ["square64", "square64_p2", "cube16", "square256"])
def test_cluster_cg_against_oracle(case):
    Th = {"square64": mesh.square(64), "square64_p2": mesh.square(64), "cube16": mesh.cube(16),
          "square256": mesh.square(256)}[case]
    Vh, a, Ao, bo = _problem(Th, "P2" if case.endswith("p2") else "P1")
    uo, it, _, _ = ffo.cg(Ao, bo, eps=1e-10)
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(a, Vh, eps=1e-10, rhs_out=b)
    A.solve(b)                              # first solve: solver setup and SpMV tuning
    assert ffgpu.lib().ffgpu_matrix_spmv_layout(A.h, 5) == 1, ffgpu.lib().ffgpu_last_error()
    u, launches = _solve_counting(A, b)
    assert launches < 8, launches           # one kernel for the whole iteration loop
    assert np.linalg.norm(u - uo) <= 1e-9 * np.linalg.norm(uo)
    assert abs(A.stats.iterations - it) <= 2
    # the regular path (a fixed layout) on the same matrix
    A.solve(b, spmv_layout=64)
    ur, launches_r = _solve_counting(A, b, spmv_layout=64)
    assert ffgpu.lib().ffgpu_matrix_spmv_layout(A.h, 5) == 0
    assert launches_r >= 2 * A.stats.iterations   # two kernels per iteration (fused direction update)
    assert np.linalg.norm(u - ur) <= 1e-12 * np.linalg.norm(ur)
    # reproducible
    u2 = A.solve(b)
    assert np.array_equal(u, u2)


def test_cluster_cg_transpose_and_nonconvergence():
    Vh, a, Ao, bo = _problem(mesh.square(48), seed=4)
    c = np.random.Generator(np.random.PCG64(8)).standard_normal(Vh.ndof)
    uo, it, _, _ = ffo.cg(Ao, c, eps=1e-10, trans=True)
    A = ffgpu.matrix(a, Vh, eps=1e-10)
    u = A.solve(c, trans=True)
    assert np.linalg.norm(u - uo) <= 1e-9 * np.linalg.norm(uo)
    assert abs(A.stats.iterations - it) <= 2
    B = ffgpu.matrix(a, Vh, eps=1e-10, itmax=3)
    with pytest.raises(ffgpu.FFGPUError) as ei:
        B.solve(c)
    assert ei.value.code == -3 and B.stats.iterations == 3


def test_cluster_cg_can_be_switched_off():
    Vh, a, Ao, bo = _problem(mesh.square(40), seed=6)
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(a, Vh, eps=1e-10, rhs_out=b)
    A.solve(b)
    u1, l1 = _solve_counting(A, b)
    os.environ["FFGPU_CLUSTER_CG"] = "0"
    try:
        A.solve(b)
        u2, l2 = _solve_counting(A, b)
    finally:
        os.environ["FFGPU_CLUSTER_CG"] = "1"
    assert l1 < 8 < l2
    assert np.linalg.norm(u1 - u2) <= 1e-12 * np.linalg.norm(u2)
