"""Mixed precision (FP32 inner PCG + FP64 refinement) against the FP64 oracle solution.

The outer loop stops on FreeFEM's CG test applied to the true FP64 residual, so the
solution is compared with the FP64 oracle's at the same eps; the bar is 1e-8 relative in
the L2 norm (the tolerance the mixed path is specified at)."""
import numpy as np
import pytest

import ffgpu
import ffo
from ffgpu import mesh
from ffgpu.fespace import FESpace

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-8


@pytest.fixture(scope="module", autouse=True)
def _lib_built():
    from ffgpu.build import build
    build()
    ffgpu.context(0)
    yield


def oracle_solution(Th, Vh, kappa=None, form="diffusion", f=1.0, labels=(1, 2, 3, 4), quad=None, eps=1e-10):
    A = ffo.assemble(Th, Vh, form=form, kappa=kappa, quad=quad)
    b = ffo.rhs(Th, Vh, f=f, quad=quad)
    ffo.setbc(A, b, Vh.on(labels))
    u, it, r, _ = ffo.cg(A, b, eps=eps)
    return u, it


@pytest.mark.parametrize("n", [8, 14])
def test_mixed_3d_diffusion_lognormal_kappa(n):
    rng = np.random.Generator(np.random.PCG64(100 + n))
    Th = mesh.cube(n)
    Vh = FESpace(Th, "P1")
    kappa = np.exp(rng.standard_normal(Th.nt))
    labels = (1, 2, 3, 4, 5, 6)
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(ffgpu.varf_diffusion(kappa=kappa, f=1.0, on=labels), Vh, eps=1e-10, rhs_out=b)
    u = A.solve_mixed(b, eps=1e-10)
    st = A.stats
    assert st.converged and st.outer_iterations >= 1
    uo, it = oracle_solution(Th, Vh, kappa=kappa, labels=labels)
    err = np.linalg.norm(u - uo) / np.linalg.norm(uo)
    assert err <= MIXED_TOL, err
    u64 = A.solve(b)
    assert np.linalg.norm(u64 - uo) <= 1e-9 * np.linalg.norm(uo)


def test_mixed_2d_poisson_and_elasticity():
    Th = mesh.square(64)
    Vh = FESpace(Th, "P1")
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(ffgpu.varf_diffusion(f=1.0, on=(1, 2, 3, 4)), Vh, eps=1e-10, rhs_out=b)
    u = A.solve_mixed(b)
    uo, _ = oracle_solution(Th, Vh)
    assert np.linalg.norm(u - uo) <= MIXED_TOL * np.linalg.norm(uo)
    Th = mesh.cube(5)
    Vh = FESpace(Th, "P2vec")
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(ffgpu.varf_elasticity(f=(0, 0, -1.0), on=(4,)), Vh, eps=1e-10, rhs_out=b)
    u = A.solve_mixed(b)
    uo, _ = oracle_solution(Th, Vh, form="elasticity", f=(0, 0, -1.0), labels=(4,))
    assert np.linalg.norm(u - uo) <= MIXED_TOL * np.linalg.norm(uo)


def test_mixed_outer_cap_reports_nonconvergence():
    Th = mesh.square(32)
    Vh = FESpace(Th, "P1")
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(ffgpu.varf_diffusion(f=1.0, on=(1, 2, 3, 4)), Vh, eps=1e-10, rhs_out=b)
    with pytest.raises(ffgpu.FFGPUError):
        A.solve_mixed(b, eps_inner=0.5, itmax_inner=2, max_outer=1)
