"""The direct solvers (sparse Cholesky and row-equilibrated sparse QR on the device,
ffgpu_solve_direct) against the oracle and dense solves.

FreeFEM's direct solvers (UMFPACK, CHOLMOD) are not in this image, so the reference is the
oracle's CG driven to eps = 1e-14, whose solution is exact to ~1e-12 on these systems, and
numpy's dense solve on small ones.  Bars: solution within 1e-9 relative (the solution bar of
the FP64 path); one factorisation serves every right-hand side; a reassembly refactors; a
nonsymmetric matrix (tgv = -1 rows, convection) is refused by CHOLESKY and solved by QR under
SPARSESOLVER, FreeFEM's name for its default direct solver; A' x = b (FreeFEM's A'^-1) is solved
from the Cholesky factors of a symmetric matrix and from a QR of A' otherwise, to the same bar.
"""
import numpy as np
import pytest

import ffgpu
import ffo
from ffgpu import mesh
from ffgpu.fespace import FESpace

pytestmark = pytest.mark.gpu

SOL_TOL = 1e-9


@pytest.fixture(scope="module", autouse=True)
def _lib_built():
    from ffgpu.build import build
    build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    ffgpu.context(0)
    yield


@pytest.mark.parametrize("case", ["square64_p1", "square24_p2", "cube8_p1", "cube3_el"])
def test_cholesky_against_oracle(case):
    rng = np.random.Generator(np.random.PCG64(7))
    if case == "cube3_el":
        Th = mesh.cube(3)
        Vh = FESpace(Th, "P2vec")
        a = ffgpu.varf_elasticity(f=(0.0, 0.0, -1.0), on=(4,))
        Ao = ffo.assemble(Th, Vh, form="elasticity")
        bo = ffo.rhs(Th, Vh, f=(0.0, 0.0, -1.0))
        on = Vh.on((4,))
    else:
        Th = {"square64_p1": mesh.square(64), "square24_p2": mesh.square(24), "cube8_p1": mesh.cube(8)}[case]
        kind = "P2" if case.endswith("p2") else "P1"
        Vh = FESpace(Th, kind)
        kappa = np.exp(rng.standard_normal(Th.nt))
        labels = (1, 2, 3, 4) if Th.dim == 2 else (1, 2, 3, 4, 5, 6)
        a = ffgpu.varf_diffusion(kappa=kappa, f=1.0, on=labels)
        Ao = ffo.assemble(Th, Vh, kappa=kappa)
        bo = ffo.rhs(Th, Vh, f=1.0)
        on = Vh.on(labels)
    ffo.setbc(Ao, bo, on)
    uo, _, _, _ = ffo.cg(Ao, bo, eps=1e-14)
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(a, Vh, solver="CHOLESKY", rhs_out=b)
    u = A.solve(b)
    assert A.stats.converged
    assert np.linalg.norm(u - uo) <= SOL_TOL * np.linalg.norm(uo)
    # several right-hand sides on the one factorisation, against numpy where small
    B = rng.standard_normal((3, Vh.ndof))
    X = A.solve(B.ravel()).reshape(3, -1)
    if Vh.ndof <= 3000:
        rp, cl, v = A.csr()
        M = np.zeros((Vh.ndof, Vh.ndof))
        M[np.repeat(np.arange(Vh.ndof), np.diff(rp)), cl] = v
        R = np.linalg.solve(M, B.T).T
        for k in range(3):
            assert np.linalg.norm(X[k] - R[k]) <= SOL_TOL * np.linalg.norm(R[k])
    for k in range(3):
        ok, _, _, _ = ffo.cg(Ao, B[k], eps=1e-14)
        assert np.linalg.norm(X[k] - ok) <= SOL_TOL * np.linalg.norm(ok)


def test_cholesky_refactors_after_reassembly_and_refuses_nonsymmetric():
    Th = mesh.square(20)
    Vh = FESpace(Th, "P1")
    k1 = np.ones(Th.nt)
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(ffgpu.varf_diffusion(kappa=k1, f=1.0, on=(1, 2, 3, 4)), Vh, solver="CHOLESKY", rhs_out=b)
    u1 = A.solve(b)
    A.reassemble(ffgpu.varf_diffusion(kappa=2.0 * k1, f=1.0, on=(1, 2, 3, 4)), rhs_out=b)
    u2 = A.solve(b)
    assert np.linalg.norm(u2 - 0.5 * u1) <= 1e-12 * np.linalg.norm(u1)
    # tgv = -1: the Dirichlet rows become unit rows, the columns stay: not symmetric
    N = ffgpu.matrix(ffgpu.varf_diffusion(f=1.0, on=(1, 2, 3, 4), tgv=-1.0), Vh, solver="CHOLESKY", rhs_out=b)
    with pytest.raises(ffgpu.FFGPUError) as ei:
        N.solve(b)
    assert ei.value.code == -1 and b"symmetric" in ffgpu.lib().ffgpu_last_error()


def _dense(A, n):
    rp, cl, v = A.csr()
    M = np.zeros((n, n))
    M[np.repeat(np.arange(n), np.diff(rp)), cl] = v
    return M


@pytest.mark.parametrize("case", ["tgv_minus1", "advection", "advection_p2"])
def test_sparsesolver_nonsymmetric_against_dense(case):
    """SPARSESOLVER (FreeFEM's direct solver name) on nonsymmetric systems takes the QR path:
    tgv = -1 rows (unit rows, columns kept) and a convection-diffusion operator."""
    rng = np.random.Generator(np.random.PCG64(3))
    if case == "tgv_minus1":
        Th = mesh.square(20)
        Vh = FESpace(Th, "P1")
        a = ffgpu.varf_diffusion(kappa=np.exp(rng.standard_normal(Th.nt)), f=1.0, on=(1, 2, 3, 4), tgv=-1.0)
    else:
        Th = mesh.square(24 if case == "advection" else 12)
        Vh = FESpace(Th, "P2" if case.endswith("p2") else "P1")
        a = ffgpu.varf_diffusion(kappa=0.05, f=1.0, on=(1, 2, 3, 4),
                                 terms=(("id", "dx", 1.0), ("id", "dy", 0.5)))
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(a, Vh, solver="SPARSESOLVER", rhs_out=b)
    M = _dense(A, Vh.ndof)
    assert np.abs(M - M.T).max() > 1e-3 * np.abs(M[np.abs(M) < 1e29]).max()   # really nonsymmetric
    u = A.solve(b)
    ref = np.linalg.solve(M, b)
    assert np.linalg.norm(u - ref) <= SOL_TOL * np.linalg.norm(ref)
    B = rng.standard_normal((2, Vh.ndof))
    X = A.solve(B.ravel()).reshape(2, -1)
    R = np.linalg.solve(M, B.T).T
    for k in range(2):
        assert np.linalg.norm(X[k] - R[k]) <= SOL_TOL * np.linalg.norm(R[k])
    # A' x = b from a QR of A' (UMFPACK_At in FreeFEM), one and several right-hand sides
    ut = A.solve(b, trans=True)
    rt = np.linalg.solve(M.T, b)
    assert np.linalg.norm(ut - rt) <= SOL_TOL * np.linalg.norm(rt)
    Xt = A.solve(B.ravel(), trans=True).reshape(2, -1)
    Rt = np.linalg.solve(M.T, B.T).T
    for k in range(2):
        assert np.linalg.norm(Xt[k] - Rt[k]) <= SOL_TOL * np.linalg.norm(Rt[k])
    # the factorisation of A is still the one A x = b uses
    assert np.linalg.norm(A.solve(b) - ref) <= SOL_TOL * np.linalg.norm(ref)
    with pytest.raises(ffgpu.FFGPUError):
        A.solve(b, solver="CHOLESKY")


def test_qr_on_symmetric_matrix_and_refactor():
    """QR forced on a symmetric positive definite matrix agrees with Cholesky; a reassembly
    refactors."""
    Th = mesh.square(24)
    Vh = FESpace(Th, "P1")
    k1 = np.exp(np.random.Generator(np.random.PCG64(4)).standard_normal(Th.nt))
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(ffgpu.varf_diffusion(kappa=k1, f=1.0, on=(1, 2, 3, 4)), Vh, rhs_out=b)
    uc = A.solve(b, solver="CHOLESKY")
    uq = A.solve(b, solver="QR")
    assert np.linalg.norm(uq - uc) <= SOL_TOL * np.linalg.norm(uc)
    # A' = A: Cholesky answers the transpose solve from its own factors, QR from a QR of A'
    assert np.array_equal(A.solve(b, solver="CHOLESKY", trans=True), uc)
    uqt = A.solve(b, solver="QR", trans=True)
    assert np.linalg.norm(uqt - uc) <= SOL_TOL * np.linalg.norm(uc)
    A.reassemble(ffgpu.varf_diffusion(kappa=3.0 * k1, f=1.0, on=(1, 2, 3, 4)), rhs_out=b)
    uq3 = A.solve(b, solver="QR")
    assert np.linalg.norm(3.0 * uq3 - uc) <= SOL_TOL * np.linalg.norm(uc)
    uq3t = A.solve(b, solver="QR", trans=True)      # both factorisations refactor
    assert np.linalg.norm(3.0 * uq3t - uc) <= SOL_TOL * np.linalg.norm(uc)


def test_transpose_solve_after_reassembly_nonsymmetric():
    """A' x = b on a convection-diffusion matrix, before and after a reassembly with other
    coefficients: the QR of A' refactors with A."""
    Th = mesh.square(16)
    Vh = FESpace(Th, "P1")
    b = np.empty(Vh.ndof)
    a1 = ffgpu.varf_diffusion(kappa=0.05, f=1.0, on=(1, 2, 3, 4), terms=(("id", "dx", 1.0), ("id", "dy", 0.5)))
    a2 = ffgpu.varf_diffusion(kappa=0.1, f=1.0, on=(1, 2, 3, 4), terms=(("id", "dx", -0.5), ("id", "dy", 2.0)))
    A = ffgpu.matrix(a1, Vh, solver="SPARSESOLVER", rhs_out=b)
    c = np.random.Generator(np.random.PCG64(8)).standard_normal(Vh.ndof)
    for a in (a1, a2):
        A.reassemble(a, rhs_out=b)
        M = _dense(A, Vh.ndof)
        rt = np.linalg.solve(M.T, c)
        assert np.linalg.norm(A.solve(c, trans=True) - rt) <= SOL_TOL * np.linalg.norm(rt)
        r = np.linalg.solve(M, c)
        assert np.linalg.norm(A.solve(c) - r) <= SOL_TOL * np.linalg.norm(r)
