"""The CUDA path against the oracle at (or next to) the sizes of the benchmark workloads.

The golden FreeFEM fixtures pin the oracle on small meshes; these tests carry the comparison to
the workloads' own scale, where the oracle still finishes in seconds on one core:
  * 2D P1 Poisson on square(256) -- the full workload;
  * 3D P1 diffusion with a seeded lognormal P0 kappa on cube(40) (the workload is cube(160));
  * [P2,P2,P2] elasticity on cube(12) (the workload is cube(64));
  * the inverse problem's forward solve, adjoint solve and gradient on square(128);
  * all 1024 problems of the batched workload (pattern and values), and a sample of 64
    solutions.
Bars: pattern bit-exact; values within 1e-12 relative per entry, where entries far below their
row's scale are compared at 1e-15 of the row's largest non-tgv entry (a few ulps of the row:
FreeFEM forms some of them as round-off residue of cancelling sums); b within 1e-12 of its
largest entry; FP64 solutions within 1e-9 relative (L2); CG iteration counts within 2; the
mixed-precision solve within 1e-8 of the oracle's FP64 solution."""
import numpy as np
import pytest

import ffgpu
import ffo
from ffgpu import adjoint, batch, mesh
from ffgpu._lib import check
from ffgpu.fespace import FESpace
from golden_cases import value_errors

pytestmark = pytest.mark.gpu

VAL_TOL = 1e-12
SOL_TOL = 1e-9
MIXED_TOL = 1e-8


@pytest.fixture(scope="module", autouse=True)
def _lib_built():
    from ffgpu.build import build
    build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    ffgpu.context(0)
    yield


def _compare(A, b, Ao, bo):
    rp, cl, v = A.csr()
    rpo, clo, vo = Ao.csr()
    assert np.array_equal(rp, rpo) and np.array_equal(cl, clo), "pattern differs from the oracle"
    assert value_errors(v, vo, rpo).max() <= VAL_TOL
    assert np.abs(b - bo).max() <= VAL_TOL * np.abs(bo).max()


def test_poisson_square256_full_size():
    Th = mesh.square(256)
    Vh = FESpace(Th, "P1")
    Ao = ffo.assemble(Th, Vh, quad="qf2pT")
    bo = ffo.rhs(Th, Vh, f=1.0, quad="qf2pT")
    ffo.setbc(Ao, bo, Vh.on((1, 2, 3, 4)))
    uo, it, _, _ = ffo.cg(Ao, bo, eps=1e-10)
    assert it == 532     # FreeFEM's count on this workload
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(ffgpu.varf_diffusion(f=1.0, on=(1, 2, 3, 4)), Vh, eps=1e-10, rhs_out=b)
    assert A.nnz == 460289
    _compare(A, b, Ao, bo)
    u = A.solve(b)
    assert np.linalg.norm(u - uo) <= SOL_TOL * np.linalg.norm(uo)
    assert abs(A.stats.iterations - it) <= 2


def test_lognormal_diffusion_cube40():
    Th = mesh.cube(40)
    Vh = FESpace(Th, "P1")
    kappa = np.exp(np.random.Generator(np.random.PCG64(3)).standard_normal(Th.nt))
    on = (1, 2, 3, 4, 5, 6)
    Ao = ffo.assemble(Th, Vh, kappa=kappa)
    bo = ffo.rhs(Th, Vh, f=1.0)
    ffo.setbc(Ao, bo, Vh.on(on))
    uo, it, _, _ = ffo.cg(Ao, bo, eps=1e-10)
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(ffgpu.varf_diffusion(kappa=kappa, f=1.0, on=on), Vh, eps=1e-10, rhs_out=b)
    assert A.nnz == 993961
    _compare(A, b, Ao, bo)
    u = A.solve(b)
    assert np.linalg.norm(u - uo) <= SOL_TOL * np.linalg.norm(uo)
    assert abs(A.stats.iterations - it) <= 2
    um = A.solve_mixed(b, eps=1e-10)
    assert np.linalg.norm(um - uo) <= MIXED_TOL * np.linalg.norm(uo)
    ud = A.solve(b, spmv_mode=1)
    assert np.linalg.norm(ud - uo) <= SOL_TOL * np.linalg.norm(uo)


def test_elasticity_cube12():
    Th = mesh.cube(12)
    Vh = FESpace(Th, "P2vec")
    Ao = ffo.assemble(Th, Vh, form="elasticity")
    bo = ffo.rhs(Th, Vh, f=(0.0, 0.0, -1.0))
    ffo.setbc(Ao, bo, Vh.on((4,)))
    uo, it, _, _ = ffo.cg(Ao, bo, eps=1e-10)
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(ffgpu.varf_elasticity(E=1.0, nu=0.3, f=(0.0, 0.0, -1.0), on=(4,)), Vh, eps=1e-10,
                     rhs_out=b)
    assert A.nnz == 3758409
    _compare(A, b, Ao, bo)
    u = A.solve(b)
    assert np.linalg.norm(u - uo) <= SOL_TOL * np.linalg.norm(uo)
    assert abs(A.stats.iterations - it) <= 2
    ud = A.solve(b, spmv_mode=1)
    assert np.linalg.norm(ud - uo) <= SOL_TOL * np.linalg.norm(uo)


def _oracle_gradient(Th, Vh, kappa, u_obs, on, eps):
    """Forward CG, transpose CG and the P0 sensitivities -lambda_e' K_e u_e on the oracle."""
    A = ffo.assemble(Th, Vh, kappa=kappa)
    b = ffo.rhs(Th, Vh, f=1.0)
    ffo.setbc(A, b, Vh.on(on))
    u, _, _, _ = ffo.cg(A, b, eps=eps)
    M = ffo.assemble(Th, Vh, mass=1.0, c_stiff=0.0)
    r = u - u_obs
    lam, _, _, _ = ffo.cg(A, M.matmul(r), eps=eps, trans=True)
    X = Th.coords[Th.elems]
    e1, e2 = X[:, 1] - X[:, 0], X[:, 2] - X[:, 0]
    area = 0.5 * (e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0])
    gu = np.zeros((Th.nt, 2))
    gl = np.zeros((Th.nt, 2))
    for i in range(3):
        p1, p2 = X[:, (i + 1) % 3], X[:, (i + 2) % 3]
        G = np.stack([-(p2[:, 1] - p1[:, 1]), p2[:, 0] - p1[:, 0]], axis=1) / (2 * area[:, None])
        gu += G * u[Th.elems[:, i], None]
        gl += G * lam[Th.elems[:, i], None]
    gk = -area * (gu * gl).sum(axis=1)
    return 0.5 * float(r @ M.matmul(r)), u, lam, gk


def test_inverse_problem_gradient_square128():
    rng = np.random.Generator(np.random.PCG64(4))
    Th = mesh.square(128)
    Vh = FESpace(Th, "P1")
    on = (1, 2, 3, 4)
    P = adjoint.DiffusionProblem(Vh, on=on, eps=1e-12)
    u_true = P.solve(np.exp(rng.standard_normal(Th.nt)), np.ones(Th.nt))
    u_obs = u_true + 0.01 * np.sqrt(np.mean(u_true ** 2)) * rng.standard_normal(Vh.ndof)
    L, gk, gf, u, lam = P.value_and_grad(np.ones(Th.nt), np.ones(Th.nt), u_obs)
    Lo, uo, lamo, gko = _oracle_gradient(Th, Vh, np.ones(Th.nt), u_obs, on, 1e-12)
    assert np.linalg.norm(u - uo) <= SOL_TOL * np.linalg.norm(uo)
    assert np.linalg.norm(lam - lamo) <= SOL_TOL * np.linalg.norm(lamo)
    assert abs(L - Lo) <= SOL_TOL * abs(Lo)
    assert np.linalg.norm(gk - gko) <= SOL_TOL * np.linalg.norm(gko)


def test_batched_workload_all_problems():
    meshes, kappas, Ns = batch.c5_meshes(1024, 16, 128, seed=0)
    B = batch.Batch(meshes)
    B.assemble(kappas, f=1.0)
    x = B.solve(eps=1e-8)
    bb = B.rhs()
    import ctypes as C
    h = ffgpu.lib().ffgpu_batch_matrix(B.h)
    n, nnz, bs = C.c_int(), C.c_int64(), C.c_int()
    ffgpu.lib().ffgpu_matrix_info(h, C.byref(n), C.byref(nnz), C.byref(bs))
    rp = np.empty(n.value + 1, np.int32); cl = np.empty(nnz.value, np.int32); vl = np.empty(nnz.value)
    check(ffgpu.lib().ffgpu_matrix_csr(h, rp.ctypes.data_as(C.c_void_p), cl.ctypes.data_as(C.c_void_p),
                                             vl.ctypes.data_as(C.c_void_p)))
    xs, bs_ = B.split(x), B.split(bb)
    solve_sample = set(np.random.Generator(np.random.PCG64(1)).choice(1024, size=64, replace=False).tolist())
    for p, (Th, k) in enumerate(zip(meshes, kappas)):
        Vh = FESpace(Th, "P1")
        Ao = ffo.assemble(Th, Vh, kappa=k)
        bo = ffo.rhs(Th, Vh, f=1.0)
        ffo.setbc(Ao, bo, Vh.on((1, 2, 3, 4)))
        r0, r1 = B.voff[p], B.voff[p + 1]
        orp, ocl, ovl = Ao.csr()
        assert np.array_equal(rp[r0:r1 + 1] - rp[r0], orp), p
        assert np.array_equal(cl[rp[r0]:rp[r1]] - r0, ocl), p
        assert value_errors(vl[rp[r0]:rp[r1]], ovl, orp).max() <= VAL_TOL, p
        assert np.abs(bs_[p] - bo).max() <= VAL_TOL * np.abs(bo).max(), p
        if p in solve_sample:
            uo, _, _, _ = ffo.cg(Ao, bo, eps=1e-10)
            # FP32 inner / FP64 refinement to eps 1e-8 (conditioning allowance 100, as the
            # batched tests state)
            assert np.linalg.norm(xs[p] - uo) <= 1e-6 * np.linalg.norm(uo), p
