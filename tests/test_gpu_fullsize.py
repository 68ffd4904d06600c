"""The two 3D workloads at their full sizes, checked through properties that do not need an
oracle run at that size: the pattern size, the kernel of the operator (rigid translations of
the elasticity stiffness, constants of the diffusion operator, on every row off the Dirichlet
boundary), symmetry, the true residual of the FP64 solve, and the agreement of independent
arithmetic paths (double-float SpMV CG, FP32-inner refinement) with the FP64 solve.  Meshes,
numbering and spaces are built on the device."""
import numpy as np
import pytest

import ffgpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib_built():
    from ffgpu.build import build
    build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    ffgpu.context(0)
    yield


def _operator_checks(A, n, off, kernel_vectors, dev):
    import torch
    g = torch.Generator(device=dev).manual_seed(11)
    # random vectors vanishing on the Dirichlet rows (whose diagonal is tgv)
    x = (torch.rand(n, dtype=torch.float64, device=dev, generator=g) - 0.5) * off
    y = (torch.rand(n, dtype=torch.float64, device=dev, generator=g) - 0.5) * off
    Ax, Ay = A.mult(x), A.mult(y)
    scale = float(Ax[off].abs().max())
    # symmetry: x.(A y) = y.(A x)
    assert abs(float(x @ Ay - y @ Ax)) <= 1e-12 * float(x.abs() @ Ay.abs())
    # kernel vectors: A t = 0 on the rows off the Dirichlet boundary
    for t in kernel_vectors:
        r = A.mult(t)
        assert float(r[off].abs().max()) <= 1e-12 * scale


def test_elasticity_cube64_full_size():
    import torch
    dev = torch.device("cuda", 0)
    S = ffgpu.device_space("P2vec", 3, 64)
    n = S.Vh.ndof
    assert n == 3 * 129 ** 3
    b = torch.empty(n, dtype=torch.float64, device=dev)
    A = ffgpu.matrix(ffgpu.varf_elasticity(E=1.0, nu=0.3, f=(0.0, 0.0, -1.0), on=(4,)), S, eps=1e-10,
                     rhs_out=b, itmax=20000)
    assert A.nnz == 547739145
    off = ~torch.from_numpy(S.bc_mask((4,)).astype(bool)).to(dev)
    ts = []
    for c in range(3):
        t = torch.zeros(n, dtype=torch.float64, device=dev)
        t[c::3] = 1.0
        ts.append(t)
    _operator_checks(A, n, off, ts, dev)
    u = A.solve(b)
    assert A.stats.converged and abs(A.stats.iterations - 3647) <= 20
    r = b - A.mult(u)
    assert float(torch.linalg.norm(r[off]) / torch.linalg.norm(b[off])) <= 1e-9
    u2 = A.solve(b, spmv_mode=1)
    assert float(torch.linalg.norm(u2 - u) / torch.linalg.norm(u)) <= 1e-9


def test_diffusion_cube160_full_size():
    import torch
    dev = torch.device("cuda", 0)
    S = ffgpu.device_space("P1", 3, 160)
    n, nt = S.Vh.ndof, S.Vh.Th.nt
    assert n == 161 ** 3 and nt == 6 * 160 ** 3
    g = torch.Generator(device=dev).manual_seed(3)
    kap = torch.exp(torch.randn(nt, dtype=torch.float64, device=dev, generator=g))
    b = torch.empty(n, dtype=torch.float64, device=dev)
    A = ffgpu.matrix(ffgpu.varf_diffusion(kappa=kap, f=1.0, on=(1, 2, 3, 4, 5, 6)), S, eps=1e-10, rhs_out=b)
    assert A.nnz == 61979041
    off = ~torch.from_numpy(S.bc_mask((1, 2, 3, 4, 5, 6)).astype(bool)).to(dev)
    _operator_checks(A, n, off, [torch.ones(n, dtype=torch.float64, device=dev)], dev)
    u = A.solve(b)
    r = b - A.mult(u)
    assert float(torch.linalg.norm(r[off]) / torch.linalg.norm(b[off])) <= 1e-9
    um = A.solve_mixed(b, eps=1e-10)
    assert float(torch.linalg.norm(um - u) / torch.linalg.norm(u)) <= 1e-8
