"""Adjoint gradients on the device path.

* against FreeFEM's own FP64 adjoint written as a script (fixture adj_p1_n8: forward CG,
  transpose solve A'^-1, P0 sensitivities by a varf) -- 1e-9 relative;
* against central finite differences (step 1e-6 relative to kappa_e) on seeded elements --
  1e-6 relative per element (floor 1e-3 x the largest gradient entry);
* the implicit-Euler heat variant: forward against FreeFEM (fixture heat_p1_n6), the
  checkpointed adjoint against the adjoint that keeps every state, and against central FD.
"""
import numpy as np
import pytest

import ffgpu
from ffgpu import adjoint, mesh
from ffgpu.fespace import FESpace
from golden_cases import load

pytestmark = pytest.mark.gpu

FD_TOL = 1e-6


@pytest.fixture(scope="module", autouse=True)
def _lib_built():
    from ffgpu.build import build
    build()
    ffgpu.context(0)
    yield


def rel_err(a, b):
    a = np.asarray(a); b = np.asarray(b)
    floor = 1e-3 * np.abs(b).max()
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


def test_adjoint_against_freefem_script():
    d, sc = load("adj_p1_n8")
    Th = mesh.square(8)
    Vh = FESpace(Th, "P1")
    P = adjoint.DiffusionProblem(Vh, eps=1e-14)
    L, gk, gf, u, lam = P.value_and_grad(d["in_kappa"], d["in_f"], d["in_uobs"])
    assert abs(L - sc["loss"]) <= 1e-10 * abs(sc["loss"])
    assert np.linalg.norm(u - d["u"]) <= 1e-10 * np.linalg.norm(d["u"])
    assert np.linalg.norm(lam - d["g_lam"]) <= 1e-8 * np.linalg.norm(d["g_lam"])
    assert np.linalg.norm(gk - d["g_gkappa"]) <= 1e-9 * np.linalg.norm(d["g_gkappa"])
    assert np.linalg.norm(gf - d["g_gf"]) <= 1e-9 * np.linalg.norm(d["g_gf"])


@pytest.mark.parametrize("n", [16, 64])
def test_adjoint_against_central_fd(n):
    rng = np.random.Generator(np.random.PCG64(2024 + n))
    Th = mesh.square(n)
    Vh = FESpace(Th, "P1")
    P = adjoint.DiffusionProblem(Vh, eps=1e-14)
    kappa = np.exp(0.5 * rng.standard_normal(Th.nt))
    f = np.ones(Th.nt)
    u_true = P.solve(np.exp(0.3 * rng.standard_normal(Th.nt)), f)
    u_obs = u_true + 0.01 * np.sqrt(np.mean(u_true ** 2)) * rng.standard_normal(Vh.ndof)
    L, gk, gf, u, lam = P.value_and_grad(kappa, f, u_obs)
    elems = rng.choice(Th.nt, size=16 if n == 16 else 64, replace=False)
    fd = P.fd_gradient(kappa, f, u_obs, elems, step=1e-6)
    err = rel_err(fd, gk[elems])
    assert err.max() <= FD_TOL, err.max()


def test_autograd_function_harness():
    import torch
    rng = np.random.Generator(np.random.PCG64(7))
    Th = mesh.square(12)
    Vh = FESpace(Th, "P1")
    P = adjoint.DiffusionProblem(Vh, eps=1e-14)
    kappa = torch.tensor(np.exp(0.2 * rng.standard_normal(Th.nt)), dtype=torch.float64, requires_grad=True)
    f = torch.tensor(1.0 + 0.1 * rng.standard_normal(Th.nt), dtype=torch.float64, requires_grad=True)
    u_obs = torch.tensor(0.01 * rng.standard_normal(Vh.ndof), dtype=torch.float64)
    L = adjoint.DiffusionLoss.apply(kappa, f, P, u_obs)
    L.backward()
    L2, gk, gf, _, _ = P.value_and_grad(kappa.detach().numpy(), f.detach().numpy(), u_obs.numpy())
    assert abs(float(L) - L2) <= 1e-14 * abs(L2)
    assert np.allclose(kappa.grad.numpy(), gk, rtol=1e-13, atol=0)
    assert np.allclose(f.grad.numpy(), gf, rtol=1e-13, atol=0)


def test_heat_forward_against_freefem():
    d, sc = load("heat_p1_n6")
    Th = mesh.square(6)
    Vh = FESpace(Th, "P1")
    H = adjoint.HeatProblem(Vh, dt=1e-2, nsteps=10, checkpoint=5)
    uN, _ = H.forward(d["in_kappa"], np.ones(Th.nt))
    assert np.linalg.norm(uN - d["g_uT"]) <= 1e-10 * np.linalg.norm(d["g_uT"])


def heat_fd(H, kappa, f, u_obs, elems, step=1e-6):
    """Central FD of the final-time loss, differences formed without cancellation:
    A+ du^n = (M/dt) du^{n-1} - 2h (dA/dkappa_k) u-^n, du^0 = 0."""
    P = adjoint.DiffusionProblem.__new__(adjoint.DiffusionProblem)
    P.Vh = H.Vh
    P._wcl = H.Vh.on(H.on).astype(bool)
    out = []
    for e in elems:
        h = step * kappa[e]
        km = kappa.copy(); km[e] -= h
        kp = kappa.copy(); kp[e] += h
        H.assemble(km, f)
        um = [np.zeros(H.Vh.ndof)]
        for n in range(H.nsteps):
            um.append(H.step(um[-1]))
        H.assemble(kp, f)
        du = np.zeros(H.Vh.ndof)
        for n in range(1, H.nsteps + 1):
            v, Ku = adjoint.DiffusionProblem.element_operator(P, e, um[n])
            rhs = H.mdt.mult(du)
            rhs[v] += -2.0 * h * Ku
            du = H.A.solve(rhs)
        rm = um[-1] - u_obs
        dL = float(du @ H.mass.mult(rm)) + 0.5 * float(du @ H.mass.mult(du))
        out.append(dL / (2 * h))
    return np.array(out)


def test_heat_adjoint_checkpointing_and_fd():
    rng = np.random.Generator(np.random.PCG64(99))
    Th = mesh.square(16)
    Vh = FESpace(Th, "P1")
    nsteps = 40
    H = adjoint.HeatProblem(Vh, dt=1e-3, nsteps=nsteps, checkpoint=10)
    kappa = np.exp(0.4 * rng.standard_normal(Th.nt))
    f = np.ones(Th.nt)
    uN, _ = H.forward(np.exp(0.3 * rng.standard_normal(Th.nt)), f)
    u_obs = uN + 0.01 * np.sqrt(np.mean(uN ** 2)) * rng.standard_normal(Vh.ndof)
    L, gk, gf = H.value_and_grad(kappa, f, u_obs)
    # solves: forward N, recompute N - N/c - (c - 1) (checkpointed states and the last
    # segment, kept by the forward pass, are not recomputed), adjoint N
    assert H.forward_solves == nsteps
    assert H.solves == nsteps + (nsteps - nsteps // 10 - 9) + nsteps
    H1 = adjoint.HeatProblem(Vh, dt=1e-3, nsteps=nsteps, checkpoint=1)
    L1, gk1, gf1 = H1.value_and_grad(kappa, f, u_obs)
    assert abs(L - L1) <= 1e-13 * abs(L1)
    assert np.linalg.norm(gk - gk1) <= 1e-11 * np.linalg.norm(gk1)
    assert np.linalg.norm(gf - gf1) <= 1e-11 * np.linalg.norm(gf1)
    elems = rng.choice(Th.nt, size=8, replace=False)
    fd = heat_fd(H, kappa, f, u_obs, elems)
    err = rel_err(fd, gk[elems])
    assert err.max() <= FD_TOL, err.max()
