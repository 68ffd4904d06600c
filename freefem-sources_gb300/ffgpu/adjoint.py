"""Adjoint gradients for -div(kappa grad u) = f (P1, P0 kappa and f) and its implicit-Euler
heat variant, on the device path.

Loss: L = 1/2 (u - u_obs)' M (u - u_obs), M the P1 mass matrix (varf int(u*v)).
Adjoint: A' lambda = M (u - u_obs) by the transpose CG (FreeFEM's A'^-1, lgmat.cpp:3219), then
dL/dkappa_e and dL/df_e from the per-element sensitivity kernel (ffgpu_diffusion_sensitivity).

Heat: (M/dt + K(kappa)) u^n = (M/dt) u^{n-1} + F, u^0 = 0, loss on u^N.  The backward pass
recomputes the states from checkpoints kept every `checkpoint` steps, so memory holds
N/checkpoint + checkpoint vectors instead of N.

``DiffusionLoss`` wraps the adjoint in a torch.autograd.Function for gradient checks.
"""
from __future__ import annotations

import ctypes as C

import math

import numpy as np

from . import api
from ._lib import check, lib
from .fespace import FESpace


def _np(a):
    if hasattr(a, "detach"):
        return a.detach().cpu().numpy().astype(np.float64)
    return np.asarray(a, np.float64)


def _on_device(a):
    return hasattr(a, "data_ptr") and getattr(a, "is_cuda", False)


def _zeros(n, like):
    """Zero vector of length n on the side (host numpy / CUDA torch) of `like`."""
    if _on_device(like):
        import torch
        return torch.zeros(n, dtype=torch.float64, device=like.device)
    return np.zeros(n)


def _copy(a):
    return a.clone() if _on_device(a) else np.array(a, copy=True)


def sensitivity(A: api.Matrix, u, lam, c_stiff=1.0):
    """(dL/dkappa_e, dL/df_e) of every element, given the state u and the adjoint lambda.
    Host arrays give numpy results; CUDA tensors give CUDA tensors (no host copy)."""
    nt = A.space.Vh.Th.nt
    if _on_device(u):
        import torch
        gk = torch.empty(nt, dtype=torch.float64, device=u.device)
        gf = torch.empty(nt, dtype=torch.float64, device=u.device)
        check(lib().ffgpu_diffusion_sensitivity(A.h, api._ptr(u.contiguous()), api._ptr(lam.contiguous()),
                                                float(c_stiff), api._ptr(gk), api._ptr(gf)))
        return gk, gf
    gk = np.empty(nt)
    gf = np.empty(nt)
    uu = np.ascontiguousarray(u, np.float64)
    ll = np.ascontiguousarray(lam, np.float64)
    check(lib().ffgpu_diffusion_sensitivity(A.h, api._ptr(uu), api._ptr(ll), float(c_stiff),
                                            api._ptr(gk), api._ptr(gf)))
    return gk, gf


class DiffusionProblem:
    """P1 diffusion with Dirichlet data on `on` labels; kappa and f are P0 arrays."""

    def __init__(self, Vh: FESpace, on=(1, 2, 3, 4), eps=1e-14, tgv=1e30, device=0):
        self.Vh = Vh
        self.on = tuple(on)
        self.eps = eps
        self.tgv = tgv
        self.space = api.DeviceSpace(Vh, device)
        self.mass = api.matrix(api.varf_diffusion(c_stiff=0.0, c_mass=1.0), self.space)
        self.A = None

    def assemble(self, kappa, f):
        """A(kappa) and b(f) on the device; CUDA tensors for kappa (and f) keep b on the device."""
        if _on_device(kappa):
            a = api.varf_diffusion(kappa=kappa.contiguous(), f=f if np.isscalar(f) else f.contiguous(),
                                   on=self.on, tgv=self.tgv)
            b = _zeros(self.Vh.ndof, kappa)
        else:
            a = api.varf_diffusion(kappa=_np(kappa), f=_np(f), on=self.on, tgv=self.tgv)
            b = np.empty(self.Vh.ndof)
        if self.A is None:
            self.A = api.matrix(a, self.space, eps=self.eps, rhs_out=b)
        else:
            self.A.reassemble(a, rhs_out=b)
        return b

    def solve(self, kappa, f):
        b = self.assemble(kappa, f)
        return self.A.solve(b)

    def loss(self, u, u_obs):
        r = u - u_obs
        return 0.5 * float(r @ self.mass.mult(r))

    def value_and_grad(self, kappa, f, u_obs):
        """L, dL/dkappa, dL/df, u, lambda: one forward solve, one transpose solve, one
        sensitivity pass (all on the device when kappa and u_obs are CUDA tensors)."""
        u = self.solve(kappa, f)
        r = u - u_obs
        Mr = self.mass.mult(r)
        L = 0.5 * float(r @ Mr)
        lam = self.A.solve(Mr, trans=True)
        gk, gf = sensitivity(self.A, u, lam)
        return L, gk, gf, u, lam

    def element_operator(self, e, u):
        """(dA/dkappa_e) u restricted to element e: (local DOFs, values), tgv diagonal dropped."""
        Th = self.Vh.Th
        v = Th.elems[e].astype(np.int64)
        X = Th.coords[v]
        if Th.dim == 2:
            area = 0.5 * ((X[1, 0] - X[0, 0]) * (X[2, 1] - X[0, 1]) - (X[1, 1] - X[0, 1]) * (X[2, 0] - X[0, 0]))
            G = np.empty((3, 2))
            for i in range(3):
                p1, p2 = X[(i + 1) % 3], X[(i + 2) % 3]
                G[i] = [-(p2[1] - p1[1]) / (2 * area), (p2[0] - p1[0]) / (2 * area)]
            meas = area
        else:
            V = X[1:] - X[0]
            meas = np.linalg.det(V) / 6.0
            Gi = np.linalg.inv(V).T
            G = np.vstack([-Gi.sum(axis=0), Gi])
        K = meas * (G @ G.T)
        on = self.A_wcl() if hasattr(self, "_wcl") else None
        Ku = K @ u[v]
        if on is not None:
            for i in range(len(v)):
                if on[v[i]]:
                    Ku[i] -= K[i, i] * u[v[i]]
        return v, Ku

    def A_wcl(self):
        return self._wcl

    def fd_gradient(self, kappa, f, u_obs, elements, step=1e-6):
        """Central finite differences (L(kappa + h e_k) - L(kappa - h e_k)) / 2h, h = step*kappa_k.

        The difference of the two losses is formed without cancellation: with A+- = A(kappa +- h e_k),
        u- = A-^-1 b and du = u+ - u- solving A+ du = -(A+ - A-) u- = -2h (dA/dkappa_k) u- (exact:
        A is affine in kappa_k), L+ - L- = du' M r- + 1/2 du' M du with r- = u- - u_obs."""
        kappa = _np(kappa).copy()
        self._wcl = self.Vh.on(self.on).astype(bool)
        out = np.empty(len(elements))
        for t, e in enumerate(elements):
            h = step * kappa[e]
            km = kappa.copy(); km[e] -= h
            kp = kappa.copy(); kp[e] += h
            um = self.solve(km, f)
            rm = um - u_obs
            v, Ku = self.element_operator(e, um)
            rhs = np.zeros(self.Vh.ndof)
            rhs[v] = -2.0 * h * Ku
            bp = self.assemble(kp, f)
            del bp
            du = self.A.solve(rhs)
            Mdu = self.mass.mult(du)
            dL = float(du @ self.mass.mult(rm)) + 0.5 * float(du @ Mdu)
            out[t] = dL / (2.0 * h)
        return out


class HeatProblem:
    """Implicit Euler for u_t - div(kappa grad u) = f, u(0) = 0, Dirichlet on `on`, loss on u^N."""

    def __init__(self, Vh: FESpace, dt, nsteps, on=(1, 2, 3, 4), checkpoint=20, eps=1e-14,
                 tgv=1e30, device=0):
        self.Vh = Vh
        self.dt = dt
        self.nsteps = nsteps
        self.on = tuple(on)
        self.checkpoint = checkpoint
        self.eps = eps
        self.tgv = tgv
        self.space = api.DeviceSpace(Vh, device)
        self.mass = api.matrix(api.varf_diffusion(c_stiff=0.0, c_mass=1.0), self.space)
        self.mdt = api.matrix(api.varf_diffusion(c_stiff=0.0, c_mass=1.0 / dt), self.space)
        self.A = None
        self.solves = 0
        self.iterations_state = 0      # CG iterations of the state solves (forward and recomputed)
        self.iterations_adjoint = 0    # CG iterations of the transpose solves

    def assemble(self, kappa, f):
        if _on_device(kappa):
            a = api.varf_diffusion(kappa=kappa.contiguous(), f=f if np.isscalar(f) else f.contiguous(),
                                   c_mass=1.0 / self.dt, on=self.on, tgv=self.tgv)
            F = _zeros(self.Vh.ndof, kappa)
        else:
            a = api.varf_diffusion(kappa=_np(kappa), f=_np(f), c_mass=1.0 / self.dt, on=self.on, tgv=self.tgv)
            F = np.empty(self.Vh.ndof)
        if self.A is None:
            self.A = api.matrix(a, self.space, eps=self.eps, rhs_out=F)
        else:
            self.A.reassemble(a, rhs_out=F)
        self.F = F
        return F

    def step(self, u_prev, x0=None, eps=None):
        """u^n from u^{n-1}: FreeFEM's u[] = A^-1*b with u[] = u^{n-1} as the initial guess, or
        from x0 with the stopping tolerance eps (eps < 0: absolute, FreeFEM's convention)."""
        self.solves += 1
        u = self.A.solve(self.mdt.mult(u_prev) + self.F, x0=u_prev if x0 is None else x0, eps=eps)
        self.iterations_state += self.A.stats.iterations
        self.last_gcg = self.A.stats.gcg
        return u

    def forward(self, kappa, f, keep_checkpoints=True):
        """u^N and the checkpoints: every `checkpoint`-th state, plus the states of the last
        segment, which the backward pass needs first and would otherwise recompute.  Also
        keeps the final (g, Cg) of every step's solve (the accuracy a recomputation matches)."""
        F = self.assemble(kappa, f)
        u = _zeros(self.Vh.ndof, F)
        ck = {0: _copy(u)}
        self.gcg = [0.0] * (self.nsteps + 1)
        N, c = self.nsteps, self.checkpoint
        last0 = ((N - 1) // c) * c
        for n in range(1, N + 1):
            u = self.step(u)
            self.gcg[n] = self.last_gcg
            if keep_checkpoints and (n % c == 0 or n > last0):
                ck[n] = _copy(u)
        return u, ck

    def _jacobi(self, like):
        """C = 1/A_ii of the current matrix (1 where |A_ii|^2 < 1e-60), the CG's Jacobi
        preconditioner, on the side (host / device) of `like`."""
        rp, cl, v = self.A.csr()
        n = rp.size - 1
        row = np.repeat(np.arange(n), np.diff(rp))
        on = row == cl
        d = np.zeros(n)
        d[row[on]] = v[on]
        cj = np.where(d * d < 1e-60, 1.0, 1.0 / np.where(d == 0.0, 1.0, d))
        if _on_device(like):
            import torch
            return torch.from_numpy(cj).to(like.device)
        return cj

    def recompute(self, n, u_prev, u_prev2):
        """u^n again, from u^{n-1} and (when there is one) u^{n-2}: the same system, started
        from the linear extrapolation 2 u^{n-1} - u^{n-2} and stopped at the residual the
        forward solve of step n reached, (g, Cg) <= its final value (absolute tolerance).  The
        state agrees with the forward's to the solver's accuracy, in fewer iterations."""
        g = self.gcg[n]
        if u_prev2 is None or not g > 0.0:
            return self.step(u_prev)
        return self.step(u_prev, x0=2.0 * u_prev - u_prev2, eps=-math.sqrt(g))

    def loss(self, uN, u_obs):
        r = uN - u_obs
        return 0.5 * float(r @ self.mass.mult(r))

    def value_and_grad(self, kappa, f, u_obs):
        """Forward with checkpoints, backward with recomputation of each segment."""
        self.solves = 0
        self.iterations_state = 0
        self.iterations_adjoint = 0
        uN, ck = self.forward(kappa, f)
        forward_solves = self.solves
        r = uN - u_obs
        L = 0.5 * float(r @ self.mass.mult(r))
        nt = self.Vh.Th.nt
        gk = _zeros(nt, uN)
        gf = _zeros(nt, uN)
        rhs_adj = self.mass.mult(r)          # dL/du^N
        lam_next = lam_next2 = None
        cj = self._jacobi(uN)
        N, c = self.nsteps, self.checkpoint
        seg_starts = sorted(k for k in ck if k < N and k % c == 0)
        for s0 in reversed(seg_starts):
            s1 = min(s0 + c, N)
            # recompute u^{s0+1..s1} from the checkpoint u^{s0}
            states = {s0: ck[s0]}
            u, up = ck[s0], None
            for n in range(s0 + 1, s1 + 1):
                un = self.recompute(n, u, up) if n not in ck or n == s0 else ck[n]
                states[n] = un
                u, up = un, u
            for n in range(s1, s0, -1):
                rhs = rhs_adj if n == N else self.mdt.mult(lam_next, trans=True)
                # the adjoint solve starts from the extrapolation of the two later adjoint states
                # and stops where a solve from zero would (FreeFEM's test for x0 = 0:
                # (g, Cg) < eps^2 (b, Cb)), as an absolute tolerance
                x0, eps_adj = lam_next, None
                if lam_next2 is not None:
                    x0 = 2.0 * lam_next - lam_next2
                    bcb = float((rhs * cj * rhs).sum())
                    eps_adj = -self.eps * math.sqrt(bcb) if bcb > 0.0 else None
                lam = self.A.solve(rhs, trans=True, x0=x0, eps=eps_adj)
                self.solves += 1
                self.iterations_adjoint += self.A.stats.iterations
                g1, g2 = sensitivity(self.A, states[n], lam)
                gk += g1
                gf += g2
                lam_next, lam_next2 = lam, lam_next
        self.forward_solves = forward_solves
        return L, gk, gf


try:
    import torch

    class DiffusionLoss(torch.autograd.Function):
        """L(kappa, f) with the adjoint gradient, for gradient-check harnesses only."""

        @staticmethod
        def forward(ctx, kappa, f, problem, u_obs):
            L, gk, gf, u, lam = problem.value_and_grad(kappa, f, _np(u_obs))
            ctx.save_for_backward(torch.from_numpy(gk), torch.from_numpy(gf))
            return torch.tensor(L, dtype=torch.float64)

        @staticmethod
        def backward(ctx, gout):
            gk, gf = ctx.saved_tensors
            return gout * gk, gout * gf, None, None
except ImportError:  # pragma: no cover
    DiffusionLoss = None
