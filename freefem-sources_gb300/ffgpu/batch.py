"""Batched independent problems: many small P1 diffusion problems in one persistent launch.

Each problem is the FreeFEM script
    mesh Th = <jittered square(N,N)>; fespace Vh(Th,P1);
    varf a(u,v) = int2d(Th)(kappa*grad(u)'*grad(v)) + int2d(Th)(f*v) + on(1,2,3,4,u=0);
    matrix A = a(Vh,Vh,solver=CG,eps=...); real[int] b = a(0,Vh); u[] = A^-1*b;
solved with FP32 inner PCG and FP64 refinement; the batch is assembled in one pass and solved
by one graph-captured persistent kernel (ffgpu_batch_* in include/ffgpu.h).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import api
from ._lib import IRParams, SolverStats, check, lib
from .mesh import Mesh


def batch_arrays(meshes: list[Mesh], on=(1, 2, 3, 4)):
    """The batch as the C ABI takes it: (nv, nt, coords, elems, onbc) -- vertex and element
    counts per problem, the problems' coordinates and (local) elements back to back, and the
    P1 on(labels) mask (the vertices of the boundary edges carrying one of the labels)."""
    nv = np.array([m.nv for m in meshes], np.int32)
    nt = np.array([m.nt for m in meshes], np.int32)
    voff = np.concatenate([[0], np.cumsum(nv)]).astype(np.int64)
    coords = np.ascontiguousarray(np.concatenate([m.coords for m in meshes]), np.float64)
    elems = np.ascontiguousarray(np.concatenate([m.elems for m in meshes]), np.int32)
    be = np.concatenate([m.belems.astype(np.int64) + voff[i] for i, m in enumerate(meshes)])
    bl = np.concatenate([m.blabel for m in meshes])
    onbc = np.zeros(int(voff[-1]), np.uint8)
    onbc[be[np.isin(bl, np.asarray(on))].ravel()] = 1
    return nv, nt, coords, elems, onbc


class Batch:
    def __init__(self, meshes: list[Mesh] | None = None, on=(1, 2, 3, 4), device=0, arrays=None):
        """A batch of independent P1 problems, from a list of meshes or from the arrays of
        batch_arrays (host or device)."""
        nv, nt, coords, elems, onbc = arrays if arrays is not None else batch_arrays(meshes, on)
        self.nv = np.asarray(nv, np.int32)
        self.nt = np.asarray(nt, np.int32)
        self.voff = np.concatenate([[0], np.cumsum(self.nv)]).astype(np.int64)
        self.toff = np.concatenate([[0], np.cumsum(self.nt)]).astype(np.int64)
        self.onbc = onbc
        h = C.c_void_p()
        check(lib().ffgpu_batch_create(api.context(device), self.nv.size, api._ptr(self.nv), api._ptr(self.nt),
                                       api._ptr(coords), api._ptr(elems), C.byref(h)))
        self.h = h
        self.stats = None
        self.iterations = None

    def close(self):
        if getattr(self, "h", None):
            lib().ffgpu_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def ndof(self) -> int:
        return int(self.voff[-1])

    def assemble(self, kappa, f=1.0, tgv=1e30):
        """kappa: list of P0 arrays (one per problem) or one concatenated array."""
        if hasattr(kappa, "data_ptr"):
            k = kappa
        else:
            k = np.ascontiguousarray(np.concatenate(kappa) if isinstance(kappa, (list, tuple)) else kappa,
                                     np.float64)
        self._kappa = k
        check(lib().ffgpu_batch_assemble(self.h, api._ptr(k), float(f), api._ptr(self.onbc), float(tgv)))

    def rhs(self):
        b = np.empty(self.ndof)
        check(lib().ffgpu_batch_rhs(self.h, api._ptr(b)))
        return b

    def solve(self, eps=1e-8, eps_inner=1e-4, itmax_inner=0, max_outer=30, out=None):
        if out is None:
            out = api._touched_zeros(self.ndof)
        p = IRParams()
        p.eps = eps
        p.eps_inner = eps_inner
        p.itmax_inner = itmax_inner
        p.max_outer = max_outer
        p.tgv = 1e30
        p.unroll = 1
        it = np.zeros(self.nv.size, np.int32)
        st = SolverStats()
        code = lib().ffgpu_batch_solve(self.h, api._ptr(out), C.byref(p), api._ptr(it), C.byref(st))
        self.stats = st
        self.iterations = it
        check(code)
        return out

    def split(self, x):
        return [x[self.voff[p]:self.voff[p + 1]] for p in range(self.nv.size)]

    def tuned(self):
        nt, lanes, ms = C.c_int(), C.c_int(), C.c_float()
        check(lib().ffgpu_batch_info(self.h, C.byref(nt), C.byref(lanes), C.byref(ms)))
        return nt.value, lanes.value, ms.value


def c5_meshes(nprob=1024, nmin=16, nmax=128, jitter=0.2, seed=0):
    """The batched benchmark family: square(N,N) with N ~ U{nmin..nmax}, interior vertices
    jittered by U(-jitter h, jitter h)^2, and ln kappa ~ N(0,1) per triangle, all seeded."""
    from .mesh import jittered_square
    rng = np.random.Generator(np.random.PCG64(seed))
    Ns = rng.integers(nmin, nmax + 1, size=nprob)
    meshes = [jittered_square(int(n), jitter, rng) for n in Ns]
    kappas = [np.exp(rng.standard_normal(m.nt)) for m in meshes]
    return meshes, kappas, Ns
