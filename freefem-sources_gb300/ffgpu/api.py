"""Host-side mirror of FreeFEM's interface for the assemble-and-solve path.

The names follow the FreeFEM script being replaced::

    mesh Th = square(256,256);             Th = square(256, 256)
    fespace Vh(Th,P1);                     Vh = fespace(Th, "P1")
    varf a(u,v) = int2d(Th)(grad u.grad v) a  = varf_diffusion(f=1.0, on=(1,2,3,4))
               + int2d(Th)(1*v) + on(1,2,3,4,u=0);
    matrix A = a(Vh,Vh,solver=CG,eps=1e-10);   A = matrix(a, Vh, solver="CG", eps=1e-10)
    real[int] b = a(0,Vh);                  b = rhs(a, Vh)
    u[] = A^-1*b;                           u = A.solve(b)          (A'^-1*b: trans=True)

Arrays are numpy (host) or CUDA torch tensors (device, passed by pointer).  Every call goes
through the C ABI of libffgpu.so; there is no CPU path.  Errors raise ``FFGPUError`` (FreeFEM
raises ExecError / ffassert at the same points, e.g. CG non-convergence,
VirtualSolverCG.hpp:188-189).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib, quadrature
from ._lib import BC, BTerm, SolverParams, SolverStats, Varf, check, lib
from .expr import Expr, c_expr, const
from .fespace import FESpace
from .mesh import Mesh

_ctx = {}


def _touched_zeros(shape):
    """A zero host array whose pages are already mapped: np.zeros maps large arrays lazily, and
    the device-to-host copy of the result into unmapped pages pays a fault per page."""
    a = np.empty(shape)
    a.fill(0.0)
    return a


def _ptr(a):
    """Raw pointer of a numpy array or a torch tensor (host or CUDA), None for None."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return a.ctypes.data_as(C.c_void_p)
    raise TypeError(f"unsupported array type {type(a)}")


def context(device: int = 0):
    """The library context of a GPU (created on first use)."""
    if device not in _ctx:
        h = C.c_void_p()
        check(lib().ffgpu_ctx_create(device, C.byref(h)))
        _ctx[device] = h
    return _ctx[device]


def kernel_launches(device: int = 0) -> int:
    return int(lib().ffgpu_ctx_kernel_launches(context(device)))


def stream_handle(device: int = 0) -> int:
    """The CUDA stream (cudaStream_t as int) all library calls of this context run on."""
    return int(lib().ffgpu_ctx_stream(context(device)) or 0)


def fespace(Th: Mesh, kind: str, dof=None) -> FESpace:
    return FESpace(Th, kind, dof)


class DeviceSpace:
    """Mesh + FE space resident on the GPU (ffgpu_space_create)."""

    def __init__(self, Vh: FESpace, device: int = 0, coords=None, elems=None, dof=None, boundary=True,
                 belems=None, blabel=None):
        self.Vh = Vh
        Th = Vh.Th
        self.device = device
        self._keep = []
        X = coords if coords is not None else np.ascontiguousarray(Th.coords, np.float64)
        E = elems if elems is not None else np.ascontiguousarray(Th.elems, np.int32)
        # P1 DOFs are the vertices (FreeFEM's P1 numbering): no DOF table crosses to the device
        D = dof if dof is not None else (None if Vh.kind == "P1" else np.ascontiguousarray(Vh.dof, np.int32))
        self._keep += [X, E, D]
        h = C.c_void_p()
        check(lib().ffgpu_space_create(context(device), Th.dim, Th.nv, _ptr(X), Th.nt, _ptr(E),
                                       Vh.fe, Vh.ndofK, _ptr(D), Vh.ndof, C.byref(h)))
        self.h = h
        self.has_boundary = False
        if boundary and Th.nbe > 0:
            be = belems if belems is not None else np.ascontiguousarray(Th.belems, np.int32)
            bl = blabel if blabel is not None else np.ascontiguousarray(Th.blabel, np.int32)
            self._keep += [be, bl]
            check(lib().ffgpu_space_set_boundary(h, Th.nbe, _ptr(be), _ptr(bl)))
            self.has_boundary = True

    def bc_mask(self, labels, components=None):
        """The on(labels) DOF mask as the device assembly computes it (host uint8 array)."""
        lab = np.ascontiguousarray(np.atleast_1d(labels), np.int32)
        cm = 0 if components is None else sum(1 << c for c in components)
        out = np.empty(self.Vh.ndof, np.uint8)
        check(lib().ffgpu_space_bc_mask(self.h, lab.size, _ptr(lab), cm, _ptr(out)))
        return out

    def close(self):
        if getattr(self, "h", None):
            lib().ffgpu_space_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class BoundaryTerm:
    """int1d(Th, labels)(robin*u*v + g*v) in 2D, int2d(Th, labels)(...) on the boundary faces in
    3D (labels empty: the whole boundary).  robin: scalar or per boundary element (nbe); g:
    scalar, per-component tuple, or per boundary element (nbe[, ncomp]).  For [P2,P2,P2] the
    Robin term is robin*(u1*v1+u2*v2+u3*v3)."""

    labels: tuple = ()
    robin: object = 0.0
    g: object = 0.0


@dataclass
class VarForm:
    """A varf of the supported family (P0 coefficients, constant or P0 sources, boundary terms)."""

    form: int = _lib.FORM_DIFFUSION
    kappa: object = None          # P0 coefficient (nt) or None
    c_stiff: float = 1.0
    c_mass: float = 0.0
    E: float = 1.0
    nu: float = 0.3
    f: object = 1.0               # scalar, per-component tuple, P0 array (nt[, ncomp]), or a
                                  # function of the coordinates, f(x, y[, z]) (a tuple of
                                  # ncomp values for [P2,P2,P2]), taken at the rule's points
    quad: str | None = None       # rule for a function source: qf2pT, qf5pT, tet2, tet5
                                  # (None: FreeFEM's default, qf5pT / tet5)
    on: tuple = ()                # boundary labels of on(..., u=g)
    g: object = None              # Dirichlet values per DOF (None = 0)
    components: tuple | None = None
    tgv: float = 1e30
    bterms: tuple = ()            # BoundaryTerm, in varf order
    terms: tuple = ()             # general volume terms (iop, jop, coef) of a scalar space:
                                  # int(coef*op_i(v)*op_j(u)), op "id"/"dx"/"dy"/"dz" (or 0..3),
                                  # coef a number or an ffgpu.expr expression
    _keep: list = field(default_factory=list)

    def c_varf(self, Vh: FESpace) -> Varf:
        v = Varf()
        v.form = self.form
        v.c_stiff = self.c_stiff
        v.c_mass = 0.0 if (callable(self.c_mass) or isinstance(self.c_mass, Expr)) else self.c_mass
        # values at quadrature points (one rule for the varf), set by the helpers below
        v.nqp = 0
        v.qp_lambda = v.qp_weight = v.f_qp = v.mass_qp = v.stiff_qp = None
        v.E = self.E if np.ndim(self.E) == 0 else 1.0
        v.nu = self.nu if np.ndim(self.nu) == 0 else 0.3
        v.lame = None
        if self.form == _lib.FORM_ELASTICITY and (np.ndim(self.E) > 0 or np.ndim(self.nu) > 0):
            # several materials: lambda, mu per element, by the same formulas as for constants
            nt = Vh.Th.nt
            Ea = np.broadcast_to(np.asarray(self.E, np.float64), (nt,))
            na = np.broadcast_to(np.asarray(self.nu, np.float64), (nt,))
            lame = np.ascontiguousarray(np.stack([Ea * na / ((1 + na) * (1 - 2 * na)), Ea / (2 * (1 + na))], axis=1))
            self._keep.append(lame)
            v.lame = _ptr(lame).value
        v.kappa = None
        v.f_expr = None
        v.nterms = 0
        v.terms = None
        self._expressions(v, Vh)
        if isinstance(self.kappa, Expr):
            pass
        elif callable(self.kappa):
            self._stiff_at_points(v, Vh)
        elif self.kappa is not None and np.ndim(self.kappa) == 0 and not hasattr(self.kappa, "data_ptr"):
            v.c_stiff = float(v.c_stiff) * float(self.kappa)   # a constant kappa: part of c_stiff
        elif self.kappa is not None:
            k = self.kappa if hasattr(self.kappa, "data_ptr") else np.ascontiguousarray(self.kappa, np.float64)
            if int(np.prod(np.shape(k))) != Vh.Th.nt:
                raise ValueError(f"kappa: one value per element expected ({Vh.Th.nt}), got shape {np.shape(k)}")
            self._keep.append(k)
            v.kappa = _ptr(k).value
        v.f = None
        if callable(self.c_mass) and not isinstance(self.c_mass, Expr):
            self._mass_at_points(v, Vh)
        if _is_expr_source(self.f):
            pass
        elif callable(self.f):
            self._source_at_points(v, Vh)
        elif np.isscalar(self.f):
            v.f_const[0] = float(self.f)
        elif hasattr(self.f, "data_ptr"):
            v.f = _ptr(self.f).value
            self._keep.append(self.f)
        else:
            fa = np.asarray(self.f, np.float64)
            nc = 3 if Vh.kind == "P2vec" else 1
            if fa.ndim == 1 and fa.size == nc and fa.size != Vh.Th.nt:
                for c in range(nc):
                    v.f_const[c] = fa[c]
            else:
                fa = np.ascontiguousarray(fa.reshape(Vh.Th.nt, nc))
                self._keep.append(fa)
                v.f = _ptr(fa).value
        v.nbterms = 0
        v.bterms = None
        if self.bterms:
            nc = 3 if Vh.kind == "P2vec" else 1
            nbe = Vh.Th.nbe
            arr = (BTerm * len(self.bterms))()
            for t, bt in enumerate(self.bterms):
                T = arr[t]
                lab = np.ascontiguousarray(np.atleast_1d(np.asarray(bt.labels, np.int32)), np.int32)
                self._keep.append(lab)
                T.nlabels = lab.size
                T.labels = _ptr(lab).value if lab.size else None
                T.robin = None
                T.robin_const = 0.0
                if np.isscalar(bt.robin):
                    T.robin_const = float(bt.robin)
                else:
                    r = bt.robin if hasattr(bt.robin, "data_ptr") else np.ascontiguousarray(bt.robin, np.float64)
                    if r.size != nbe:
                        raise ValueError("BoundaryTerm.robin: one value per boundary element expected")
                    self._keep.append(r)
                    T.robin = _ptr(r).value
                T.g = None
                if np.isscalar(bt.g):
                    T.g_const[0] = float(bt.g)
                elif hasattr(bt.g, "data_ptr"):
                    self._keep.append(bt.g)
                    T.g = _ptr(bt.g).value
                else:
                    ga = np.asarray(bt.g, np.float64)
                    if ga.ndim == 1 and ga.size == nc and ga.size != nbe:
                        for c in range(nc):
                            T.g_const[c] = ga[c]
                    else:
                        ga = np.ascontiguousarray(ga.reshape(nbe, nc))
                        self._keep.append(ga)
                        T.g = _ptr(ga).value
            self._keep.append(arr)
            v.nbterms = len(self.bterms)
            v.bterms = C.cast(arr, C.c_void_p).value
        return v

    def _expressions(self, v: Varf, Vh: FESpace) -> None:
        """Coefficients and sources given as ffgpu.expr expressions: evaluated on the device at
        the points of the varf's rule.  kappa -> the terms (dx,dx)+(dy,dy)[+(dz,dz)] with
        coefficient c_stiff*kappa; c_mass -> the term (id,id); f -> f_expr; plus self.terms."""
        dim = Vh.Th.dim
        ops = {"id": 0, "dx": 1, "dy": 2, "dz": 3}
        terms = []
        if isinstance(self.kappa, Expr):
            terms += [(d + 1, d + 1, self.c_stiff, self.kappa) for d in range(dim)]
            v.c_stiff = 0.0          # the closed-form stiffness then contributes nothing
        if isinstance(self.c_mass, Expr):
            terms.append((0, 0, 1.0, self.c_mass))
            v.c_mass = 0.0
        for t in self.terms:
            iop, jop, coef = t
            iop = ops.get(iop, iop)
            jop = ops.get(jop, jop)
            if isinstance(coef, Expr):
                terms.append((int(iop), int(jop), 1.0, coef))
            else:
                terms.append((int(iop), int(jop), float(coef), None))
        fexpr = _is_expr_source(self.f)
        if not terms and not fexpr:
            return
        if self.form != _lib.FORM_DIFFUSION and terms:
            raise ValueError("expression coefficients and general terms need the scalar diffusion form")
        lam, w = quadrature.rule(self.quad, dim)
        self._keep += [lam, w]
        v.nqp = lam.shape[0]
        v.qp_lambda = _ptr(lam).value
        v.qp_weight = _ptr(w).value
        if terms:
            arr = (_lib.TermC * len(terms))()
            for k, (iop, jop, c, e) in enumerate(terms):
                arr[k].iop, arr[k].jop, arr[k].c = iop, jop, c
                if e is None:
                    arr[k].expr = None
                else:
                    ex = c_expr(e, self._keep)
                    self._keep.append(ex)
                    arr[k].expr = C.addressof(ex)
            self._keep.append(arr)
            v.nterms = len(terms)
            v.terms = C.cast(arr, C.c_void_p).value
        if fexpr:
            nc = 3 if Vh.kind == "P2vec" else 1
            comps = list(self.f) if isinstance(self.f, (tuple, list)) else [self.f]
            if len(comps) != nc:
                raise ValueError(f"the source needs {nc} component(s)")
            arr = (_lib.ExprC * nc)()
            for c, e in enumerate(comps):
                arr[c] = c_expr(e if isinstance(e, Expr) else const(e), self._keep)
            self._keep.append(arr)
            v.f_expr = C.cast(arr, C.c_void_p).value

    def _rule_points(self, v: Varf, Vh: FESpace):
        """The rule (set once in v) and the physical points of every element."""
        Th = Vh.Th
        if not hasattr(Th, "coords"):
            raise ValueError("a coefficient or source function needs the mesh coordinates on the host")
        lam, w = quadrature.rule(self.quad, Th.dim)
        self._keep += [lam, w]
        v.nqp = lam.shape[0]
        v.qp_lambda = _ptr(lam).value
        v.qp_weight = _ptr(w).value
        return lam, quadrature.points(Th.coords, Th.elems, lam)

    def _mass_at_points(self, v: Varf, Vh: FESpace) -> None:
        """c(x, y[, z]) of the c*u*v term at the quadrature points, as Element_Op takes it."""
        if self.form != _lib.FORM_DIFFUSION:
            raise ValueError("a mass coefficient function needs the diffusion form")
        lam, xq = self._rule_points(v, Vh)
        val = self.c_mass(*[xq[..., d] for d in range(Vh.Th.dim)])
        cq = np.ascontiguousarray(np.broadcast_to(np.asarray(val, np.float64), xq.shape[:2]))
        self._keep.append(cq)
        v.mass_qp = _ptr(cq).value

    def _stiff_at_points(self, v: Varf, Vh: FESpace) -> None:
        """c_stiff * kappa(x, y[, z]) of the grad u . grad v term at the quadrature points."""
        if self.form != _lib.FORM_DIFFUSION:
            raise ValueError("a stiffness coefficient function needs the diffusion form")
        lam, xq = self._rule_points(v, Vh)
        val = self.kappa(*[xq[..., d] for d in range(Vh.Th.dim)])
        kq = np.ascontiguousarray(np.broadcast_to(np.asarray(val, np.float64) * self.c_stiff, xq.shape[:2]))
        self._keep.append(kq)
        v.stiff_qp = _ptr(kq).value

    def _source_at_points(self, v: Varf, Vh: FESpace) -> None:
        """f(x, y[, z]) at the quadrature points of every element, as Element_rhs takes it."""
        Th = Vh.Th
        lam, xq = self._rule_points(v, Vh)
        val = self.f(*[xq[..., d] for d in range(Th.dim)])
        nc = 3 if Vh.kind == "P2vec" else 1
        shape = (Th.nt, lam.shape[0])
        if nc == 1:
            fq = np.broadcast_to(np.asarray(val, np.float64), shape)[..., None]
        else:
            if len(val) != 3:
                raise ValueError("[P2,P2,P2]: the source function returns three components")
            fq = np.stack([np.broadcast_to(np.asarray(c, np.float64), shape) for c in val], axis=-1)
        fq = np.ascontiguousarray(fq)
        self._keep.append(fq)
        v.f_qp = _ptr(fq).value

    def c_bc(self, Vh: FESpace, device_marking: bool = False) -> BC:
        """on(labels): with device_marking the assembly marks the DOFs on the device from the
        space's boundary elements; otherwise the host mask FESpace.on is passed."""
        bc = BC()
        bc.tgv = self.tgv
        bc.onbc = None
        bc.g = None
        bc.nlabels = 0
        bc.labels = None
        bc.comp_mask = 0
        if self.on and device_marking:
            lab = np.ascontiguousarray(self.on, np.int32)
            self._keep.append(lab)
            bc.nlabels = lab.size
            bc.labels = _ptr(lab).value
            bc.comp_mask = 0 if self.components is None else sum(1 << c for c in self.components)
            if self.g is not None:
                g = np.ascontiguousarray(self.g, np.float64)
                self._keep.append(g)
                bc.g = _ptr(g).value
        elif self.on:
            m = Vh.on(self.on, self.components)
            self._keep.append(m)
            bc.onbc = _ptr(m).value
            if self.g is not None:
                g = np.ascontiguousarray(self.g, np.float64)
                self._keep.append(g)
                bc.g = _ptr(g).value
        return bc


def _is_expr_source(f):
    if isinstance(f, Expr):
        return True
    return isinstance(f, (tuple, list)) and any(isinstance(c, Expr) for c in f)


def varf_diffusion(kappa=None, f=1.0, on=(), g=None, c_mass=0.0, c_stiff=1.0, tgv=1e30,
                   bterms=(), quad=None, terms=()) -> VarForm:
    """varf a(u,v) = int(c_stiff*kappa*grad u.grad v + c_mass*u*v) + int(f*v)
    + the boundary terms (BoundaryTerm: robin*u*v + g*v on labelled boundary edges/faces)
    + on(on, u=g).  kappa, c_mass and f may be functions of the coordinates, f(x, y[, z]),
    taken at the points of `quad` on the host, or ffgpu.expr expressions (x, y, z, FE functions
    by their DOF values, their derivatives), evaluated on the device at those points.
    terms: further volume terms (iop, jop, coef) = int(coef*op_i(v)*op_j(u)) with op "id",
    "dx", "dy", "dz" -- anisotropic diffusion, advection, reaction."""
    return VarForm(form=_lib.FORM_DIFFUSION, kappa=kappa, f=f, on=tuple(on), g=g, c_mass=c_mass,
                   c_stiff=c_stiff, tgv=tgv, bterms=tuple(bterms), quad=quad, terms=tuple(terms))


def varf_elasticity(E=1.0, nu=0.3, f=(0.0, 0.0, -1.0), on=(), components=None, tgv=1e30,
                    bterms=(), quad=None) -> VarForm:
    """varf a([u],[v]) = int(lambda div u div v + 2mu eps(u):eps(v)) + int(f.v)
    + the boundary terms (tractions g.v, Robin robin*u.v) + on(on, u=0).  E and nu may be
    arrays per element (several materials); f may be a function f(x, y, z) returning three
    components, taken at the points of `quad`."""
    return VarForm(form=_lib.FORM_ELASTICITY, E=E, nu=nu, f=f, on=tuple(on), components=components,
                   tgv=tgv, bterms=tuple(bterms), quad=quad)


# direct solver names -> ffgpu_direct_method (FFGPU_DIRECT_AUTO / _CHOLESKY / _QR)
DIRECT_METHODS = {"SPARSESOLVER": 0, "UMFPACK": 0, "LU": 0, "CHOLESKY": 1, "CHOLMOD": 1, "QR": 2}


class Matrix:
    """``matrix A = a(Vh,Vh, solver=..., eps=..., ...)`` with a device-resident pattern/values."""

    def __init__(self, h, space: DeviceSpace | None, solver="CG", eps=1e-6, itmax=0,
                 dim_krylov=1000, tgv=1e30, device=0):
        self.h = h
        self.space = space
        self.solver = solver
        self.eps = eps
        self.itmax = itmax
        self.dim_krylov = dim_krylov
        self.tgv = tgv
        self.device = device
        self.stats = None
        n = C.c_int()
        nnz = C.c_int64()
        bs = C.c_int()
        check(lib().ffgpu_matrix_info(h, C.byref(n), C.byref(nnz), C.byref(bs)))
        self.n, self.nnz, self.block_size = n.value, nnz.value, bs.value

    def close(self):
        if getattr(self, "h", None):
            lib().ffgpu_matrix_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self, eps=None, itmax=None, unroll=8, spmv_mode=0, spmv_layout=0) -> SolverParams:
        p = SolverParams()
        p.spmv_mode = spmv_mode
        p.spmv_layout = spmv_layout
        p.eps = self.eps if eps is None else eps
        p.itmax = self.itmax if itmax is None else itmax
        p.dim_krylov = self.dim_krylov
        p.tgv = self.tgv
        p.verb = 0
        p.unroll = unroll
        return p

    def solve(self, b, x0=None, trans=False, solver=None, eps=None, itmax=None, out=None, unroll=8,
              spmv_mode=0, spmv_layout=0):
        """u[] = A^-1*b (A'^-1*b when trans).  x0 is the initial guess (FreeFEM: u[] before).
        spmv_layout: 0 = tuned per shape; a layout code (see ffgpu_solver_params) fixes it."""
        solver = (solver or self.solver).upper()
        dev_in = hasattr(b, "data_ptr")
        if out is None:
            if dev_in:
                import torch
                out = torch.zeros_like(b) if x0 is None else x0.clone()
            else:
                out = _touched_zeros(np.shape(b)) if x0 is None else np.array(x0, np.float64)
        elif x0 is not None:
            out[...] = x0
        bb = b if dev_in else np.ascontiguousarray(b, np.float64)
        nrhs = int(np.prod(np.shape(b))) // self.n
        st = SolverStats()
        if solver in DIRECT_METHODS:
            # direct: the factorisation is kept for later solves of this numeric state; Cholesky
            # (symmetric positive definite), QR (any nonsingular matrix) or the choice between
            # them by symmetry (SPARSESOLVER, FreeFEM's default direct solver name); trans solves
            # A' x = b (a symmetric matrix from its own factors, a nonsymmetric one from a QR of A')
            check(lib().ffgpu_direct_method(self.h, DIRECT_METHODS[solver]))
            code = lib().ffgpu_solve_direct_trans(self.h, _ptr(bb), _ptr(out), nrhs, int(trans), C.byref(st))
            self.stats = st
            check(code)
            return out
        p = self.params(eps, itmax, unroll, spmv_mode, spmv_layout)
        fn = lib().ffgpu_solve_cg if solver == "CG" else lib().ffgpu_solve_gmres
        if solver not in ("CG", "GMRES"):
            raise ValueError(f"solver {solver!r}: the device path provides CG, GMRES and the direct solvers "
                             f"{', '.join(DIRECT_METHODS)}")
        code = fn(self.h, _ptr(bb), _ptr(out), nrhs, int(trans), C.byref(p), C.byref(st))
        self.stats = st
        check(code)
        return out

    def solve_mixed(self, b, x0=None, eps=None, eps_inner=0.0, itmax_inner=0, max_outer=30,
                    out=None, unroll=8, restart_inner=False):
        """u[] = A^-1*b by FP32 inner PCG + FP64 iterative refinement, same stopping rule
        as the FP64 CG on the true residual.  Default: residual replacement keeping the search
        direction, eps_inner the residual drop between replacements (0: 1e-2); with
        restart_inner a fresh inner PCG per refinement step (0: 1e-5)."""
        dev_in = hasattr(b, "data_ptr")
        if out is None:
            if dev_in:
                import torch
                out = torch.zeros_like(b) if x0 is None else x0.clone()
            else:
                out = _touched_zeros(np.shape(b)) if x0 is None else np.array(x0, np.float64)
        bb = b if dev_in else np.ascontiguousarray(b, np.float64)
        p = _lib.IRParams()
        p.eps = self.eps if eps is None else eps
        p.eps_inner = eps_inner
        p.itmax_inner = itmax_inner
        p.max_outer = max_outer
        p.tgv = self.tgv
        p.unroll = unroll
        p.restart_inner = int(bool(restart_inner))
        st = SolverStats()
        code = lib().ffgpu_solve_ir(self.h, _ptr(bb), _ptr(out), C.byref(p), C.byref(st))
        self.stats = st
        check(code)
        return out

    def spmv_layout(self, mode=0):
        """The SpMV layout the tuner chose for mode 0 (FP64 CG), 1 (double-float CG) or 2 (FP32
        inner solve): 'sell32' (chunk ranges) or 'sell32-rot', with '-deep' for the deeper unroll and
        '-batch' / '-batch-deep' for the batched row loop, 'bsr/T' (T lanes per block row) or None."""
        v = int(lib().ffgpu_matrix_spmv_layout(self.h, int(mode)))
        if v <= 0:
            return None
        if 64 <= v < 72:
            loop = ["", "-deep", "-batch", "-batch-deep"][(v - 64) >> 1]
            return ("sell32" if (v - 64) % 2 == 0 else "sell32-rot") + loop
        return f"bsr/{v}"

    def layout_code(self, mode=0):
        """The raw layout code of spmv_layout (the value Matrix.solve(spmv_layout=...) takes)."""
        return int(lib().ffgpu_matrix_spmv_layout(self.h, int(mode)))

    def save(self, path, format="coo"):
        """``ofstream f(path); f << A;``: FreeFEM's text form of the matrix (sorted)."""
        rp, cl, vl = self.csr()
        write_matrix_text(path, rp, cl, vl, format=format)

    def time_spmv(self, mode=0, nrep=20):
        """Mean device time (ms) of nrep back-to-back launches of the solver's SpMV kernel for
        mode 0/1/2 (see spmv_layout), CUDA events on the library stream; solve in that mode first."""
        ms = C.c_float(0)
        check(lib().ffgpu_matrix_time_spmv(self.h, int(mode), int(nrep), C.byref(ms)))
        return float(ms.value)

    def mult(self, x, trans=False, out=None):
        if out is None:
            out = np.empty(self.n) if not hasattr(x, "data_ptr") else x.new_empty(self.n)
        xx = x if hasattr(x, "data_ptr") else np.ascontiguousarray(x, np.float64)
        check(lib().ffgpu_matrix_mult(self.h, _ptr(xx), _ptr(out), int(trans)))
        return out

    def csr(self):
        """(rowptr, col, val) of the matrix in FreeFEM's sorted (row, column) order."""
        rp = np.empty(self.n + 1, np.int32)
        cl = np.empty(self.nnz, np.int32)
        vl = np.empty(self.nnz, np.float64)
        check(lib().ffgpu_matrix_csr(self.h, _ptr(rp), _ptr(cl), _ptr(vl)))
        return rp, cl, vl

    def coo(self):
        """[I,J,C] = A (row-major sorted COO, as FreeFEM's [I,J,C]=A gives)."""
        rp, cl, vl = self.csr()
        return np.repeat(np.arange(self.n, dtype=np.int32), np.diff(rp)), cl, vl

    def reassemble(self, varf: VarForm, rhs_out=None):
        Vh = self.space.Vh
        v = varf.c_varf(Vh)
        bc = varf.c_bc(Vh, device_marking=self.space.has_boundary)
        check(lib().ffgpu_matrix_reassemble(self.h, C.byref(v), C.byref(bc), _ptr(rhs_out)))
        return rhs_out


def matrix(varf: VarForm, Vh, solver="CG", eps=1e-6, itmax=0, dim_krylov=1000, rhs_out=None,
           device=0) -> Matrix:
    """matrix A = a(Vh,Vh, solver=..., eps=...).  Vh: FESpace or DeviceSpace.  If rhs_out is
    given the linear form a(0,Vh) is assembled into it in the same device pass."""
    space = Vh if isinstance(Vh, DeviceSpace) else DeviceSpace(Vh, device)
    V = space.Vh
    v = varf.c_varf(V)
    bc = varf.c_bc(V, device_marking=space.has_boundary)
    h = C.c_void_p()
    check(lib().ffgpu_matrix_assemble(space.h, C.byref(v), C.byref(bc), _ptr(rhs_out), C.byref(h)))
    return Matrix(h, space, solver=solver, eps=eps, itmax=itmax, dim_krylov=dim_krylov,
                  tgv=varf.tgv, device=device)


def rhs(varf: VarForm, Vh, out=None, device=0):
    """real[int] b = a(0,Vh)."""
    space = Vh if isinstance(Vh, DeviceSpace) else DeviceSpace(Vh, device)
    V = space.Vh
    if out is None:
        out = _touched_zeros(V.ndof)
    v = varf.c_varf(V)
    bc = varf.c_bc(V, device_marking=space.has_boundary)
    check(lib().ffgpu_rhs_assemble(space.h, C.byref(v), C.byref(bc), _ptr(out)))
    return out


# ------------------------------------------------------------------ meshes and numbering on the device
class _DeviceMeshInfo:
    """Sizes of a mesh whose arrays live on the GPU (what DeviceSpace and VarForm read)."""

    def __init__(self, dim, nv, nt, nbe):
        self.dim, self.nv, self.nt, self.nbe = dim, nv, nt, nbe


class _DeviceSpaceInfo:
    """FE-space metadata of a device-built space (kind, element code, DOFs)."""

    def __init__(self, Th, kind, ndof):
        self.Th, self.kind = Th, kind
        self.fe = {"P1": 1, "P2": 2, "P2vec": 3}[kind]
        self.bs = 3 if kind == "P2vec" else 1
        nn = Th.dim + 1 if kind == "P1" else (10 if Th.dim == 3 else 6)
        self.ndofK = nn * self.bs
        self.ndof = ndof


def device_mesh(dim, nx, ny=None, nz=None, device=0):
    """FreeFEM's square(nx, ny) (dim 2) or cube(nx, ny, nz) (dim 3) built on the GPU: a dict of
    torch tensors on the device (coords, elems, belems, blabel) and the sizes."""
    import torch
    ny = nx if ny is None else ny
    nz = (nx if nz is None else nz) if dim == 3 else 0
    nv, nt, nbe = C.c_int(), C.c_int(), C.c_int()
    check(lib().ffgpu_mesh_sizes(dim, nx, ny, nz, C.byref(nv), C.byref(nt), C.byref(nbe)))
    dev = torch.device("cuda", device)
    X = torch.empty((nv.value, dim), dtype=torch.float64, device=dev)
    E = torch.empty((nt.value, dim + 1), dtype=torch.int32, device=dev)
    BE = torch.empty((nbe.value, dim), dtype=torch.int32, device=dev)
    BL = torch.empty(nbe.value, dtype=torch.int32, device=dev)
    check(lib().ffgpu_mesh_build(context(device), dim, nx, ny, nz, _ptr(X), _ptr(E), _ptr(BE), _ptr(BL)))
    return dict(dim=dim, nv=nv.value, nt=nt.value, nbe=nbe.value, coords=X, elems=E, belems=BE, blabel=BL)


def number_p2(elems, nv, device=0):
    """FreeFEM's first-encounter P2 node table of a tetrahedral mesh, computed on the GPU:
    (nodes (nt, 10) int32 on the device, node count)."""
    import torch
    E = elems if hasattr(elems, "data_ptr") else torch.as_tensor(np.ascontiguousarray(elems, np.int32),
                                                                  device=torch.device("cuda", device))
    nt = E.shape[0]
    nodes = torch.empty((nt, 10), dtype=torch.int32, device=E.device)
    nn = C.c_int()
    check(lib().ffgpu_number_p2(context(device), int(nv), nt, _ptr(E), _ptr(nodes), C.byref(nn)))
    return nodes, nn.value


def number_p2_2d(elems, nv):
    """FreeFEM's P2 node table of a triangular mesh (host arrays): vertex nodes, edge nodes by
    first encounter, then FreeFEM's Gibbs renumbering -> (nodes (nt, 6) int32, node count)."""
    E = np.ascontiguousarray(elems, np.int32)
    nodes = np.empty((E.shape[0], 6), np.int32)
    nn = C.c_int()
    check(lib().ffgpu_number_p2_2d(int(nv), E.shape[0], _ptr(E), _ptr(nodes), C.byref(nn)))
    return nodes, nn.value


def device_space(kind, dim, nx, ny=None, nz=None, device=0):
    """``fespace Vh(square(...)/cube(...), kind)`` with the mesh, the DOF numbering and the space
    built on the GPU (no host arrays): a DeviceSpace for ffgpu.matrix / ffgpu.rhs."""
    import torch
    m = device_mesh(dim, nx, ny, nz, device)
    Th = _DeviceMeshInfo(dim, m["nv"], m["nt"], m["nbe"])
    if kind == "P1":
        dof, ndof = m["elems"], m["nv"]
    elif dim == 3 and kind in ("P2", "P2vec"):
        nodes, nn = number_p2(m["elems"], m["nv"], device)
        if kind == "P2":
            dof, ndof = nodes, nn
        else:
            n3 = 3 * nodes
            dof, ndof = torch.cat([n3, n3 + 1, n3 + 2], dim=1).contiguous(), 3 * nn
    elif dim == 2 and kind == "P2":
        # FreeFEM's Gibbs renumbering is a sequential graph algorithm: it runs on the host
        nodes, ndof = number_p2_2d(m["elems"].cpu().numpy(), m["nv"])
        dof = torch.from_numpy(nodes).to(m["elems"].device)
    else:
        raise NotImplementedError("on the device: P1, P2 (2D, 3D) and [P2,P2,P2] on tetrahedra")
    S = DeviceSpace(_DeviceSpaceInfo(Th, kind, ndof), device=device, coords=m["coords"], elems=m["elems"],
                    dof=dof, belems=m["belems"], blabel=m["blabel"])
    S.arrays = dict(m, dof=dof)
    return S


# ------------------------------------------------------------------ FreeFEM's text forms
_TEXT_FORMATS = {"coo": 0, "morse": 1}


def read_matrix_text(path):
    """``matrix A; ifstream f(path); f >> A;``: FreeFEM's "(COO)" or "(Morse)" text form ->
    (n, m, half, rowptr, col, val), sorted CSR (a repeated entry keeps its last value)."""
    n, m, half = C.c_int(), C.c_int(), C.c_int()
    nnz = C.c_int64()
    bp = str(path).encode()
    check(lib().ffgpu_matrix_text_read(bp, C.byref(n), C.byref(m), C.byref(nnz), C.byref(half),
                                       None, None, None))
    rp = np.empty(n.value + 1, np.int32)
    cl = np.empty(nnz.value, np.int32)
    vl = np.empty(nnz.value, np.float64)
    check(lib().ffgpu_matrix_text_read(bp, C.byref(n), C.byref(m), C.byref(nnz), C.byref(half),
                                       _ptr(rp), _ptr(cl), _ptr(vl)))
    return n.value, m.value, half.value, rp, cl, vl


def write_matrix_text(path, rowptr, col, val, m=None, half=0, format="coo"):
    """``ofstream f(path); f << A;`` for a sorted CSR: format "coo" (FreeFEM's default print of
    a sorted matrix) or "morse"."""
    rp = np.ascontiguousarray(rowptr, np.int32)
    cl = np.ascontiguousarray(col, np.int32)
    vl = np.ascontiguousarray(val, np.float64)
    n = rp.size - 1
    check(lib().ffgpu_matrix_text_write(str(path).encode(), _TEXT_FORMATS[format], n,
                                        n if m is None else int(m), int(half), _ptr(rp), _ptr(cl), _ptr(vl)))


def read_vector_text(path):
    """``real[int] b(n); ifstream f(path); f >> b;`` (RNM_tpl.hpp:112-125): the length, then the
    values."""
    with open(path) as f:
        tok = f.read().split()
    n = int(tok[0])
    if len(tok) < n + 1:
        raise ValueError(f"{path}: {len(tok) - 1} values for a vector of length {n}")
    return np.array([float(t) for t in tok[1:n + 1]])


def write_vector_text(path, v, digits=17):
    """``ofstream f(path); f << b;`` (RNM_tpl.hpp:100-110: the length, then five values per
    line); `digits` significant digits (FreeFEM writes at least 10)."""
    v = np.asarray(v, np.float64)
    parts = [f"{v.size}\t\n\t"]
    for i, x in enumerate(v):
        x = 0.0 if abs(x) < 1e-305 else float(x)
        parts.append(f"{x:3.{digits}g}" + ("\n\t" if i % 5 == 4 else "\t"))
    with open(path, "w") as f:
        f.write("".join(parts) + "\n")


def matrix_from_file(path, solver="CG", eps=1e-6, tgv=1e30, device=0) -> Matrix:
    """A matrix FreeFEM wrote (``f << A``) loaded into the device solver."""
    n, m, half, rp, cl, vl = read_matrix_text(path)
    if n != m:
        raise ValueError(f"{path}: {n} x {m} matrix, the solvers need a square one")
    if half:
        raise ValueError(f"{path}: half (symmetric) storage; the device path keeps full storage")
    return matrix_from_csr(rp, cl, vl, solver=solver, eps=eps, tgv=tgv, device=device)


def matrix_from_csr(rowptr, col, val, solver="CG", eps=1e-6, tgv=1e30, device=0) -> Matrix:
    """A FreeFEM-assembled matrix handed to the device solver (the addsolver path)."""
    rp = np.ascontiguousarray(rowptr, np.int32)
    cl = np.ascontiguousarray(col, np.int32)
    vl = np.ascontiguousarray(val, np.float64)
    h = C.c_void_p()
    check(lib().ffgpu_matrix_from_csr(context(device), rp.size - 1, cl.size, _ptr(rp), _ptr(cl),
                                      _ptr(vl), C.byref(h)))
    return Matrix(h, None, solver=solver, eps=eps, tgv=tgv, device=device)
