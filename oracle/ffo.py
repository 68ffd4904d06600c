"""Python face of the CPU oracle (test infrastructure only).

Loads ``oracle/_build/libffo.so`` (the C restatement, ``ffo.c``) and, when present,
``oracle/_ref/libffref.so`` (FreeFEM's own HashMatrix.cpp and CG.cpp compiled from the
FreeFEM sources).  Only tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg use this module, as the checker.  Nothing in the product imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libffo.so")
REFLIB = os.path.join(HERE, "_ref", "libffref.so")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_bp = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")

QUAD = {"qf2pT": 2, "qf5pT": 5, "qf2pT4P1": 2, "tet2": 102, "tet5": 105}

_lib = None
_ref = None


def build(ref_dir: str | None = None) -> None:
    """Compile the oracle (and oracle/_ref when the FreeFEM sources are reachable)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    from paths import REFERENCE
    src = ref_dir or REFERENCE
    if os.path.isdir(os.path.join(src, "src", "femlib")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={src}"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.ffo_hm_new.restype = C.c_void_p
        L.ffo_hm_new.argtypes = [C.c_int]
        L.ffo_hm_free.argtypes = [C.c_void_p]
        L.ffo_hm_nnz.restype = C.c_int64
        L.ffo_hm_nnz.argtypes = [C.c_void_p]
        L.ffo_hm_coo.argtypes = [C.c_void_p, _ip, _ip, _dp]
        L.ffo_hm_csr.argtypes = [C.c_void_p, _ip, _ip, _dp]
        L.ffo_assemble.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, _ip, C.c_int, _ip, C.c_int,
                                   C.c_int, C.c_int, C.c_void_p, C.c_double, C.c_double, C.c_double,
                                   C.c_void_p, C.c_void_p, C.c_void_p]
        L.ffo_element_matrix.argtypes = [C.c_int, _dp, _ip, C.c_int, C.c_int, C.c_int, C.c_int,
                                         C.c_int, C.c_void_p, C.c_double, C.c_double, C.c_double, _dp]
        L.ffo_rhs.argtypes = [_dp, C.c_int, C.c_int, _dp, _ip, C.c_int, _ip, C.c_int, C.c_int,
                              C.c_void_p, C.c_int, _dp, C.c_void_p]
        L.ffo_quad_points.restype = C.c_int
        L.ffo_quad_points.argtypes = [C.c_int, _dp, _dp]
        L.ffo_setbc.argtypes = [C.c_void_p, C.c_void_p, _bp, C.c_void_p, C.c_double]
        L.ffo_bterm.argtypes = [C.c_void_p, C.c_void_p, C.c_int, _dp, _ip, C.c_int, _ip, C.c_int,
                                C.c_int, _ip, _ip, _ip, C.c_int, C.c_void_p, C.c_void_p, C.c_double,
                                C.c_void_p, C.c_int, _dp]
        L.ffo_cg.restype = C.c_int
        L.ffo_cg.argtypes = [C.c_void_p, _dp, _dp, C.c_double, C.c_int, C.c_int, C.c_double,
                             C.POINTER(C.c_int), _dp]
        L.ffo_fgmres.restype = C.c_int
        L.ffo_fgmres.argtypes = [C.c_void_p, _dp, _dp, C.c_double, C.c_int, C.c_int, C.c_int,
                                 C.c_double, C.POINTER(C.c_int), _dp]
        L.ffo_matmul.argtypes = [C.c_void_p, _dp, _dp, C.c_int]
        L.ffo_number_nodes.restype = C.c_int
        L.ffo_number_nodes.argtypes = [C.c_int, C.c_int, C.c_int, _ip, C.c_int, C.c_int, _ip]
        _lib = L
    return _lib


def reflib():
    """FreeFEM's own HashMatrix + CG (None when oracle/_ref was not built here)."""
    global _ref
    if _ref is None and os.path.exists(REFLIB):
        L = C.CDLL(REFLIB)
        L.ref_hm_new.restype = C.c_void_p
        L.ref_hm_new.argtypes = [C.c_int]
        L.ref_hm_free.argtypes = [C.c_void_p]
        L.ref_hm_add.argtypes = [C.c_void_p, C.c_long, _ip, _ip, _dp]
        L.ref_hm_setbc.argtypes = [C.c_void_p, _bp, C.c_double]
        L.ref_hm_nnz.restype = C.c_long
        L.ref_hm_nnz.argtypes = [C.c_void_p]
        L.ref_hm_coo.argtypes = [C.c_void_p, _ip, _ip, _dp]
        L.ref_hm_csr.argtypes = [C.c_void_p, _ip, _ip, _dp]
        L.ref_cg.restype = C.c_int
        L.ref_cg.argtypes = [C.c_void_p, _dp, _dp, C.c_double, C.c_int, C.c_int, C.c_double,
                             C.POINTER(C.c_int)]
        L.ref_fgmres.restype = C.c_int
        L.ref_fgmres.argtypes = [C.c_void_p, _dp, _dp, C.c_double, C.c_int, C.c_int, C.c_int,
                                 C.c_double, C.POINTER(C.c_int)]
        _ref = L
    return _ref


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class HashMatrix:
    """Oracle sparse matrix (restated HashMatrix: COO in insertion order + hash)."""

    def __init__(self, n: int):
        self.L = lib()
        self.n = n
        self.h = self.L.ffo_hm_new(n)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ffo_hm_free(self.h)
            self.h = None

    @property
    def nnz(self) -> int:
        return int(self.L.ffo_hm_nnz(self.h))

    def coo(self):
        m = self.nnz
        I = np.empty(m, np.int32); J = np.empty(m, np.int32); V = np.empty(m, np.float64)
        self.L.ffo_hm_coo(self.h, I, J, V)
        return I, J, V

    def csr(self):
        m = self.nnz
        rp = np.empty(self.n + 1, np.int32); cl = np.empty(m, np.int32); v = np.empty(m, np.float64)
        self.L.ffo_hm_csr(self.h, rp, cl, v)
        return rp, cl, v

    def matmul(self, x, trans=False):
        y = np.empty(self.n)
        self.L.ffo_matmul(self.h, np.ascontiguousarray(x, np.float64), y, int(trans))
        return y


def points_values(Th, quad, fn):
    """fn(x, y[, z]) at the points of oracle rule `quad` of every element -> (nt, nq[, ...])."""
    L = lib()
    dim = Th.dim
    P, W = np.zeros(14 * 3), np.zeros(14)
    nq = L.ffo_quad_points(int(quad), P, W)
    P = P[:nq * dim].reshape(nq, dim)
    X = Th.coords[Th.elems]                                   # (nt, dim+1, dim)
    xq = X[:, None, 0, :] * (1.0 - P.sum(axis=1))[None, :, None]
    for i in range(dim):
        xq = xq + X[:, None, i + 1, :] * P[None, :, i, None]
    return fn(*[xq[..., d] for d in range(dim)]), nq


def assemble(Th, Vh, form="diffusion", kappa=None, E=1.0, nu=0.3, mass=0.0, quad=None,
             c_stiff=1.0):
    """matrix A = a(Vh,Vh) of the oracle (no BC).  Returns a HashMatrix.  kappa: P0 array or a
    function k(x, y[, z]); mass: constant or a function c(x, y[, z]); functions are taken at the
    rule's points."""
    L = lib()
    dim = Th.dim
    if quad is None:
        quad = 5 if dim == 2 else 105
    elif isinstance(quad, str):
        quad = QUAD[quad]
    A = HashMatrix(Vh.ndof)
    X = np.ascontiguousarray(Th.coords, np.float64)
    el = np.ascontiguousarray(Th.elems, np.int32)
    dof = np.ascontiguousarray(Vh.dof, np.int32)
    fe = {"P1": 1, "P2": 2, "P2vec": 3}[Vh.kind]
    coef = None
    kqp = None
    if callable(kappa):
        val, nq = points_values(Th, quad, kappa)
        kqp = np.ascontiguousarray(np.broadcast_to(np.asarray(val, np.float64) * c_stiff, (Th.nt, nq)))
    elif kappa is not None or c_stiff != 1.0:
        coef = np.ascontiguousarray(
            (np.ones(Th.nt) if kappa is None else np.asarray(kappa, np.float64)) * c_stiff)
    mqp = None
    if callable(mass):
        val, nq = points_values(Th, quad, mass)
        mqp = np.ascontiguousarray(np.broadcast_to(np.asarray(val, np.float64), (Th.nt, nq)))
        mass = 0.0
    lame = None
    if form == "elasticity" and (np.ndim(E) > 0 or np.ndim(nu) > 0):
        Ea = np.broadcast_to(np.asarray(E, np.float64), (Th.nt,))
        na = np.broadcast_to(np.asarray(nu, np.float64), (Th.nt,))
        lame = np.ascontiguousarray(np.stack([Ea * na / ((1 + na) * (1 - 2 * na)), Ea / (2 * (1 + na))], axis=1))
        E, nu = 1.0, 0.3
    L.ffo_assemble(A.h, dim, Th.nt, X, el, Vh.ndofK, dof, fe, 1 if form == "elasticity" else 0,
                   int(quad), _ptr(coef), float(E), float(nu), float(mass), _ptr(mqp), _ptr(kqp), _ptr(lame))
    A._keep = (coef, mqp, kqp, lame)
    return A


def rhs(Th, Vh, f=1.0, quad=None):
    """real[int] b = a(0,Vh) for int(f . v); f scalar, per-component tuple, P0 array (nt[,nc]),
    or a function f(x, y[, z]) (a tuple of components for [P2,P2,P2]) taken at the rule's
    points, mapped as K(P) = sum_i lambda_i X_i."""
    L = lib()
    dim = Th.dim
    if quad is None:
        quad = 5 if dim == 2 else 105
    elif isinstance(quad, str):
        quad = QUAD[quad]
    nc = 3 if Vh.kind == "P2vec" else 1
    b = np.zeros(Vh.ndof)
    fe = {"P1": 1, "P2": 2, "P2vec": 3}[Vh.kind]
    fconst = np.zeros(3)
    fP0 = None
    fqp = None
    if callable(f):
        val, nq = points_values(Th, quad, f)
        if nc == 1:
            fqp = np.broadcast_to(np.asarray(val, np.float64), (Th.nt, nq))[..., None]
        else:
            fqp = np.stack([np.broadcast_to(np.asarray(c, np.float64), (Th.nt, nq)) for c in val], axis=-1)
        fqp = np.ascontiguousarray(fqp)
    elif np.isscalar(f):
        fconst[0] = f
    else:
        fa = np.asarray(f, np.float64)
        if fa.ndim == 1 and fa.size == nc and fa.size != Th.nt:
            fconst[:nc] = fa
        else:
            fP0 = np.ascontiguousarray(fa.reshape(Th.nt, nc))
    L.ffo_rhs(b, dim, Th.nt, np.ascontiguousarray(Th.coords), np.ascontiguousarray(Th.elems, np.int32),
              Vh.ndofK, np.ascontiguousarray(Vh.dof, np.int32), fe, int(quad), _ptr(fP0), nc, fconst,
              _ptr(fqp))
    return b


def boundary_adjacency(Th):
    """(element, local edge/face) of every boundary element: the element whose edge/face
    opposite local vertex f has the boundary element's vertices (the smallest element index if
    two do).  Independent numpy restatement of Mesh::BoundaryElement."""
    dim = Th.dim
    faces = [[1, 2], [2, 0], [0, 1]] if dim == 2 else [[3, 2, 1], [0, 2, 3], [3, 1, 0], [0, 1, 2]]
    el = np.asarray(Th.elems, np.int64)
    fv = np.sort(el[:, faces], axis=2).reshape(-1, dim)          # (nt*(dim+1), dim)
    bv = np.sort(np.asarray(Th.belems, np.int64), axis=1)
    nv = int(Th.nv)
    key = fv[:, 0]
    bkey = bv[:, 0]
    for c in range(1, dim):
        key = key * nv + fv[:, c]
        bkey = bkey * nv + bv[:, c]
    order = np.argsort(key, kind="stable")                         # stable: smallest element first
    pos = np.searchsorted(key[order], bkey)
    if np.any(pos >= key.size) or np.any(key[order][np.minimum(pos, key.size - 1)] != bkey):
        raise ValueError("boundary element without an adjacent element")
    idx = order[pos]
    return (idx // (dim + 1)).astype(np.int32), (idx % (dim + 1)).astype(np.int32)


def bterm(Th, Vh, labels=(), robin=None, g=None, A: HashMatrix | None = None, b=None, adj=None):
    """One boundary term on the boundary elements carrying one of `labels` (all when empty):
    robin (scalar or per boundary element) adds robin*u.v to A, g (scalar, per-component tuple
    or per boundary element [x ncomp]) adds g.v to b."""
    L = lib()
    bel_elem, bel_face = boundary_adjacency(Th) if adj is None else adj
    nc = 3 if Vh.kind == "P2vec" else 1
    fe = {"P1": 1, "P2": 2, "P2vec": 3}[Vh.kind]
    lab = np.ascontiguousarray(labels, np.int32)
    cP, cc = None, 0.0
    if robin is not None:
        if np.isscalar(robin):
            cc = float(robin)
        else:
            cP = np.ascontiguousarray(robin, np.float64)
    gP, gconst = None, np.zeros(3)
    if g is not None:
        if np.isscalar(g):
            gconst[0] = float(g)
        else:
            ga = np.asarray(g, np.float64)
            if ga.ndim == 1 and ga.size == nc and ga.size != Th.nbe:
                gconst[:nc] = ga
            else:
                gP = np.ascontiguousarray(ga.reshape(Th.nbe, nc))
    L.ffo_bterm(A.h if (A is not None and robin is not None) else None,
                _ptr(b) if (b is not None and g is not None) else None, Th.dim,
                np.ascontiguousarray(Th.coords, np.float64), np.ascontiguousarray(Th.elems, np.int32),
                Vh.ndofK, np.ascontiguousarray(Vh.dof, np.int32), fe, Th.nbe, bel_elem, bel_face,
                np.ascontiguousarray(Th.blabel, np.int32), lab.size, _ptr(lab) if lab.size else None,
                _ptr(cP), cc, _ptr(gP), nc, gconst)


def setbc(A: HashMatrix, b, onbc, g=None, tgv=1e30):
    onbc = np.ascontiguousarray(onbc, np.uint8)
    gg = None if g is None else np.ascontiguousarray(g, np.float64)
    lib().ffo_setbc(A.h, _ptr(b), onbc, _ptr(gg), float(tgv))


def cg(A: HashMatrix, b, x0=None, eps=1e-10, itmax=0, trans=False, tgv=1e30):
    x = np.zeros(A.n) if x0 is None else np.array(x0, np.float64)
    it = C.c_int(0)
    g = np.zeros(2)
    r = lib().ffo_cg(A.h, np.ascontiguousarray(b, np.float64), x, eps, itmax, int(trans), tgv,
                     C.byref(it), g)
    return x, it.value, r, g


def fgmres(A: HashMatrix, b, x0=None, eps=1e-10, itmax=0, restart=50, trans=False, tgv=1e30):
    x = np.zeros(A.n) if x0 is None else np.array(x0, np.float64)
    it = C.c_int(0)
    rr = np.zeros(1)
    r = lib().ffo_fgmres(A.h, np.ascontiguousarray(b, np.float64), x, eps, itmax, restart, int(trans),
                         tgv, C.byref(it), rr)
    return x, it.value, r, rr[0]


def number_nodes(Th, with_vertices=True, with_edges=True):
    nn = (Th.dim + 1 if with_vertices else 0) + ((6 if Th.dim == 3 else 3) if with_edges else 0)
    tab = np.empty((Th.nt, nn), np.int32)
    cnt = lib().ffo_number_nodes(Th.dim, Th.nv, Th.nt, np.ascontiguousarray(Th.elems, np.int32),
                                 int(with_vertices), int(with_edges), tab)
    return tab, cnt


# ------------------------------------------------------------------ FreeFEM's own code
class RefHashMatrix:
    """FreeFEM's HashMatrix<int,double> fed with the oracle's element contributions."""

    def __init__(self, n: int, I, J, V):
        self.L = reflib()
        if self.L is None:
            raise RuntimeError("oracle/_ref/libffref.so is not built")
        self.n = n
        self.h = self.L.ref_hm_new(n)
        self.L.ref_hm_add(self.h, len(I), np.ascontiguousarray(I, np.int32),
                          np.ascontiguousarray(J, np.int32), np.ascontiguousarray(V, np.float64))

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ref_hm_free(self.h)
            self.h = None

    @property
    def nnz(self):
        return int(self.L.ref_hm_nnz(self.h))

    def setbc(self, onbc, tgv=1e30):
        self.L.ref_hm_setbc(self.h, np.ascontiguousarray(onbc, np.uint8), float(tgv))

    def coo(self):
        m = self.nnz
        I = np.empty(m, np.int32); J = np.empty(m, np.int32); V = np.empty(m)
        self.L.ref_hm_coo(self.h, I, J, V)
        return I, J, V

    def csr(self):
        m = self.nnz
        rp = np.empty(self.n + 1, np.int32); cl = np.empty(m, np.int32); v = np.empty(m)
        self.L.ref_hm_csr(self.h, rp, cl, v)
        return rp, cl, v

    def cg(self, b, x0=None, eps=1e-10, itmax=0, trans=False, tgv=1e30):
        x = np.zeros(self.n) if x0 is None else np.array(x0, np.float64)
        it = C.c_int(0)
        r = self.L.ref_cg(self.h, np.ascontiguousarray(b, np.float64), x, eps, itmax, int(trans), tgv,
                          C.byref(it))
        return x, it.value, r

    def fgmres(self, b, x0=None, eps=1e-10, itmax=0, restart=50, trans=False, tgv=1e30):
        x = np.zeros(self.n) if x0 is None else np.array(x0, np.float64)
        it = C.c_int(0)
        r = self.L.ref_fgmres(self.h, np.ascontiguousarray(b, np.float64), x, eps, itmax, restart,
                              int(trans), tgv, C.byref(it))
        return x, it.value, r


def element_contributions(Th, Vh, form="diffusion", kappa=None, E=1.0, nu=0.3, mass=0.0, quad=None,
                          c_stiff=1.0):
    """All element-matrix entries (I, J, V) in FreeFEM's scatter order (element, row, col)."""
    L = lib()
    dim = Th.dim
    if quad is None:
        quad = 5 if dim == 2 else 105
    elif isinstance(quad, str):
        quad = QUAD[quad]
    fe = {"P1": 1, "P2": 2, "P2vec": 3}[Vh.kind]
    nd = Vh.ndofK
    X = np.ascontiguousarray(Th.coords, np.float64)
    el = np.ascontiguousarray(Th.elems, np.int32)
    coef = None
    kqp = None
    if callable(kappa):
        val, nq = points_values(Th, quad, kappa)
        kqp = np.ascontiguousarray(np.broadcast_to(np.asarray(val, np.float64) * c_stiff, (Th.nt, nq)))
    elif kappa is not None or c_stiff != 1.0:
        coef = np.ascontiguousarray(
            (np.ones(Th.nt) if kappa is None else np.asarray(kappa, np.float64)) * c_stiff)
    V = np.empty((Th.nt, nd, nd))
    M = np.empty(nd * nd)
    for k in range(Th.nt):
        L.ffo_element_matrix(dim, X, el, k, nd, fe, 1 if form == "elasticity" else 0, int(quad),
                             _ptr(coef), float(E), float(nu), float(mass), M)
        V[k] = M.reshape(nd, nd)
    d = Vh.dof.astype(np.int32)
    I = np.repeat(d[:, :, None], nd, axis=2).ravel()
    J = np.repeat(d[:, None, :], nd, axis=1).ravel()
    return I, J, V.ravel()
