"""Meshes in FreeFEM's own vertex/element order.

``square`` and ``cube`` reproduce the meshes FreeFEM's ``square(nx,ny)`` and ``cube(nx,ny,nz)``
build (vertex numbering, element vertex order, boundary elements and labels), because the
DOF numbering and therefore the sparsity pattern follow from that order.

* ``square``: ``Carre_`` in src/fflib/lgmesh.cpp:1229-1384 -- vertex (i,j) -> i + j*(nx+1) at
  (i/nx, j/ny); each square split (i0,i1,i2), (i0,i2,i3); boundary edges bottom (label 1),
  right (2), top (3), left (4).
* ``cube``: ``BuildCube`` in src/fflib/msh3.cpp:7879-8132 (kind 6) -- vertex p = i + (nx+1) j
  + (nx+1)(ny+1) k at (i/nx, j/ny, k/nz) computed as x0 + (1/nx)*i; every hexahedron split
  into the same 6 tetrahedra; boundary faces labelled 1 (y=0), 2 (x=1), 3 (y=1), 4 (x=0),
  5 (z=0), 6 (z=1).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

# The six tetrahedra of one hexahedron as corners c = a + 2b + 4c' of the unit hex, in the
# order (and vertex order) FreeFEM's cube(...) emits them for its default split (kind 6).
HEX6_TETS = np.array([[4, 0, 6, 7], [0, 4, 5, 7], [1, 0, 5, 7],
                      [0, 1, 3, 7], [2, 0, 3, 7], [0, 2, 6, 7]], dtype=np.int64)
# local faces of a tetrahedron (vertex triples), FreeFEM's Tet::nvface order
TET_FACES = np.array([[3, 2, 1], [0, 2, 3], [3, 1, 0], [0, 1, 2]], dtype=np.int64)
# cube boundary bit (1<<b: x=0, x=1, y=0, y=1, z=0, z=1) -> face label
CUBE_BIT_LABEL = np.array([4, 2, 1, 3, 5, 6], dtype=np.int64)


@dataclass
class Mesh:
    """Simplicial mesh: ``coords`` (nv, dim) float64, ``elems`` (nt, dim+1) int32,
    ``belems`` (nbe, dim) int32 boundary elements with labels ``blabel``."""

    dim: int
    coords: np.ndarray
    elems: np.ndarray
    belems: np.ndarray
    blabel: np.ndarray
    vlabel: np.ndarray = field(default=None)

    @property
    def nv(self) -> int:
        return int(self.coords.shape[0])

    @property
    def nt(self) -> int:
        return int(self.elems.shape[0])

    @property
    def nbe(self) -> int:
        return int(self.belems.shape[0])

    def measures(self) -> np.ndarray:
        X = self.coords
        v = self.elems
        if self.dim == 2:
            a, b, c = X[v[:, 0]], X[v[:, 1]], X[v[:, 2]]
            return 0.5 * ((b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0]))
        a = X[v[:, 0]]
        m = np.stack([X[v[:, 1]] - a, X[v[:, 2]] - a, X[v[:, 3]] - a], axis=1)
        return np.linalg.det(m) / 6.0


def square(nx: int, ny: int | None = None) -> Mesh:
    """FreeFEM ``square(nx, ny)`` on [0,1]^2 with the default diagonal."""
    ny = nx if ny is None else ny
    if nx < 1 or ny < 1:
        raise ValueError("square: nx, ny must be >= 1")
    nx1 = nx + 1
    j, i = np.meshgrid(np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    coords = np.stack([i.ravel() / nx, j.ravel() / ny], axis=1).astype(np.float64)
    jj, ii = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    i0 = (ii + jj * nx1).ravel()
    i1 = i0 + 1
    i2 = i1 + nx1
    i3 = i2 - 1
    t = np.empty((2 * nx * ny, 3), dtype=np.int64)
    t[0::2] = np.stack([i0, i1, i2], axis=1)
    t[1::2] = np.stack([i0, i2, i3], axis=1)
    # boundary edges: bottom, right, top, left
    ib = np.arange(nx)
    jb = np.arange(ny)
    bottom = np.stack([ib, ib + 1], axis=1)
    right = np.stack([nx + jb * nx1, nx + jb * nx1 + nx1], axis=1)
    top = np.stack([ib + ny * nx1, ib + ny * nx1 + 1], axis=1)
    left = np.stack([jb * nx1, jb * nx1 + nx1], axis=1)
    be = np.concatenate([bottom, right, top, left]).astype(np.int32)
    bl = np.concatenate([np.full(nx, 1), np.full(ny, 2), np.full(nx, 3), np.full(ny, 4)]).astype(np.int32)
    vl = np.zeros(coords.shape[0], dtype=np.int64)
    for e, l in zip(be, bl):
        vl[e] = l
    return Mesh(2, coords, t.astype(np.int32), be, bl, vl)


def cube(nx: int, ny: int | None = None, nz: int | None = None) -> Mesh:
    """FreeFEM ``cube(nx, ny, nz)`` (load "msh3") on [0,1]^3, 6 tetrahedra per hexahedron."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    if min(nx, ny, nz) < 1:
        raise ValueError("cube: sizes must be >= 1")
    nj = nx + 1
    nk = nj * (ny + 1)
    k, j, i = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    xd, yd, zd = 1.0 / nx, 1.0 / ny, 1.0 / nz
    coords = np.stack([0.0 + xd * i, 0.0 + yd * j, 0.0 + zd * k], axis=1)
    vbits = (1 * (i == 0) + 2 * (i == nx) + 4 * (j == 0) + 8 * (j == ny) + 16 * (k == 0)
             + 32 * (k == nz)).astype(np.int64)
    hk, hj, hi = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    hi, hj, hk = hi.ravel(), hj.ravel(), hk.ravel()
    corners = np.empty((hi.size, 8), dtype=np.int64)
    for c in range(2):
        for b in range(2):
            for a in range(2):
                corners[:, a + 2 * b + 4 * c] = (hi + a) + nj * (hj + b) + nk * (hk + c)
    tets = corners[:, HEX6_TETS].reshape(-1, 4)            # hex-major, 6 tets per hex
    # boundary faces in element order, face order f = 0..3, bit order b = 0..5
    fv = tets[:, TET_FACES]                                # (nt, 4, 3)
    common = vbits[fv[..., 0]] & vbits[fv[..., 1]] & vbits[fv[..., 2]]
    sel = np.zeros(common.shape + (6,), dtype=bool)
    for b in range(6):
        sel[..., b] = common == (1 << b)
    # FreeFEM loops element, face, bit: flatten in that order
    e_idx, f_idx, b_idx = np.nonzero(sel)
    order = np.lexsort((b_idx, f_idx, e_idx))
    e_idx, f_idx, b_idx = e_idx[order], f_idx[order], b_idx[order]
    be = fv[e_idx, f_idx].astype(np.int32)
    bl = CUBE_BIT_LABEL[b_idx].astype(np.int32)
    return Mesh(3, coords.astype(np.float64), tets.astype(np.int32), be, bl, vbits)


def movemesh(Th: Mesh, coords: np.ndarray) -> Mesh:
    """Same topology and numbering, new vertex coordinates (FreeFEM ``movemesh``)."""
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    if coords.shape != Th.coords.shape:
        raise ValueError("movemesh: coordinate array has the wrong shape")
    return Mesh(Th.dim, coords, Th.elems, Th.belems, Th.blabel, Th.vlabel)


def jittered_square(n: int, amplitude: float, rng: np.random.Generator) -> Mesh:
    """square(n,n) with interior vertices moved by U(-amplitude*h, amplitude*h)^2, h = 1/n."""
    Th = square(n, n)
    h = 1.0 / n
    d = rng.uniform(-amplitude * h, amplitude * h, size=(Th.nv, 2))
    ij = np.stack([np.arange(Th.nv) % (n + 1), np.arange(Th.nv) // (n + 1)], axis=1)
    border = (ij[:, 0] == 0) | (ij[:, 0] == n) | (ij[:, 1] == 0) | (ij[:, 1] == n)
    d[border] = 0.0
    return movemesh(Th, Th.coords + d)
