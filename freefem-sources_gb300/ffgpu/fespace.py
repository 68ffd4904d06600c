"""Finite element spaces with FreeFEM's DOF numbering, and Dirichlet DOF masks.

* P0: DOF = element number.
* P1: DOF = vertex number (nodes are the vertices, ``FESpace.cpp:698-701``,
  ``GenericMesh.hpp:1760-1764``).
* P2 on tetrahedra: nodes numbered by first encounter over the elements, each element
  contributing its 4 vertex keys then its 6 edge keys {01,02,03,12,13,23}
  (``GenericMesh::BuildDFNumbering``, src/femlib/GenericMesh.hpp:1878-1929).
* [P2,P2,P2] on tetrahedra: DOF = 3*node + component (FESpacen.hpp:582,656-657); the local
  DOF c*10 + i of an element is component c of its local node i, as ``Vh(k, i)`` lists them.
* P2 on triangles: vertex nodes, edge nodes by first encounter, then FreeFEM's Gibbs profile
  renumbering (``FESpace.cpp:623-877``, ``gibbs.cpp:1094-1166``), computed by the library's
  host routine ``ffgpu_number_p2_2d``; ``dof=`` still takes a table given by FreeFEM.

``on(labels)`` returns the DOF mask of ``on(labels, u=...)``: the DOFs of the boundary
elements carrying one of the labels (AssembleBC, src/fflib/problem.cpp:9881-10034).
"""
from __future__ import annotations

import numpy as np

from .mesh import Mesh

TET_EDGES = np.array([[0, 1], [0, 2], [0, 3], [1, 2], [1, 3], [2, 3]], dtype=np.int64)
TRI_EDGES = np.array([[1, 2], [2, 0], [0, 1]], dtype=np.int64)

FE_CODES = {"P1": 1, "P2": 2, "P2vec": 3}


def first_encounter_nodes(Th: Mesh) -> tuple[np.ndarray, int]:
    """P2 node table (nt, nvk + nedges) numbered by first encounter."""
    nvk = Th.dim + 1
    E = TET_EDGES if Th.dim == 3 else TRI_EDGES
    el = Th.elems.astype(np.int64)
    a = el[:, E[:, 0]]
    b = el[:, E[:, 1]]
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    big = np.int64(Th.nv + 1)
    vkeys = el * big + Th.nv            # (v, infinity)
    ekeys = lo * big + hi
    keys = np.concatenate([vkeys, ekeys], axis=1).ravel()
    uniq, first, inv = np.unique(keys, return_index=True, return_inverse=True)
    order = np.argsort(first, kind="stable")
    rank = np.empty_like(order)
    rank[order] = np.arange(order.size)
    nodes = rank[inv].reshape(Th.nt, nvk + E.shape[0])
    return nodes.astype(np.int32), int(uniq.size)


class FESpace:
    """``fespace Vh(Th, kind)``: kind in {"P0", "P1", "P2", "P2vec"} ("P2vec" = [P2,P2,P2])."""

    def __init__(self, Th: Mesh, kind: str, dof: np.ndarray | None = None):
        self.Th = Th
        self.kind = kind
        if kind == "P0":
            self.dof = np.arange(Th.nt, dtype=np.int32)[:, None]
            self.ndof = Th.nt
            self.nodes = self.dof
            self.bs = 1
        elif kind == "P1":
            self.dof = np.ascontiguousarray(Th.elems, dtype=np.int32)
            self.ndof = Th.nv
            self.nodes = self.dof
            self.bs = 1
        elif kind in ("P2", "P2vec"):
            if dof is not None:
                self.nodes = np.ascontiguousarray(dof, dtype=np.int32)
                nn = int(self.nodes.max()) + 1
            elif Th.dim == 3:
                self.nodes, nn = first_encounter_nodes(Th)
            else:
                if kind == "P2vec":
                    raise NotImplementedError("[P2,P2,P2] is provided on tetrahedra")
                from .api import number_p2_2d
                self.nodes, nn = number_p2_2d(Th.elems, Th.nv)
            if kind == "P2":
                self.dof = self.nodes
                self.ndof = nn
                self.bs = 1
            else:
                if Th.dim != 3:
                    raise NotImplementedError("[P2,P2,P2] is provided on tetrahedra")
                n3 = 3 * self.nodes.astype(np.int64)
                self.dof = np.concatenate([n3, n3 + 1, n3 + 2], axis=1).astype(np.int32)
                self.ndof = 3 * nn
                self.bs = 3
        else:
            raise ValueError(f"unknown finite element {kind!r}")
        self.fe = FE_CODES.get(kind, 0)

    @property
    def ndofK(self) -> int:
        return int(self.dof.shape[1])

    def on(self, labels, components=None) -> np.ndarray:
        """uint8 mask of the DOFs of ``on(labels, ...)`` for the given components."""
        Th = self.Th
        labels = np.atleast_1d(np.asarray(labels))
        sel = np.isin(Th.blabel, labels)
        bel = Th.belems[sel].astype(np.int64)
        mask = np.zeros(self.ndof, dtype=np.uint8)
        if bel.size == 0:
            return mask
        if self.kind == "P1":
            mask[np.unique(bel.ravel())] = 1
            return mask
        if self.kind == "P0":
            raise ValueError("on() is not defined for P0")
        # P2: vertex nodes and edge nodes of the boundary elements
        nvk = Th.dim + 1
        E = TET_EDGES if Th.dim == 3 else TRI_EDGES
        el = Th.elems.astype(np.int64)
        big = np.int64(Th.nv + 1)
        vnode = np.full(Th.nv, -1, dtype=np.int64)
        vnode[el.ravel()] = self.nodes[:, :nvk].astype(np.int64).ravel()
        a, b = el[:, E[:, 0]], el[:, E[:, 1]]
        ekey = (np.minimum(a, b) * big + np.maximum(a, b)).ravel()
        enode = self.nodes[:, nvk:].astype(np.int64).ravel()
        ukey, idx = np.unique(ekey, return_index=True)
        # edges of the boundary elements (segments in 2D, triangles in 3D)
        if Th.dim == 2:
            bedges = bel[:, [0, 1]]
        else:
            bedges = np.concatenate([bel[:, [0, 1]], bel[:, [1, 2]], bel[:, [0, 2]]])
        bk = np.minimum(bedges[:, 0], bedges[:, 1]) * big + np.maximum(bedges[:, 0], bedges[:, 1])
        pos = np.searchsorted(ukey, bk)
        if np.any(pos >= ukey.size) or np.any(ukey[np.minimum(pos, ukey.size - 1)] != bk):
            raise ValueError("boundary element edge not found in the mesh")
        nodes = np.unique(np.concatenate([vnode[np.unique(bel.ravel())], enode[idx[pos]]]))
        if self.kind == "P2":
            mask[nodes] = 1
        else:
            comps = [0, 1, 2] if components is None else list(components)
            for c in comps:
                mask[3 * nodes + c] = 1
        return mask
