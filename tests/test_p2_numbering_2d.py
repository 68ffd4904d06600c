"""FreeFEM's numbering of the scalar P2 space on triangles (host code of the library).

* Against FreeFEM itself: the DOF tables ``Vh(k,i)`` FreeFEM printed for nine meshes
  (structured squares, Delaunay disks, an annulus, two disjoint squares, a truncated square)
  are reproduced bit for bit by ``ffgpu_number_p2_2d``.
* Against FreeFEM's own ``gibbsa_`` (``src/femlib/gibbs.cpp`` compiled into ``oracle/_ref``):
  the renumbering, both profiles included, on random graphs and on the node graphs of the
  fixture meshes.
"""
import ctypes as C

import numpy as np
import pytest

import ffgpu
import ffo
from ffgpu import _lib, mesh
from ffgpu.fespace import FESpace
from golden_cases import load

FIXTURES = ["p2sq_n4", "p2sqm_n4", "bt_p2sq_5x4", "p2num_sq7x3", "p2num_disk", "p2num_annulus",
            "p2num_two", "p2num_lshape", "p2num_disk80"]


@pytest.mark.parametrize("name", FIXTURES)
def test_p2_2d_numbering_equals_freefem(name):
    d, _ = load(name)
    nodes, nn = ffgpu.number_p2_2d(d["elems"], d["coords"].shape[0])
    assert nn == int(d["dof"].max()) + 1
    assert np.array_equal(nodes, d["dof"])


def test_fespace_2d_p2_uses_freefem_numbering():
    d, _ = load("p2sq_n4")
    Vh = FESpace(mesh.square(4), "P2")
    assert np.array_equal(Vh.dof, d["dof"]) and Vh.ndof == 81


def test_p2_2d_numbering_rejects_bad_meshes():
    with pytest.raises(ffgpu.FFGPUError):
        ffgpu.number_p2_2d(np.array([[0, 1, 5]], np.int32), 3)          # vertex out of range
    tri = np.array([[0, 1, 2], [1, 0, 3], [0, 1, 4]], np.int32)          # edge (0,1) thrice
    with pytest.raises(ffgpu.FFGPUError):
        ffgpu.number_p2_2d(tri, 5)


def _gibbs_mine(ptv, adj):
    n = ptv.size - 1
    a = adj.copy()
    r = np.empty(n, np.int64)
    po, pn = C.c_int64(), C.c_int64()
    rc = _lib.lib().ffgpu_gibbs_renumber(n, ptv.ctypes.data_as(C.c_void_p), a.ctypes.data_as(C.c_void_p),
                                         r.ctypes.data_as(C.c_void_p), C.byref(po), C.byref(pn))
    assert rc == 0
    return r, po.value, pn.value


def _gibbs_ref(ptv, adj):
    L = ffo.reflib()
    n = ptv.size - 1
    p = ptv.astype(np.int64).copy()
    a = np.concatenate([adj.astype(np.int64), np.zeros(100, np.int64)])
    r = np.zeros(n + 1, np.int64)
    po, pn = C.c_long(), C.c_long()
    L.ref_gibbs.restype = C.c_int
    L.ref_gibbs.argtypes = [C.c_long, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_long),
                            C.POINTER(C.c_long)]
    rc = L.ref_gibbs(n, p.ctypes.data, a.ctypes.data, r.ctypes.data, C.byref(po), C.byref(pn))
    assert rc == 0
    return r[:n], po.value, pn.value


def _random_graph(rng, n, avg, self_loops, ncomp):
    """Symmetric graph in 1-based CSR, neighbour lists in random order, ncomp components."""
    comp = rng.integers(0, ncomp, n)
    nbr = [set([i]) if self_loops else set() for i in range(n)]
    for _ in range(int(n * avg / 2)):
        i, j = rng.integers(0, n, 2)
        if i != j and comp[i] == comp[j]:
            nbr[i].add(j)
            nbr[j].add(i)
    ptv = [1]
    adj = []
    for i in range(n):
        lst = list(nbr[i])
        rng.shuffle(lst)
        adj += [v + 1 for v in lst]
        ptv.append(len(adj) + 1)
    return np.array(ptv, np.int64), np.array(adj, np.int64)


def _node_graph(nodes, nn):
    """FESpace::gibbsv: elements of each node ascending, their nodes in local order, first kept."""
    nt = nodes.shape[0]
    tris = [[] for _ in range(nn)]
    for t in range(nt):
        for v in nodes[t]:
            tris[v].append(t)
    ptv, adj = [1], []
    for i in range(nn):
        seen = set()
        for t in tris[i]:
            for v in nodes[t]:
                if v not in seen:
                    seen.add(v)
                    adj.append(v + 1)
        ptv.append(len(adj) + 1)
    return np.array(ptv, np.int64), np.array(adj, np.int64)


need_ref = pytest.mark.skipif(ffo.reflib() is None or not hasattr(ffo.reflib(), "ref_gibbs"),
                              reason="oracle/_ref (FreeFEM's own gibbs.cpp) not built here")


@need_ref
@pytest.mark.parametrize("seed", range(24))
def test_gibbs_equals_freefem_gibbsa_on_random_graphs(seed):
    rng = np.random.Generator(np.random.PCG64(1000 + seed))
    n = int(rng.integers(1, 400))
    ptv, adj = _random_graph(rng, n, avg=float(rng.uniform(0.5, 9.0)), self_loops=bool(seed % 3),
                             ncomp=int(rng.integers(1, 6)))
    r1, po1, pn1 = _gibbs_mine(ptv, adj)
    r2, po2, pn2 = _gibbs_ref(ptv, adj)
    assert np.array_equal(r1, r2)
    assert (po1, pn1) == (po2, pn2)
    assert np.array_equal(np.sort(r1), np.arange(1, n + 1))


@need_ref
@pytest.mark.parametrize("name", ["p2num_disk", "p2num_annulus", "p2num_two", "p2num_disk80"])
def test_gibbs_equals_freefem_gibbsa_on_p2_node_graphs(name):
    d, _ = load(name)
    E = d["elems"]
    nv = d["coords"].shape[0]
    # the numbering before the renumbering: vertices, then edges by first encounter
    edge_of = {}
    pre = np.empty((E.shape[0], 6), np.int64)
    nn = nv
    for t in range(E.shape[0]):
        pre[t, :3] = E[t]
        for j in range(3):
            key = tuple(sorted((int(E[t, (j + 1) % 3]), int(E[t, (j + 2) % 3]))))
            if key not in edge_of:
                edge_of[key] = nn
                nn += 1
            pre[t, 3 + j] = edge_of[key]
    ptv, adj = _node_graph(pre, nn)
    r1, po1, pn1 = _gibbs_mine(ptv, adj)
    r2, po2, pn2 = _gibbs_ref(ptv, adj)
    assert np.array_equal(r1, r2) and (po1, pn1) == (po2, pn2)
    if pn1 <= po1:
        assert np.array_equal(r1[pre] - 1, d["dof"])
