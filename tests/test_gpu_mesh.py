"""FreeFEM's square/cube meshes and its P2 first-encounter numbering built on the device,
against this repository's host builders (which match FreeFEM's dumps bit for bit) and the
oracle's numbering."""
import numpy as np
import pytest

import ffgpu
import ffo
from ffgpu import mesh
from ffgpu.fespace import FESpace, first_encounter_nodes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib_built():
    from ffgpu.build import build
    build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    ffgpu.context(0)
    yield


@pytest.mark.parametrize("dims", [(1, 1), (7, 5), (2, 9), (1, 1, 1), (4, 3, 2), (2, 5, 3)])
def test_device_mesh_equals_freefem_order_builders(dims):
    m = ffgpu.device_mesh(len(dims), *dims)
    Th = mesh.square(*dims) if len(dims) == 2 else mesh.cube(*dims)
    assert (m["nv"], m["nt"], m["nbe"]) == (Th.nv, Th.nt, Th.nbe)
    assert np.array_equal(m["coords"].cpu().numpy(), Th.coords)
    assert np.array_equal(m["elems"].cpu().numpy(), Th.elems)
    assert np.array_equal(m["belems"].cpu().numpy(), Th.belems)
    assert np.array_equal(m["blabel"].cpu().numpy(), Th.blabel)


@pytest.mark.parametrize("dims", [(1, 1, 1), (3, 2, 2), (5, 4, 3)])
def test_device_p2_numbering(dims):
    Th = mesh.cube(*dims)
    nodes, nn = ffgpu.number_p2(Th.elems, Th.nv)
    ref, nref = first_encounter_nodes(Th)
    assert nn == nref and np.array_equal(nodes.cpu().numpy(), ref)
    tab, cnt = ffo.number_nodes(Th)
    assert cnt == nn and np.array_equal(tab, ref)


def test_device_p2_numbering_on_a_shuffled_mesh():
    """First encounter on an unstructured order: elements permuted, vertices relabelled."""
    Th = mesh.cube(4, 3, 3)
    rng = np.random.default_rng(7)
    perm_v = rng.permutation(Th.nv)
    el = perm_v[Th.elems][rng.permutation(Th.nt)].astype(np.int32)
    sh = mesh.Mesh(3, Th.coords[np.argsort(perm_v)], el, perm_v[Th.belems].astype(np.int32), Th.blabel, Th.vlabel)
    nodes, nn = ffgpu.number_p2(el, Th.nv)
    ref, nref = first_encounter_nodes(sh)
    assert nn == nref and np.array_equal(nodes.cpu().numpy(), ref)


@pytest.mark.parametrize("kind,dims", [("P1", (9, 7)), ("P1", (4, 3, 3)), ("P2", (3, 3, 2)), ("P2vec", (2, 2, 3)),
                                       ("P2", (6, 5))])
def test_device_built_space_assembles_the_same_matrix(kind, dims):
    S = ffgpu.device_space(kind, len(dims), *dims)
    Th = mesh.square(*dims) if len(dims) == 2 else mesh.cube(*dims)
    Vh = FESpace(Th, kind)
    assert S.Vh.ndof == Vh.ndof
    if kind == "P2vec":
        a = ffgpu.varf_elasticity(on=(4,))
    else:
        a = ffgpu.varf_diffusion(f=1.0, on=(1, 2))
    b1, b2 = np.empty(Vh.ndof), np.empty(Vh.ndof)
    A1 = ffgpu.matrix(a, S, eps=1e-10, rhs_out=b1)
    A2 = ffgpu.matrix(a, Vh, eps=1e-10, rhs_out=b2)
    for x, y in zip(A1.csr(), A2.csr()):
        assert np.array_equal(x, y)
    assert np.array_equal(b1, b2)


def test_2d_p2_device_space_matches_freefem():
    """square(4) P2: mesh on the device, FreeFEM's Gibbs numbering on the host; the assembled
    matrix equals FreeFEM's own (pattern exact, values within 1e-12)."""
    from golden_cases import load, value_errors
    d, _ = load("p2sq_n4")
    S = ffgpu.device_space("P2", 2, 4, 4)
    assert np.array_equal(S.arrays["dof"].cpu().numpy(), d["dof"])
    A = ffgpu.matrix(ffgpu.varf_diffusion(f=1.0, on=(1, 2, 3, 4)), S, eps=1e-10)
    I, J, V = A.coo()
    assert np.array_equal(I, d["I"]) and np.array_equal(J, d["J"])
    rowptr = A.csr()[0]
    assert value_errors(V, d["C"], rowptr).max() <= 1e-12
