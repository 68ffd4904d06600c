"""The batch in the C ABI's layout (host only): counts, back-to-back coordinates and local
elements, and the P1 on(labels) mask, equal to the per-mesh FESpace builders."""
import numpy as np

from ffgpu import batch
from ffgpu.fespace import FESpace


def test_batch_arrays_match_the_per_mesh_spaces():
    meshes, _, _ = batch.c5_meshes(40, 16, 40, seed=3)
    nv, nt, X, E, on = batch.batch_arrays(meshes, on=(1, 3))
    assert np.array_equal(nv, [m.nv for m in meshes]) and np.array_equal(nt, [m.nt for m in meshes])
    assert np.array_equal(X, np.concatenate([m.coords for m in meshes]))
    assert np.array_equal(E, np.concatenate([m.elems for m in meshes]))
    ref = np.concatenate([FESpace(m, "P1").on((1, 3)) for m in meshes])
    assert np.array_equal(on, ref)
