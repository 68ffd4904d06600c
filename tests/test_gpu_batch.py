"""Batched problems against lone assemblies, the oracle and a FreeFEM fixture.

Each block of the batch matrix must be the matrix FreeFEM assembles for that problem alone
(pattern bit-exact, values 1e-12); each solution (FP32 inner / FP64 refinement to eps=1e-8)
must match the FP64 oracle solution to 1e-6 relative (BATCH_TOL: the outer tolerance 1e-8 times
a conditioning allowance of 100 for these meshes)."""
import numpy as np
import pytest

import ffgpu
import ffo
from ffgpu import batch, mesh
from ffgpu.fespace import FESpace
from golden_cases import load, value_errors

pytestmark = pytest.mark.gpu

BATCH_TOL = 1e-6


@pytest.fixture(scope="module", autouse=True)
def _lib_built():
    from ffgpu.build import build
    build()
    ffgpu.context(0)
    yield


def oracle_problem(Th, kappa, eps=1e-10):
    Vh = FESpace(Th, "P1")
    A = ffo.assemble(Th, Vh, kappa=kappa)
    b = ffo.rhs(Th, Vh, f=1.0)
    ffo.setbc(A, b, Vh.on((1, 2, 3, 4)))
    u, it, r, _ = ffo.cg(A, b, eps=eps)
    return A, b, u


def test_batch_against_oracle_and_freefem_fixture():
    d, sc = load("p1sqk_n8_jit")
    fix_mesh = mesh.movemesh(mesh.square(8), d["coords"])
    meshes, kappas, Ns = batch.c5_meshes(nprob=11, nmin=4, nmax=20, seed=5)
    meshes.insert(3, fix_mesh)
    kappas.insert(3, d["in_kappa"])
    B = batch.Batch(meshes)
    B.assemble(kappas, f=1.0)
    x = B.solve(eps=1e-8)
    assert B.stats.converged
    nt, lanes, ms = B.tuned()
    assert nt in (128, 256, 512, 1024) and lanes in (2, 4) and ms > 0
    bb = B.rhs()
    A = ffgpu.Matrix(ffgpu.lib().ffgpu_batch_matrix(B.h), None)
    A.h = None   # owned by the batch: do not destroy through this view
    xs, bs_ = B.split(x), B.split(bb)
    for p, (Th, k) in enumerate(zip(meshes, kappas)):
        Ao, bo, uo = oracle_problem(Th, k)
        assert np.abs(bs_[p] - bo).max() <= 1e-12 * np.abs(bo).max()
        err = np.linalg.norm(xs[p] - uo) / np.linalg.norm(uo)
        assert err <= BATCH_TOL, (p, err)
    # the fixture problem: FreeFEM's own solution
    p = 3
    assert np.linalg.norm(xs[p] - d["u"]) <= BATCH_TOL * np.linalg.norm(d["u"])
    assert np.abs(bs_[p] - d["b"]).max() <= 1e-12 * np.abs(d["b"]).max()


def test_batch_blocks_equal_lone_assemblies():
    meshes, kappas, Ns = batch.c5_meshes(nprob=6, nmin=3, nmax=9, seed=9)
    B = batch.Batch(meshes)
    B.assemble(kappas)
    h = ffgpu.lib().ffgpu_batch_matrix(B.h)
    view = ffgpu.Matrix.__new__(ffgpu.Matrix)
    import ctypes as C
    n, nnz, bs = C.c_int(), C.c_int64(), C.c_int()
    ffgpu.lib().ffgpu_matrix_info(h, C.byref(n), C.byref(nnz), C.byref(bs))
    rp = np.empty(n.value + 1, np.int32); cl = np.empty(nnz.value, np.int32); vl = np.empty(nnz.value)
    ffgpu.lib().ffgpu_matrix_csr(h, rp.ctypes.data_as(C.c_void_p), cl.ctypes.data_as(C.c_void_p),
                                 vl.ctypes.data_as(C.c_void_p))
    for p, (Th, k) in enumerate(zip(meshes, kappas)):
        r0, r1 = B.voff[p], B.voff[p + 1]
        sub_rp = rp[r0:r1 + 1] - rp[r0]
        sub_cl = cl[rp[r0]:rp[r1]] - r0
        sub_vl = vl[rp[r0]:rp[r1]]
        Ao, bo, uo = oracle_problem(Th, k)
        orp, ocl, ovl = Ao.csr()
        assert np.array_equal(sub_rp, orp) and np.array_equal(sub_cl, ocl)
        assert value_errors(sub_vl, ovl, orp).max() <= 1e-12


def test_batch_reassemble_and_resolve():
    meshes, kappas, Ns = batch.c5_meshes(nprob=8, nmin=6, nmax=14, seed=11)
    B = batch.Batch(meshes)
    B.assemble(kappas)
    x1 = B.solve(eps=1e-8).copy()
    B.assemble([2.0 * k for k in kappas])
    x2 = B.solve(eps=1e-8)
    # kappa scaled by 2 => solution halved
    assert np.linalg.norm(x2 - 0.5 * x1) <= 1e-6 * np.linalg.norm(x1)


def test_batch_from_arrays_equals_batch_from_meshes():
    meshes, kappas, _ = batch.c5_meshes(24, 16, 48, seed=11)
    B1 = batch.Batch(meshes)
    B1.assemble(kappas, f=1.0)
    x1 = B1.solve(eps=1e-8)
    B2 = batch.Batch(arrays=batch.batch_arrays(meshes))
    B2.assemble(np.concatenate(kappas), f=1.0)
    x2 = B2.solve(eps=1e-8)
    assert np.array_equal(x1, x2)


def test_batch_with_a_problem_of_more_than_65536_dofs():
    """A problem of 66 049 DOFs (square(256)) among small ones: the solver keeps 32-bit global
    columns (problem-local 16-bit columns need every problem below 65 536 DOFs); the same bar
    against the FP64 oracle, for the small problems alone too (16-bit columns)."""
    rng = np.random.Generator(np.random.PCG64(21))
    small, ks, _ = batch.c5_meshes(nprob=5, nmin=8, nmax=24, seed=13)
    big = mesh.square(256)
    kb = np.exp(rng.standard_normal(big.nt))
    meshes, kappas = [small[0], big] + small[1:], [ks[0], kb] + ks[1:]
    B = batch.Batch(meshes)
    B.assemble(kappas, f=1.0)
    xs = B.split(B.solve(eps=1e-8).copy())
    assert B.stats.converged
    for p, (Th, k) in enumerate(zip(meshes, kappas)):
        _, _, uo = oracle_problem(Th, k)
        err = np.linalg.norm(xs[p] - uo) / np.linalg.norm(uo)
        assert err <= BATCH_TOL, (p, err)
    S = batch.Batch(small)
    S.assemble(ks, f=1.0)
    ys = S.split(S.solve(eps=1e-8))
    for q, p in enumerate([0, 2, 3, 4, 5]):
        assert np.linalg.norm(ys[q] - xs[p]) <= 2 * BATCH_TOL * np.linalg.norm(xs[p]), p


def test_batch_create_rejects_a_vertex_out_of_range():
    """A problem whose element names a vertex outside its own mesh is refused with
    FFGPU_EINVAL naming the first such problem (checked on the device, no fault)."""
    meshes, _, _ = batch.c5_meshes(nprob=5, nmin=4, nmax=8, seed=3)
    nv, nt, coords, elems, onbc = batch.batch_arrays(meshes)
    toff = np.concatenate([[0], np.cumsum(nt)])
    bad = elems.copy()
    bad[toff[2] + 1, 2] = nv[2]          # one past problem 2's last vertex
    with pytest.raises(ffgpu.FFGPUError) as ei:
        batch.Batch(arrays=(nv, nt, coords, bad, onbc))
    assert ei.value.code == -1 and b"problem 2" in ffgpu.lib().ffgpu_last_error()
    neg = elems.copy()
    neg[toff[4], 0] = -1
    with pytest.raises(ffgpu.FFGPUError):
        batch.Batch(arrays=(nv, nt, coords, neg, onbc))
    # the context stays usable
    B = batch.Batch(arrays=(nv, nt, coords, elems, onbc))
    B.assemble([np.ones(m.nt) for m in meshes])
    B.solve(eps=1e-8)
    assert B.stats.converged


def test_batch_from_device_arrays_equals_host_arrays():
    """The mesh arrays may live on the device (torch CUDA tensors): the same batch, the same
    bits as from host arrays."""
    import torch
    meshes, kappas, _ = batch.c5_meshes(12, 16, 40, seed=17)
    nv, nt, coords, elems, onbc = batch.batch_arrays(meshes)
    B1 = batch.Batch(arrays=(nv, nt, coords, elems, onbc))
    B1.assemble(np.concatenate(kappas), f=1.0)
    x1 = B1.solve(eps=1e-8).copy()
    dev = torch.device("cuda", 0)
    B2 = batch.Batch(arrays=(nv, nt, torch.from_numpy(coords).to(dev), torch.from_numpy(elems).to(dev),
                             torch.from_numpy(onbc).to(dev)))
    B2.assemble(torch.from_numpy(np.concatenate(kappas)).to(dev), f=1.0)
    x2 = B2.solve(eps=1e-8)
    assert np.array_equal(x1, x2)
    assert np.array_equal(B1.rhs(), B2.rhs())
