"""The allocation-free CG entry point, for callers that cannot allocate device memory.

It is checked against the regular entry point (ffgpu_solve_cg through Matrix.solve) on the
same matrix, with the tolerances of the other parity tests (solution 1e-9 relative, iteration
count within 2), on two calls in a row -- the second call must not see the first call's
leftovers in the shared scratch array.  This file runs last in the suite on purpose."""
import ctypes as C

import numpy as np
import pytest

import ffgpu
from ffgpu import _lib, mesh
from ffgpu.fespace import FESpace

pytestmark = pytest.mark.gpu

SOL_TOL = 1e-9


@pytest.fixture(scope="module", autouse=True)
def _lib_built():
    from ffgpu.build import build
    build()
    ffgpu.context(0)
    yield


def _noalloc(rp, cl, vl, b, x, eps=1e-10, itmax=0, tgv=1e30):
    it = C.c_int(0)
    g = np.zeros(2)
    code = _lib.lib().ffgpu_solve_cg_csr_noalloc(
        int(rp.numel() - 1), int(cl.numel()), C.c_void_p(rp.data_ptr()), C.c_void_p(cl.data_ptr()),
        C.c_void_p(vl.data_ptr()), C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()), eps, itmax, tgv,
        None, C.byref(it), g.ctypes.data_as(C.c_void_p))
    return code, it.value


def test_noalloc_cg_matches_regular_entry_point_twice():
    import torch
    Th = mesh.cube(12)
    Vh = FESpace(Th, "P1")
    kappa = np.exp(np.random.default_rng(3).standard_normal(Th.nt))
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(ffgpu.varf_diffusion(kappa=kappa, f=1.0, on=(1, 2, 3, 4, 5, 6)), Vh, eps=1e-10, rhs_out=b)
    rp, cl, vl = A.csr()
    drp = torch.from_numpy(rp).cuda()
    dcl = torch.from_numpy(cl).cuda()
    dvl = torch.from_numpy(vl).cuda()
    for scale in (1.0, -2.5):
        u_ref = A.solve(scale * b)
        it_ref = A.stats.iterations
        db = torch.from_numpy(scale * b).cuda()
        dx = torch.zeros(Vh.ndof, dtype=torch.float64, device="cuda")
        code, it = _noalloc(drp, dcl, dvl, db, dx)
        assert code == 0, _lib.lib().ffgpu_last_error()
        u = dx.cpu().numpy()
        assert np.linalg.norm(u - u_ref) <= SOL_TOL * np.linalg.norm(u_ref)
        assert abs(it - it_ref) <= 2


def test_noalloc_rejects_oversize_and_host_arrays():
    import torch
    n = 524288 + 1
    rp = torch.zeros(n + 1, dtype=torch.int32, device="cuda")
    cl = torch.zeros(1, dtype=torch.int32, device="cuda")
    vl = torch.zeros(1, dtype=torch.float64, device="cuda")
    v = torch.zeros(n, dtype=torch.float64, device="cuda")
    it = C.c_int(0)
    code = _lib.lib().ffgpu_solve_cg_csr_noalloc(n, 1, C.c_void_p(rp.data_ptr()), C.c_void_p(cl.data_ptr()),
                                                 C.c_void_p(vl.data_ptr()), C.c_void_p(v.data_ptr()),
                                                 C.c_void_p(v.data_ptr()), 1e-10, 0, 1e30, None, C.byref(it), None)
    assert code == -1
    assert b"exceeds" in _lib.lib().ffgpu_last_error()
    hb = np.zeros(8)
    code = _lib.lib().ffgpu_solve_cg_csr_noalloc(8, 8, C.c_void_p(rp.data_ptr()), C.c_void_p(cl.data_ptr()),
                                                 C.c_void_p(vl.data_ptr()), hb.ctypes.data_as(C.c_void_p),
                                                 C.c_void_p(v.data_ptr()), 1e-10, 0, 1e30, None, C.byref(it), None)
    assert code == -1
    assert b"device memory" in _lib.lib().ffgpu_last_error()
