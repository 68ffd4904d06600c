"""CUDA path vs the oracle and FreeFEM's golden outputs, through the C ABI.

Bars: pattern and DOF numbering bit-exact; matrix values within 1e-12 relative
per entry (floor 1e-3 x the row's largest non-tgv entry, see golden_cases.value_errors);
solution within 1e-9 relative in the L2 norm; CG/GMRES iteration counts equal to FreeFEM's
within 2 (device reductions sum in a different order than the reference's serial loops).
"""
import numpy as np
import pytest

import ffgpu
import ffo
from ffgpu import mesh
from ffgpu.fespace import FESpace
from golden_cases import MATRIX_CASES, case, load, value_errors

pytestmark = pytest.mark.gpu

VAL_TOL = 1e-12
SOL_TOL = 1e-9


@pytest.fixture(scope="module", autouse=True)
def _lib_built():
    from ffgpu.build import build
    build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    ffgpu.context(0)
    yield


def gpu_varf(c):
    if c["form"] == "elasticity":
        return ffgpu.varf_elasticity(E=1.0, nu=0.3, f=c["f"], on=c["labels"])
    return ffgpu.varf_diffusion(kappa=c["kappa"], f=c["f"], on=c["labels"], c_mass=c.get("mass", 0.0))


@pytest.mark.parametrize("name", MATRIX_CASES)
def test_assembly_and_solve_against_freefem(name):
    c = case(name)
    d, sc = c["d"], c["sc"]
    Vh = FESpace(c["Th"], c["kind"], c.get("dof"))
    a = gpu_varf(c)
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(a, Vh, solver=c["solver"], eps=c["eps"], rhs_out=b)
    rp, cl, v = A.csr()
    I = np.repeat(np.arange(Vh.ndof), np.diff(rp))
    assert A.nnz == d["J"].size
    assert np.array_equal(I, d["I"]) and np.array_equal(cl, d["J"]), "pattern differs"
    assert value_errors(v, d["C"], rp).max() <= VAL_TOL
    assert np.abs(b - d["b"]).max() <= VAL_TOL * np.abs(d["b"]).max()
    u = A.solve(b)
    assert np.linalg.norm(u - d["u"]) <= SOL_TOL * np.linalg.norm(d["u"])
    assert abs(A.stats.iterations - int(sc["nit"])) <= 2
    # linear form alone (a(0,Vh)) equals the one assembled with the matrix
    b2 = ffgpu.rhs(a, A.space)
    assert np.array_equal(b, b2)


@pytest.mark.parametrize("name", ["p1sq_n16", "p1cubek_n4", "p2el_n2", "p2cube_n2"])
def test_transpose_mult_and_solve_against_oracle(name):
    c = case(name)
    Th = c["Th"]
    Vh = FESpace(Th, c["kind"], c.get("dof"))
    Ao = ffo.assemble(Th, Vh, form=c["form"], kappa=c["kappa"], quad=c["quad"], mass=c.get("mass", 0.0))
    bo = ffo.rhs(Th, Vh, f=c["f"], quad=c["quad"])
    ffo.setbc(Ao, bo, Vh.on(c["labels"]))
    A = ffgpu.matrix(gpu_varf(c), Vh, eps=1e-10)
    rng = np.random.default_rng(5)
    x = rng.standard_normal(Vh.ndof)
    for trans in (False, True):
        y = A.mult(x, trans=trans)
        yo = Ao.matmul(x, trans=trans)
        assert np.abs(y - yo).max() <= 1e-12 * np.abs(yo).max()
    ut = A.solve(bo, trans=True)
    uo, it, r, _ = ffo.cg(Ao, bo, eps=1e-10, trans=True)
    assert np.linalg.norm(ut - uo) <= SOL_TOL * np.linalg.norm(uo)
    assert abs(A.stats.iterations - it) <= 2


@pytest.mark.parametrize("name", [n for n in MATRIX_CASES if "gmres" not in n])
def test_double_float_spmv_mode(name):
    """spmv_mode=1 (products formed exactly on the FP32 pipe, double-float sums): same bars as
    the FP64 path -- solution 1e-9 relative to FreeFEM's, iterations within 2 (or 1%)."""
    c = case(name)
    d, sc = c["d"], c["sc"]
    Vh = FESpace(c["Th"], c["kind"], c.get("dof"))
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(gpu_varf(c), Vh, eps=c["eps"], rhs_out=b)
    u = A.solve(b, spmv_mode=1)
    assert np.linalg.norm(u - d["u"]) <= SOL_TOL * np.linalg.norm(d["u"])
    it = int(sc["nit"])
    assert abs(A.stats.iterations - it) <= max(2, it // 100)
    ut = A.solve(b, trans=True, spmv_mode=1)
    assert np.linalg.norm(ut - d["u"]) <= 1e-8 * np.linalg.norm(d["u"])


def test_double_float_spmv_mode_medium_elasticity():
    Th = mesh.cube(10)
    Vh = FESpace(Th, "P2vec")
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(ffgpu.varf_elasticity(f=(0, 0, -1.0), on=(4,)), Vh, eps=1e-10, rhs_out=b)
    u0 = A.solve(b)
    it0 = A.stats.iterations
    u1 = A.solve(b, spmv_mode=1)
    assert np.linalg.norm(u1 - u0) <= SOL_TOL * np.linalg.norm(u0)
    assert abs(A.stats.iterations - it0) <= max(2, it0 // 100)


@pytest.mark.parametrize("tag,tgv,solver", [("m1", -1.0, "GMRES"), ("m2", -2.0, "CG"), ("m3", -3.0, "GMRES"),
                                            ("p", 1e30, "CG")])
def test_tgv_variants_against_freefem(tag, tgv, solver):
    """FreeFEM's on(..., u=x) with tgv = -1 (unit diagonal, row zeroed), -2 (row and column),
    -3 (column only) and 1e30, non-zero Dirichlet data, on the device path."""
    d, sc = load("p1sq_n6_tgv" + tag)
    Th = mesh.square(6)
    Vh = FESpace(Th, "P1")
    g = np.ascontiguousarray(Th.coords[:, 0])
    a = ffgpu.varf_diffusion(f=1.0, on=(1, 2, 3, 4), g=g, tgv=tgv)
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(a, Vh, solver=solver, eps=1e-12, rhs_out=b)
    rp, cl, v = A.csr()
    assert np.array_equal(np.repeat(np.arange(Vh.ndof), np.diff(rp)), d["I"]) and np.array_equal(cl, d["J"])
    assert value_errors(v, d["C"], rp).max() <= VAL_TOL
    assert np.abs(b - d["b"]).max() <= VAL_TOL * np.abs(d["b"]).max()
    assert np.array_equal(ffgpu.rhs(a, A.space), b)
    u = A.solve(b)
    assert np.linalg.norm(u - d["u"]) <= SOL_TOL * np.linalg.norm(d["u"])
    assert abs(A.stats.iterations - int(sc["nit"])) <= 2


def test_multiple_rhs():
    c = case("p1sq_n16")
    Vh = FESpace(c["Th"], "P1")
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(gpu_varf(c), Vh, eps=1e-10, rhs_out=b)
    u = A.solve(b)
    B = np.stack([b, 2 * b, -b]).ravel()
    U = A.solve(B)
    U = U.reshape(3, -1)
    for k, s in enumerate([1, 2, -1]):
        assert np.linalg.norm(U[k] - s * u) <= 1e-9 * np.linalg.norm(u)


def test_repeated_solves_reuse_graph_safely():
    """The CUDA graph of the CG loop is cached per matrix; every solve must use its own x/b."""
    c = case("p1sqk_n8_jit")
    d = c["d"]
    Vh = FESpace(c["Th"], "P1")
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(gpu_varf(c), Vh, eps=1e-10, rhs_out=b)
    ref = A.solve(b)
    for s in (2.0, -0.5, 3.0):
        u = A.solve(s * b)
        assert np.linalg.norm(u - s * ref) <= 1e-9 * np.linalg.norm(s * ref)
    assert np.linalg.norm(ref - d["u"]) <= SOL_TOL * np.linalg.norm(d["u"])


def test_addsolver_path_matrix_from_csr():
    """A FreeFEM-assembled matrix (sorted CSR) solved on the device, as `set(A,solver=GPUCG)`."""
    c = case("p1sqk_n8_jit")
    d, sc = c["d"], c["sc"]
    rp = np.zeros(d["b"].size + 1, np.int32)
    np.add.at(rp, d["I"] + 1, 1)
    rp = np.cumsum(rp).astype(np.int32)
    A = ffgpu.matrix_from_csr(rp, d["J"], d["C"], eps=1e-10)
    u = A.solve(d["b"])
    assert np.linalg.norm(u - d["u"]) <= SOL_TOL * np.linalg.norm(d["u"])
    assert abs(A.stats.iterations - int(sc["nit"])) <= 2
    ug = A.solve(d["b"], solver="GMRES")
    assert np.linalg.norm(ug - d["u"]) <= 1e-8 * np.linalg.norm(d["u"])


def test_reassemble_matches_fresh_assembly():
    c = case("p1cubek_n4")
    Vh = FESpace(c["Th"], "P1")
    a1 = gpu_varf(c)
    A = ffgpu.matrix(a1, Vh)
    kap2 = np.asarray(c["kappa"]) * 2.5 + 0.1
    a2 = ffgpu.varf_diffusion(kappa=kap2, f=1.0, on=c["labels"])
    b = np.empty(Vh.ndof)
    A.reassemble(a2, rhs_out=b)
    B = ffgpu.matrix(a2, A.space)
    assert np.array_equal(A.csr()[2], B.csr()[2])
    assert np.array_equal(b, ffgpu.rhs(a2, A.space))


def test_reassemble_then_solve_uses_new_values():
    """A solve caches the solver layout and graph; a reassembly must invalidate both."""
    c = case("p1cubek_n4")
    Vh = FESpace(c["Th"], "P1")
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(gpu_varf(c), Vh, eps=1e-12, rhs_out=b)
    A.solve(b)
    A.solve(b, trans=True)
    kap2 = np.asarray(c["kappa"]) * 2.5 + 0.1
    a2 = ffgpu.varf_diffusion(kappa=kap2, f=1.0, on=c["labels"])
    A.reassemble(a2, rhs_out=b)
    B = ffgpu.matrix(a2, A.space, eps=1e-12)
    for trans in (False, True):
        ua = A.solve(b, trans=trans)
        ub = B.solve(b, trans=trans)
        assert np.array_equal(ua, ub)


def test_reassemble_after_many_tuned_shapes():
    """The SpMV layout of a shape is chosen once per context: after more shapes than any fixed
    cache would hold (each large enough to be timed), a fresh matrix of an already-seen shape
    still gets that shape's layout, so it solves bit for bit like the first one."""
    mats = []
    for n in range(100, 140):
        Vh = FESpace(mesh.square(n), "P1")
        A = ffgpu.matrix(ffgpu.varf_diffusion(f=1.0, on=(1, 2, 3, 4)), Vh, eps=1e-10)
        A.solve(np.ones(Vh.ndof))
        mats.append(A)
    Vh = FESpace(mesh.square(100), "P1")
    a = ffgpu.varf_diffusion(f=1.0, on=(1, 2, 3, 4))
    b = np.empty(Vh.ndof)
    B = ffgpu.matrix(a, Vh, eps=1e-12, rhs_out=b)
    ub = B.solve(b)
    assert B.layout_code() == mats[0].layout_code()
    u0 = mats[0].solve(b, eps=1e-12)
    assert np.array_equal(u0, ub)
    test_reassemble_then_solve_uses_new_values()


@pytest.mark.parametrize("name", ["p1sq_n16", "p2el_n2"])
def test_every_spmv_layout_against_freefem(name):
    """Each layout the tuner may pick (SELL-32 variants, block CSR lanes) solves FreeFEM's
    system to the solution bar; the same fixed layout gives the same bits in two matrices."""
    c = case(name)
    d = c["d"]
    Vh = FESpace(c["Th"], c["kind"], c.get("dof"))
    codes = list(range(64, 72)) + [1, 2, 4, 8]
    for code in codes:
        b = np.empty(Vh.ndof)
        A = ffgpu.matrix(gpu_varf(c), Vh, eps=c["eps"], rhs_out=b)
        u = A.solve(b, spmv_layout=code)
        assert A.layout_code() == code
        assert np.linalg.norm(u - d["u"]) <= SOL_TOL * np.linalg.norm(d["u"]), code
        B = ffgpu.matrix(gpu_varf(c), A.space, eps=c["eps"])
        assert np.array_equal(B.solve(b, spmv_layout=code), u), code
    for code in (5, 63, 72):
        with pytest.raises(ffgpu.FFGPUError):
            A.solve(b, spmv_layout=code)


def test_wide_band_matrix_against_oracle():
    """Rows and columns randomly permuted (bandwidth above 2^15, so the SpMV keeps 32-bit
    column indices): same solution as the oracle's on the unpermuted matrix."""
    Th = mesh.square(200)
    Vh = FESpace(Th, "P1")
    Ao = ffo.assemble(Th, Vh)
    bo = ffo.rhs(Th, Vh, f=1.0)
    ffo.setbc(Ao, bo, Vh.on((1, 2, 3, 4)))
    uo, it, _, _ = ffo.cg(Ao, bo, eps=1e-10)
    rp, cl, v = Ao.csr()
    n = Vh.ndof
    p = np.random.Generator(np.random.PCG64(5)).permutation(n)      # new row k = old row p[k]
    inv = np.empty(n, np.int64); inv[p] = np.arange(n)
    rows = np.repeat(np.arange(n), np.diff(rp))
    ni, nj = inv[rows], inv[cl]
    order = np.lexsort((nj, ni))
    ni, nj, nv = ni[order], nj[order], v[order]
    assert np.abs(ni - nj).max() >= 1 << 15
    prp = np.zeros(n + 1, np.int64)
    np.add.at(prp, ni + 1, 1)
    A = ffgpu.matrix_from_csr(np.cumsum(prp).astype(np.int32), nj.astype(np.int32), nv, eps=1e-10)
    up = A.solve(bo[p])
    u = up[inv]
    assert np.linalg.norm(u - uo) <= SOL_TOL * np.linalg.norm(uo)
    assert abs(A.stats.iterations - it) <= 2


def test_device_resident_inputs_torch():
    """Mesh, DOF table and vectors already in HBM (torch CUDA tensors) through the same ABI."""
    import torch
    c = case("p2el_n2")
    d = c["d"]
    Th = c["Th"]
    Vh = FESpace(Th, "P2vec")
    X = torch.from_numpy(Th.coords).cuda()
    E = torch.from_numpy(Th.elems).cuda()
    D = torch.from_numpy(Vh.dof).cuda()
    S = ffgpu.DeviceSpace(Vh, coords=X, elems=E, dof=D)
    b = torch.empty(Vh.ndof, dtype=torch.float64, device="cuda")
    A = ffgpu.matrix(gpu_varf(c), S, eps=1e-10, rhs_out=b)
    u = A.solve(b)
    torch.cuda.synchronize()
    uh = u.cpu().numpy()
    assert np.linalg.norm(uh - d["u"]) <= SOL_TOL * np.linalg.norm(d["u"])


def test_p1_space_without_dof_table_equals_explicit_table():
    """A P1 space created with no DOF table (its DOFs are the vertices) assembles the same
    matrix and right-hand side, bit for bit, as one given FreeFEM's table explicitly."""
    import torch
    Th = mesh.cube(6)
    Vh = FESpace(Th, "P1")
    kappa = np.exp(np.random.Generator(np.random.PCG64(5)).standard_normal(Th.nt))
    a = ffgpu.varf_diffusion(kappa=kappa, f=1.0, on=(1, 3))
    S0 = ffgpu.DeviceSpace(Vh)                                        # no table crosses
    S1 = ffgpu.DeviceSpace(Vh, dof=np.ascontiguousarray(Vh.dof))      # FreeFEM's table
    E = torch.from_numpy(Th.elems).cuda()
    S2 = ffgpu.DeviceSpace(Vh, elems=E)                               # device mesh, no table
    out = []
    for S in (S0, S1, S2):
        b = np.empty(Vh.ndof)
        A = ffgpu.matrix(a, S, rhs_out=b)
        rp, cl, v = A.csr()
        out.append((rp, cl, v, b))
    for rp, cl, v, b in out[1:]:
        assert np.array_equal(rp, out[0][0]) and np.array_equal(cl, out[0][1])
        assert np.array_equal(v, out[0][2]) and np.array_equal(b, out[0][3])


def test_full_size_2d_poisson_known_answers():
    """square(256,256) P1 Poisson, qf2pT (the CPU-runnable headline case): nnz formula
    7 nv - 8 n - 6 = 460289, FreeFEM's recorded umax 0.0736705 and ||u|| 10.5628 (532 CG
    iterations), and the oracle's solution at 1e-9."""
    Th = mesh.square(256)
    Vh = FESpace(Th, "P1")
    a = ffgpu.varf_diffusion(f=1.0, on=(1, 2, 3, 4))
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(a, Vh, eps=1e-10, rhs_out=b)
    assert A.nnz == 7 * Th.nv - 8 * 256 - 6 == 460289
    u = A.solve(b)
    assert abs(u.max() - 0.0736705) < 5e-7
    assert abs(np.linalg.norm(u) - 10.5628) < 5e-4
    assert abs(A.stats.iterations - 532) <= 2
    Ao = ffo.assemble(Th, Vh, quad="qf2pT")
    bo = ffo.rhs(Th, Vh, f=1.0, quad="qf2pT")
    ffo.setbc(Ao, bo, Vh.on((1, 2, 3, 4)))
    rp, cl, v = A.csr()
    rpo, clo, vo = Ao.csr()
    assert np.array_equal(rp, rpo) and np.array_equal(cl, clo)
    assert value_errors(v, vo, rpo).max() <= VAL_TOL
    uo, it, r, _ = ffo.cg(Ao, bo, eps=1e-10)
    assert np.linalg.norm(u - uo) <= SOL_TOL * np.linalg.norm(uo)


@pytest.mark.parametrize("n", [6, 10])
def test_elasticity_medium_against_oracle(n):
    Th = mesh.cube(n)
    Vh = FESpace(Th, "P2vec")
    a = ffgpu.varf_elasticity(f=(0, 0, -1.0), on=(4,))
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(a, Vh, eps=1e-10, rhs_out=b)
    Ao = ffo.assemble(Th, Vh, form="elasticity")
    bo = ffo.rhs(Th, Vh, f=(0, 0, -1.0))
    ffo.setbc(Ao, bo, Vh.on((4,)))
    rp, cl, v = A.csr()
    rpo, clo, vo = Ao.csr()
    assert np.array_equal(rp, rpo) and np.array_equal(cl, clo)
    assert value_errors(v, vo, rpo).max() <= VAL_TOL
    assert np.abs(b - bo).max() <= VAL_TOL * np.abs(bo).max()
    u = A.solve(b)
    uo, it, r, _ = ffo.cg(Ao, bo, eps=1e-10)
    assert np.linalg.norm(u - uo) <= SOL_TOL * np.linalg.norm(uo)
    assert abs(A.stats.iterations - it) <= max(2, it // 100)


def test_gmres_against_freefem():
    c = case("p1sq_n12_gmres")
    d, sc = c["d"], c["sc"]
    Vh = FESpace(c["Th"], "P1")
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(gpu_varf(c), Vh, solver="GMRES", eps=1e-10, rhs_out=b)
    u = A.solve(b)
    assert np.linalg.norm(u - d["u"]) <= SOL_TOL * np.linalg.norm(d["u"])
    assert abs(A.stats.iterations - int(sc["nit"])) <= 2


def test_nonconvergence_is_an_error():
    """FreeFEM aborts (ffassert) when CG exhausts itmax; the device path returns ENOCONV."""
    c = case("p1sq_n16")
    Vh = FESpace(c["Th"], "P1")
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(gpu_varf(c), Vh, eps=1e-10, itmax=3, rhs_out=b)
    with pytest.raises(ffgpu.FFGPUError) as ei:
        A.solve(b)
    assert ei.value.code == -3
    assert A.stats.iterations == 3


@pytest.mark.parametrize("name", MATRIX_CASES)
def test_bc_mask_device_equals_host(name):
    """on(labels) marked on the device from the boundary elements = the host FESpace.on mask
    (which the FreeFEM fixtures pin through the assembled tgv rows)."""
    c = case(name)
    Vh = FESpace(c["Th"], c["kind"], c.get("dof"))
    S = ffgpu.DeviceSpace(Vh)
    assert np.array_equal(S.bc_mask(c["labels"]), Vh.on(c["labels"]))
    if c["kind"] == "P2vec":
        assert np.array_equal(S.bc_mask(c["labels"], components=(0, 2)), Vh.on(c["labels"], (0, 2)))
    for labels in [(1,), (2, 3)]:
        assert np.array_equal(S.bc_mask(labels), Vh.on(labels))


def test_bad_inputs_rejected_on_host_or_device():
    Th = mesh.square(4)
    Vh = FESpace(Th, "P1")
    bad = Vh.dof.copy()
    bad[3, 1] = Vh.ndof + 7          # DOF out of range: found by the device check, no fault
    with pytest.raises(ffgpu.FFGPUError):
        ffgpu.DeviceSpace(Vh, dof=bad)
    with pytest.raises(ffgpu.FFGPUError):
        ffgpu.matrix(ffgpu.varf_elasticity(f=1.0, on=(1,)), Vh)   # elasticity on a scalar space


def test_matrix_from_freefem_text_file_and_save(tmp_path):
    """A matrix in FreeFEM's text form (f << A) solved on the device; a device matrix saved in
    that form reads back unchanged."""
    d, sc = load("p1sq_n16")
    n = d["b"].size
    rp = np.concatenate([[0], np.cumsum(np.bincount(d["I"], minlength=n))]).astype(np.int32)
    p = tmp_path / "A.txt"
    ffgpu.write_matrix_text(p, rp, d["J"], d["C"])
    A = ffgpu.matrix_from_file(p, eps=1e-10)
    u = A.solve(d["b"])
    assert np.linalg.norm(u - d["u"]) <= SOL_TOL * np.linalg.norm(d["u"])
    assert abs(A.stats.iterations - int(sc["nit"])) <= 2
    c = case("p2el_n2")
    Vh = FESpace(c["Th"], c["kind"])
    B = ffgpu.matrix(gpu_varf(c), Vh, eps=1e-10)
    for fmt in ("coo", "morse"):
        B.save(tmp_path / f"B_{fmt}.txt", format=fmt)
        n2, m2, half, rp2, cl2, vl2 = ffgpu.read_matrix_text(tmp_path / f"B_{fmt}.txt")
        rpb, clb, vlb = B.csr()
        assert np.array_equal(rp2, rpb) and np.array_equal(cl2, clb) and np.array_equal(vl2, vlb)
