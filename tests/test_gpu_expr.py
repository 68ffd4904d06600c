"""Coefficients and sources as expressions evaluated on the device (ffgpu_expr), and general
volume terms int(coef * op_i(v) * op_j(u)).

* FreeFEM's fixtures of coefficient and source functions (mq_*, kq_*, src_*), with the function
  written as an expression of x, y, z: matrix, b and solution as FreeFEM's (same bars as the
  host-evaluated path: values 1e-12, b 1e-12 of max |b|, solution 1e-9).
* FE functions by their DOF values (P0, P1, P2) and their derivatives: an interpolant that
  reproduces its function exactly (P1 of a linear, P2 of a quadratic function) gives the
  matrix of the function itself.
* General terms: (dx,dx)+(dy,dy) equals the built-in stiffness; an anisotropic tensor and an
  advection term against a numpy assembly of the same element matrices; GMRES on the
  nonsymmetric system against scipy's direct solve.
"""
import numpy as np
import pytest

import ffgpu
from ffgpu import expr as E
from ffgpu import mesh
from ffgpu.fespace import FESpace
from golden_cases import load, value_errors

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib_built():
    from ffgpu.build import build
    build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    ffgpu.context(0)
    yield


x, y, z = E.x, E.y, E.z
COEF = {
    "mq_sq_p1": ("P1", 1 + x * y, (1,)),
    "mq_sq_p2": ("P2", E.exp(x + y), (1, 2)),
    "mq_cube_p1": ("P1", 1 + z * x, (1,)),
    "mq_cube_p2": ("P2", 2 + E.cos(x) * y, (1,)),
    "kq_sq_p1": ("P1", 1 + x * x * y, (1, 3)),
    "kq_sq_p2": ("P2", E.exp(x - y), (1, 2)),
    "kq_cube_p2": ("P2", 1 + x * y * z, (1, 2)),
}
SRC = {
    "src_sq_p1": ("P1", E.sin(3 * x) * E.cos(2 * y) + x * y, None),
    "src_sq_p1_qf2": ("P1", E.exp(x) * (1 + y * y), "qf2pT"),
    "src_sq_p2": ("P2", E.exp(x) * y - E.cos(5 * y), None),
    "src_cube_p1": ("P1", x * y * z + E.sin(2 * z), None),
    "src_cube_p2": ("P2", E.cos(x + 2 * y) * z, None),
    "src_cube_el": ("P2vec", (x, y * z, -1 + x * x), None),
}


def fixture_space(name, kind):
    d, sc = load(name)
    dim = d["coords"].shape[1]
    Th = mesh.Mesh(dim, d["coords"], d["elems"], d["belems"], d["blabel"], d["vlabel"])
    Vh = FESpace(Th, kind)
    assert np.array_equal(Vh.dof, d["dof"])
    return d, sc, Th, Vh


@pytest.mark.parametrize("name", list(COEF))
def test_coefficient_expression_equals_freefem(name):
    kind, c, labels = COEF[name]
    d, sc, Th, Vh = fixture_space(name, kind)
    kw = dict(kappa=c) if name.startswith("kq_") else dict(c_mass=c)
    a = ffgpu.varf_diffusion(f=1.0, on=labels, **kw)
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(a, Vh, eps=1e-12, rhs_out=b)
    rp, cl, v = A.csr()
    I = np.repeat(np.arange(rp.size - 1), np.diff(rp))
    assert np.array_equal(I, d["I"]) and np.array_equal(cl, d["J"])
    assert value_errors(v, d["C"], rp).max() <= 1e-12
    assert np.abs(b - d["b"]).max() <= 1e-12 * np.abs(d["b"]).max()
    u = A.solve(b)
    assert np.linalg.norm(u - d["u"]) <= 1e-9 * np.linalg.norm(d["u"])
    assert abs(A.stats.iterations - int(sc["nit"])) <= 2


@pytest.mark.parametrize("name", list(SRC))
def test_source_expression_equals_freefem(name):
    kind, f, quad = SRC[name]
    d, sc, Th, Vh = fixture_space(name, kind)
    a = ffgpu.varf_elasticity(f=f, quad=quad) if kind == "P2vec" else ffgpu.varf_diffusion(f=f, quad=quad)
    b = ffgpu.rhs(a, Vh)
    assert np.max(np.abs(b - d["b"])) <= 1e-12 * np.max(np.abs(d["b"]))
    b2 = np.empty(Vh.ndof)
    ffgpu.matrix(a, Vh, rhs_out=b2)
    assert np.max(np.abs(b2 - d["b"])) <= 1e-12 * np.max(np.abs(d["b"]))


def _csr(a, Vh):
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(a, Vh, rhs_out=b)
    return A.csr(), b


def _close(m1, m2, tol=1e-12):
    (rp, cl, v), b = m1
    (rp2, cl2, v2), b2 = m2
    assert np.array_equal(rp, rp2) and np.array_equal(cl, cl2)
    assert value_errors(v, v2, rp).max() <= tol
    assert np.abs(b - b2).max() <= tol * np.abs(b2).max()


@pytest.mark.parametrize("dim", [2, 3])
def test_fe_functions_reproduce_their_functions(dim):
    Th = mesh.square(7, 5) if dim == 2 else mesh.cube(3, 2, 4)
    X = Th.coords
    lin = lambda p: 1.5 + 0.5 * p[..., 0] - 0.25 * p[..., 1] + (0.75 * p[..., 2] if dim == 3 else 0)
    ex_lin = 1.5 + 0.5 * x - 0.25 * y + (0.75 * z if dim == 3 else 0)
    V1 = FESpace(Th, "P1")
    uh = E.fe("P1", lin(X))
    on = (1, 2)
    # P1 interpolant of a linear function, as a stiffness coefficient and as a source
    _close(_csr(ffgpu.varf_diffusion(kappa=uh, f=uh, on=on), V1),
           _csr(ffgpu.varf_diffusion(kappa=ex_lin, f=ex_lin, on=on), V1))
    # its derivatives are the constant gradient
    _close(_csr(ffgpu.varf_diffusion(kappa=2 + E.dx(uh) * E.dy(uh), on=on), V1),
           _csr(ffgpu.varf_diffusion(kappa=E.const(2 + 0.5 * -0.25), on=on), V1))
    # P2 interpolant of a quadratic, on a P2 space (the space's own DOF table) and as a
    # function of another space (its table given) in a P1 assembly
    V2 = FESpace(Th, "P2")
    quad = lambda p: 1 + p[..., 0] * p[..., 1] + 0.5 * p[..., 0] ** 2
    ex_quad = 1 + x * y + 0.5 * x * x
    nodes = np.zeros((V2.ndof, dim))
    nodes[V2.dof[:, :dim + 1].ravel()] = X[Th.elems].reshape(-1, dim)
    edges = [(1, 2), (2, 0), (0, 1)] if dim == 2 else [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
    for k, (i, j) in enumerate(edges):
        nodes[V2.dof[:, dim + 1 + k]] = 0.5 * (X[Th.elems[:, i]] + X[Th.elems[:, j]])
    u2 = E.fe("P2", quad(nodes))
    _close(_csr(ffgpu.varf_diffusion(c_mass=u2, kappa=1 + E.dy(u2), on=on), V2),
           _csr(ffgpu.varf_diffusion(c_mass=ex_quad, kappa=1 + x, on=on), V2), tol=1e-11)
    u2b = E.fe("P2", quad(nodes), dof=V2.dof)
    _close(_csr(ffgpu.varf_diffusion(kappa=u2b * u2b, on=on), V1),
           _csr(ffgpu.varf_diffusion(kappa=ex_quad * ex_quad, on=on), V1), tol=1e-11)
    # P0: the per-element array path
    k0 = np.exp(np.random.Generator(np.random.PCG64(1)).standard_normal(Th.nt))
    _close(_csr(ffgpu.varf_diffusion(kappa=E.fe("P0", k0), on=on), V1),
           _csr(ffgpu.varf_diffusion(kappa=k0, on=on), V1))


def _elem_geometry(Th):
    X = Th.coords[Th.elems]
    d = Th.dim
    J = np.stack([X[:, i + 1] - X[:, 0] for i in range(d)], axis=2)     # columns = edges
    det = np.linalg.det(J)
    Jinv = np.linalg.inv(J)
    G = np.zeros((Th.nt, d + 1, d))
    G[:, 1:, :] = Jinv
    G[:, 0, :] = -Jinv.sum(axis=1)
    meas = np.abs(det) / (2 if d == 2 else 6)
    return meas, G


def _assemble_numpy(Th, Ke):
    import scipy.sparse as sp
    nt, k = Ke.shape[:2]
    rows = np.repeat(Th.elems, k, axis=1).ravel()
    cols = np.tile(Th.elems, (1, k)).ravel()
    n = Th.nv
    return sp.coo_matrix((Ke.ravel(), (rows, cols)), shape=(n, n)).tocsr()


def test_general_terms_against_numpy():
    pytest.importorskip("scipy")
    Th = mesh.jittered_square(12, 0.2, np.random.Generator(np.random.PCG64(3)))
    Vh = FESpace(Th, "P1")
    meas, G = _elem_geometry(Th)
    # isotropic through terms = the built-in stiffness
    _close(_csr(ffgpu.varf_diffusion(kappa=None, c_stiff=0.0, terms=[("dx", "dx", 1.0), ("dy", "dy", 1.0)]), Vh),
           _csr(ffgpu.varf_diffusion(), Vh))
    # anisotropic K and advection beta . grad u, constant coefficients
    K = np.array([[2.0, 0.3], [0.3, 0.5]])
    beta = np.array([1.0, -0.5])
    terms = [("dx", "dx", K[0, 0]), ("dx", "dy", K[0, 1]), ("dy", "dx", K[1, 0]), ("dy", "dy", K[1, 1]),
             ("id", "dx", beta[0]), ("id", "dy", beta[1])]
    a = ffgpu.varf_diffusion(kappa=None, c_stiff=0.0, terms=terms)
    (rp, cl, v), _ = _csr(a, Vh)
    # numpy: A_e[i, j] = |K| (G_i K G_j + beta . G_j / 3)   (int phi_i = |K|/3 for P1)
    Ke = meas[:, None, None] * (np.einsum("eid,dc,ejc->eij", G, K, G) + (G @ beta)[:, None, :] / 3.0)
    R = _assemble_numpy(Th, Ke)
    R.sort_indices()
    dense = np.zeros(v.size)
    rows = np.repeat(np.arange(Vh.ndof), np.diff(rp))
    dense[:] = np.asarray(R[rows, cl]).ravel()
    assert value_errors(v, dense, rp).max() <= 1e-12


def test_advection_diffusion_gmres_against_scipy():
    pytest.importorskip("scipy")
    import scipy.sparse.linalg as spl
    Th = mesh.square(24)
    Vh = FESpace(Th, "P1")
    on = (1, 2, 3, 4)
    # -div(k grad u) + (y - 0.5, 0.5 - x) . grad u + 0.1 u = exp(x), k = 1 + x^2
    terms = [("id", "dx", y - 0.5), ("id", "dy", 0.5 - x), ("id", "id", 0.1)]
    a = ffgpu.varf_diffusion(kappa=1 + x * x, f=E.exp(x), on=on, terms=terms, tgv=-1.0)
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(a, Vh, solver="GMRES", eps=1e-12, dim_krylov=60, rhs_out=b)
    rp, cl, v = A.csr()
    import scipy.sparse as sp
    M = sp.csr_matrix((v, cl, rp), shape=(Vh.ndof, Vh.ndof))
    assert abs(M - M.T).max() > 1e-3           # nonsymmetric
    u_ref = spl.spsolve(M.tocsc(), b)
    u = A.solve(b)
    assert A.stats.converged
    assert np.linalg.norm(u - u_ref) <= 1e-9 * np.linalg.norm(u_ref)


def test_expression_errors():
    Th = mesh.square(4)
    Vh = FESpace(Th, "P1")
    with pytest.raises(ValueError):
        ffgpu.varf_elasticity(f=(x, y)).c_varf(FESpace(mesh.cube(1), "P2vec"))
    # a P2 FE function without its table on a P1 space
    with pytest.raises(ffgpu.FFGPUError):
        ffgpu.matrix(ffgpu.varf_diffusion(kappa=E.fe("P2", np.ones(25))), Vh)
