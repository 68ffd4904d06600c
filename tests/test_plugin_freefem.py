"""The FreeFEM plugin compiled with FreeFEM's own ff-c++ and loaded into FreeFEM.

Needs a FreeFEM installation (FREEFEM_BIN, FREEFEM_FFCXX; defaults are the from-source build
used for the golden fixtures) and is skipped without one.  Without a GPU the device solver
must stop the script with FreeFEM's ExecError -- never fall back to a CPU solve."""
import os
import shutil
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
from paths import FF_BIN, FF_CXX, FF_LOADPATH   # oracle/paths.py

pytestmark = pytest.mark.skipif(not (os.path.exists(FF_BIN) and os.path.exists(FF_CXX)),
                                reason="FreeFEM is not installed here")

SCRIPT = r"""
load "%s"
mesh Th=square(8,8);
fespace Vh(Th,P1);
Vh u,v;
varf a(u,v)=int2d(Th,qft=qf2pT)(dx(u)*dx(v)+dy(u)*dy(v)) + int2d(Th,qft=qf2pT)(1.*v) + on(1,2,3,4,u=0);
matrix A=a(Vh,Vh,solver=GPUCG,eps=1e-10);
real[int] b=a(0,Vh);
u[]=0; u[]=A^-1*b;
cout << "umax " << u[].max << endl;
"""


@pytest.fixture(scope="module")
def plugin(tmp_path_factory):
    """The plugin compiled with FreeFEM's ff-c++ against this repository's libffgpu.so."""
    from ffgpu.build import build
    lib = build()
    d = tmp_path_factory.mktemp("plugin")
    shutil.copy(os.path.join(REPO, "freefem-sources_gb300", "plugin", "ffgpu.cpp"), d / "ffgpu.cpp")
    r = subprocess.run([FF_CXX, "-auto", "ffgpu.cpp", "-I" + os.path.join(REPO, "include"), lib],
                       cwd=d, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and (d / "ffgpu.so").exists(), r.stdout + r.stderr
    env = dict(os.environ, FF_LOADPATH=FF_LOADPATH,
               LD_LIBRARY_PATH=os.path.dirname(lib) + ":" + os.environ.get("LD_LIBRARY_PATH", ""))
    return d, env


def run_script(plugin, name, body, extra_env=None):
    d, env = plugin
    (d / name).write_text(('load "%s"\n' % str(d / "ffgpu")) + body)
    r = subprocess.run([FF_BIN, "-nw", name, "-v", "2"], cwd=d, env=dict(env, **(extra_env or {})),
                       capture_output=True, text=True, timeout=300)
    return r, r.stdout + r.stderr


def gpu_present():
    import torch
    return torch.cuda.is_available()


def test_plugin_registers_solvers_and_refuses_cpu_fallback(plugin):
    r, out = run_script(plugin, "t.edp", SCRIPT.split("\n", 2)[2])
    assert "load: ffgpu (GPUCG, GPUGMRES, GPUCGMIXED, GPUCHOLESKY, GPUSPARSESOLVER)" in out
    assert "ffgpu: device assembly P1 dim 2" in out
    if gpu_present():
        assert r.returncode == 0 and "umax 0.07" in out, out[-2000:]
    else:
        assert r.returncode != 0
        assert "ffgpu: no usable CUDA device" in out
        # (-v 2 echoes the script, so look for the printed value, not the word)
        assert not any(line.startswith("umax ") for line in r.stdout.splitlines())


P0_CUBE = r"""
load "msh3"
mesh3 Th=cube(3,3,3);
fespace Vh(Th,P1); fespace Ph(Th,P0);
Ph kappa; kappa = 1 + x + 2*y*y;
Vh u,v;
varf a(u,v)=int3d(Th)(kappa*(dx(u)*dx(v)+dy(u)*dy(v)+dz(u)*dz(v))) + on(1,2,3,4,5,6,u=0);
real s=0; for (int k=0;k<Th.nt;k++) s += kappa[][k]*(k%7+1);
cout.precision(17); cout << "ksum " << s << endl;
matrix A=a(Vh,Vh);
cout << "nnz " << A.nnz << endl;
"""

ELASTICITY = r"""
load "msh3"
mesh3 Th=cube(2,2,2);
fespace Vh(Th,[P2,P2,P2]);
Vh [u1,u2,u3],[v1,v2,v3];
real E=1, nu=0.3; real mu=E/(2*(1+nu)); real lambda=E*nu/((1+nu)*(1-2*nu));
real s2=sqrt(2.);
macro epsilon(u1,u2,u3) [dx(u1),dy(u2),dz(u3),(dz(u2)+dy(u3))/s2,(dz(u1)+dx(u3))/s2,(dy(u1)+dx(u2))/s2] // EOM
macro div(u1,u2,u3) (dx(u1)+dy(u2)+dz(u3)) // EOM
varf a([u1,u2,u3],[v1,v2,v3])=int3d(Th)(lambda*div(u1,u2,u3)*div(v1,v2,v3)+2.*mu*(epsilon(u1,u2,u3)'*epsilon(v1,v2,v3))) + int3d(Th)(-1.*v3) + on(4,u1=0,u2=0,u3=0);
matrix A=a(Vh,Vh,solver=CG,eps=1e-10);
cout << "nnz " << A.nnz << endl;
"""


def _dumped(d):
    import numpy as np
    return {k: np.fromfile(d / f"{k}.bin", dt) for k, dt in
            [("coords", np.float64), ("elems", np.int32), ("dof", np.int32), ("belems", np.int32),
             ("blabel", np.int32), ("kappa", np.float64)]}


def test_device_assembly_hook_extracts_freefem_arrays(plugin, tmp_path):
    """`matrix A = a(Vh,Vh)` on a recognised form goes to the device path; the arrays it hands
    to the C ABI equal, bit for bit, this repository's FreeFEM-order mesh and DOF builders."""
    import numpy as np
    from ffgpu import mesh
    from ffgpu.fespace import FESpace
    d1 = tmp_path / "p0"
    d1.mkdir()
    r, out = run_script(plugin, "p0.edp", P0_CUBE, {"FFGPU_PLUGIN_DUMP": str(d1)})
    ksum = [l for l in r.stdout.splitlines() if l.startswith("ksum ")][0].split()[1]
    assert f"ffgpu: device assembly P1 dim 3 nt 162 ndof 64 kappa-check {ksum} mass 0" in out
    a = _dumped(d1)
    Th = mesh.cube(3)
    Vh = FESpace(Th, "P1")
    assert np.array_equal(a["coords"], Th.coords.ravel()) and np.array_equal(a["elems"], Th.elems.ravel())
    assert np.array_equal(a["dof"], Vh.dof.ravel())
    assert np.array_equal(a["belems"], Th.belems.ravel()) and np.array_equal(a["blabel"], Th.blabel)
    bc = Th.coords[Th.elems].mean(axis=1)
    assert np.abs(a["kappa"] - (1 + bc[:, 0] + 2 * bc[:, 1] ** 2)).max() <= 1e-15
    d2 = tmp_path / "el"
    d2.mkdir()
    r, out = run_script(plugin, "el.edp", ELASTICITY, {"FFGPU_PLUGIN_DUMP": str(d2)})
    assert "ffgpu: device assembly [P2,P2,P2] dim 3 nt 48 ndof 375 lambda 0.576923 mu 0.384615" in out
    assert "components 7 labels 4" in out
    a = _dumped(d2)
    Th = mesh.cube(2)
    assert np.array_equal(a["dof"], FESpace(Th, "P2vec").dof.ravel())
    if not gpu_present():
        assert r.returncode != 0 and "ffgpu: no usable CUDA device" in out
        assert not any(line.startswith("nnz ") for line in r.stdout.splitlines())


def test_unsupported_forms_are_assembled_by_freefem(plugin):
    body = r"""
mesh Th=square(6,6);
fespace Vh(Th,P1);
Vh u,v;
fespace Wh(Th,P2);
Wh w,z;
varf a(w,z)=int2d(Th)((1+x*y)*dx(w)*dx(z)+(2+x*y)*dy(w)*dy(z)) + on(1,2,3,4,w=0);
matrix A=a(Wh,Wh);
cout << "nnzA " << A.nnz << endl;
varf b(w,z)=int2d(Th,qft=qf1pT)(dx(w)*dx(z)+dy(w)*dy(z)) + on(1,2,3,4,w=0);
matrix B=b(Wh,Wh);
cout << "nnzB " << B.nnz << endl;
fespace Bh(Th,P1b);
Bh p,q;
varf c(p,q)=int2d(Th)(dx(p)*dx(q)+dy(p)*dy(q));
matrix C=c(Bh,Bh);
cout << "nnzC " << C.nnz << endl;
varf e(u,v)=int2d(Th)(dx(u)*dy(v));
matrix D=e(Vh,Vh);
cout << "nnzD " << D.nnz << endl;
"""
    r, out = run_script(plugin, "fb.edp", body)
    assert r.returncode == 0, out[-2000:]
    for why in ("anisotropic diffusion", "quadrature not exact for the form", "element type",
                "mixed derivative term"):
        assert f"ffgpu: form assembled by FreeFEM on the CPU ({why})" in out
    nnz = {l.split()[0]: int(l.split()[1]) for l in r.stdout.splitlines() if l.startswith("nnz")}
    # square(6) P1: 7 nv - 8 n - 6 entries
    assert nnz["nnzD"] == 7 * 49 - 8 * 6 - 6


def test_strict_mode_stops_on_unsupported_form(plugin):
    """`ffgpustrict = 1;`: a form the device does not assemble is an error, not a silent CPU
    assembly."""
    body = r"""
ffgpustrict = 1;
mesh Th=square(6,6);
fespace Vh(Th,P1);
Vh u,v;
varf e(u,v)=int2d(Th)(dx(u)*dy(v));
matrix D=e(Vh,Vh);
cout << "after " << D.nnz << endl;
"""
    r, out = run_script(plugin, "strict.edp", body)
    assert r.returncode != 0
    assert "ffgpustrict" in out and "mixed derivative term" in out
    assert "after " not in r.stdout


def test_linear_form_hook(plugin):
    """`b = a(0,Vh)`: a constant/P0 source with constant on() values goes to the device
    (ffgpu_rhs_assemble); a source with an operator on v is FreeFEM's own operator."""
    body = r"""
mesh Th=square(6,6);
fespace Vh(Th,P1);
Vh u,v;
varf a(u,v)=int2d(Th)(dx(u)*dx(v)+dy(u)*dy(v)) + int2d(Th)(x*dx(v)) + on(1,2,3,4,u=0);
real[int] b=a(0,Vh);
cout << "bsum " << b.sum << endl;
varf a2(u,v)=int2d(Th)(dx(u)*dx(v)+dy(u)*dy(v)) + int2d(Th)(2.5*v) + on(1,3,u=1.5);
real[int] b2=a2(0,Vh);
cout << "b2sum " << b2.sum << endl;
"""
    r, out = run_script(plugin, "lf.edp", body)
    assert "ffgpu: linear form assembled by FreeFEM on the CPU (operator)" in out
    assert any(line.startswith("bsum ") for line in r.stdout.splitlines())
    # 72 triangles, f = 2.5: sum_k 2.5 (k % 7 + 1) = 707.5
    assert "ffgpu: device linear form P1 dim 2 f-check 707.5 g 1.5 tgv 1e+30" in out
    if not gpu_present():
        assert r.returncode != 0 and "ffgpu: no usable CUDA device" in out


@pytest.mark.parametrize("dim", [2, 3])
def test_function_sources_go_to_the_device_at_the_rule_points(plugin, tmp_path, dim):
    """A source that is a function of the point is handed to the device by its values at the
    points of the form's rule, evaluated by FreeFEM itself (checked against the same function
    at the dumped points); volume sources with different rules stay FreeFEM's."""
    if dim == 2:
        body = r"""
mesh Th=square(5,4);
fespace Vh(Th,P2);
Vh u,v;
varf a(u,v)=int2d(Th)(dx(u)*dx(v)+dy(u)*dy(v)) + int2d(Th)(sin(3*x)*y*v) + int2d(Th)(0.5*v) + on(1,u=0);
real[int] b=a(0,Vh);
"""
        f = lambda x, y: np.sin(3 * x) * y + 0.5
    else:
        body = r"""
load "msh3"
mesh3 Th=cube(3,2,2);
fespace Vh(Th,P1);
Vh u,v;
varf a(u,v)=int3d(Th)(dx(u)*dx(v)+dy(u)*dy(v)+dz(u)*dz(v)) + int3d(Th)(x*exp(z)*v) + on(1,u=0);
real[int] b=a(0,Vh);
"""
        f = lambda x, y, z: x * np.exp(z)
    d1 = tmp_path / "src"
    d1.mkdir()
    r, out = run_script(plugin, "fs.edp", body, {"FFGPU_PLUGIN_DUMP": str(d1)})
    nq = 7 if dim == 2 else 14
    assert f"at {nq} points, fq-check" in out
    X = np.fromfile(d1 / "rhs_coords.bin", np.float64).reshape(-1, dim)
    E = np.fromfile(d1 / "rhs_elems.bin", np.int32).reshape(-1, dim + 1)
    lam = np.fromfile(d1 / "rhs_lambda.bin", np.float64).reshape(nq, dim + 1)
    w = np.fromfile(d1 / "rhs_weight.bin", np.float64)
    fq = np.fromfile(d1 / "rhs_fqp.bin", np.float64).reshape(E.shape[0], nq)
    from ffgpu import quadrature
    lam_ref, w_ref = quadrature.rule(None, dim)          # FreeFEM's default rule
    assert np.allclose(lam, lam_ref, rtol=0, atol=1e-15) and np.allclose(w, w_ref, rtol=0, atol=1e-15)
    xq = quadrature.points(X, E, lam)
    ref = f(*[xq[..., k] for k in range(dim)])
    assert np.max(np.abs(fq - ref)) <= 1e-14 * np.max(np.abs(ref))
    if not gpu_present():
        assert r.returncode != 0 and "ffgpu: no usable CUDA device" in out
    body2 = r"""
mesh Th=square(4,4);
fespace Vh(Th,P1);
Vh u,v;
varf a(u,v)=int2d(Th,qft=qf2pT)(x*v) + int2d(Th)(y*v);
real[int] b=a(0,Vh);
cout << "bsum " << b.sum << endl;
"""
    r, out = run_script(plugin, "fs2.edp", body2)
    assert "ffgpu: linear form assembled by FreeFEM on the CPU (volume sources with different quadrature rules)" in out
    assert any(line.startswith("bsum ") for line in r.stdout.splitlines())


def test_p1_stiffness_with_a_p1_coefficient(plugin):
    """A coefficient linear on every element (a P1 function) in a P1 stiffness term: its mean
    over the element is its barycentre value, exactly FreeFEM's P0 interpolation of it."""
    body = r"""
mesh Th=square(6,6);
fespace Vh(Th,P1);
Vh u,v, kap = 1 + x + 2*y;
varf a(u,v)=int2d(Th)(kap*(dx(u)*dx(v)+dy(u)*dy(v))) + on(1,2,3,4,u=0);
fespace Ph(Th,P0); Ph kb = 1 + x + 2*y;
real s=0; for (int k=0;k<Th.nt;k++) s += kb[][k]*(k%7+1);
cout.precision(17); cout << "ksum " << s << endl;
matrix A=a(Vh,Vh);
"""
    r, out = run_script(plugin, "p1k.edp", body)
    ksum = float([l for l in r.stdout.splitlines() if l.startswith("ksum ")][0].split()[1])
    line = [l for l in out.splitlines() if "ffgpu: device assembly P1 dim 2 nt 72 ndof 49 kappa-check" in l][0]
    assert abs(float(line.split("kappa-check ")[1].split()[0]) - ksum) <= 1e-13 * abs(ksum)


def test_p1_stiffness_with_any_coefficient_uses_the_rule_average(plugin, tmp_path):
    """A P1 stiffness coefficient of any form (here exp(x+y)) enters as its average by the
    form's quadrature rule (default T_5 on triangles), exactly the weighted sum FreeFEM forms."""
    import numpy as np
    from ffgpu import mesh
    body = r"""
mesh Th=square(6,6);
fespace Vh(Th,P1);
Vh u,v;
varf a(u,v)=int2d(Th)(exp(x+y)*(dx(u)*dx(v)+dy(u)*dy(v))) + on(1,2,3,4,u=0);
matrix A=a(Vh,Vh);
"""
    d1 = tmp_path / "ek"
    d1.mkdir()
    r, out = run_script(plugin, "ek.edp", body, {"FFGPU_PLUGIN_DUMP": str(d1)})
    assert "ffgpu: device assembly P1 dim 2 nt 72" in out, out[-2000:]
    kap = np.fromfile(d1 / "kappa.bin", np.float64)
    Th = mesh.square(6)
    s15 = np.sqrt(15.0)
    t, r1, s1, u1, v1 = 1 / 3, (6 - s15) / 21, (9 + 2 * s15) / 21, (6 + s15) / 21, (9 - 2 * s15) / 21
    P = np.array([[t, t], [r1, r1], [r1, s1], [s1, r1], [u1, u1], [u1, v1], [v1, u1]])
    W = np.array([0.225] + [(155 - s15) / 1200] * 3 + [(155 + s15) / 1200] * 3)
    X = Th.coords[Th.elems]                                  # (nt, 3, 2)
    lam = np.stack([1 - P[:, 0] - P[:, 1], P[:, 0], P[:, 1]], axis=1)   # (7, 3)
    xq = np.einsum("qi,kid->kqd", lam, X)
    want = (np.exp(xq[..., 0] + xq[..., 1]) * W).sum(axis=1)
    assert np.abs(kap - want).max() <= 1e-14 * want.max()


def test_boundary_terms_in_the_device_hook(plugin, tmp_path):
    """int1d / boundary int2d terms: Robin c*u*v into the device matrix, g*v into the device
    linear form, per boundary element in FreeFEM's boundary order (checksums below); terms the
    device does not assemble stay FreeFEM's."""
    import numpy as np
    from ffgpu import mesh
    body = r"""
mesh Th=square(6,6);
fespace Vh(Th,P1);
Vh u,v;
varf a(u,v)=int2d(Th)(dx(u)*dx(v)+dy(u)*dy(v)) + int1d(Th,3)(2.5*u*v) + int2d(Th)(1.*v) + int1d(Th,2)((1+y)*v) + on(1,4,u=0);
matrix A=a(Vh,Vh);
"""
    d1 = tmp_path / "bt"
    d1.mkdir()
    r, out = run_script(plugin, "bt.edp", body, {"FFGPU_PLUGIN_DUMP": str(d1)})
    Th = mesh.square(6)
    w = np.arange(Th.nbe) % 7 + 1
    rob = np.where(Th.blabel == 3, 2.5, 0.0)
    assert f"| robin-check {'%.17g' % (rob * w).sum()} on 3" in out, out[-3000:]
    assert np.array_equal(np.fromfile(d1 / "robin0.bin", np.float64), rob)
    if not gpu_present():
        assert r.returncode != 0 and "ffgpu: no usable CUDA device" in out
    # the linear form: g = 1 + y is not constant on the right edges -> FreeFEM; 1 + x is
    body2 = r"""
mesh Th=square(6,6);
fespace Vh(Th,P1);
Vh u,v;
varf a(u,v)=int2d(Th)(dx(u)*dx(v)+dy(u)*dy(v)) + int2d(Th)(1.*v) + int1d(Th,2)((1+y)*v) + on(1,4,u=0);
real[int] b=a(0,Vh);
varf a2(u,v)=int2d(Th)(dx(u)*dx(v)+dy(u)*dy(v)) + int2d(Th)(1.*v) + int1d(Th,2)((1+x)*v) + int1d(Th,3)((2+y)*v) + on(1,4,u=0);
real[int] b2=a2(0,Vh);
"""
    r, out = run_script(plugin, "bt2.edp", body2)
    assert "ffgpu: linear form assembled by FreeFEM on the CPU (boundary source not constant on boundary elements)" in out
    # right edges (x = 1): 1 + x = 2; top edges (y = 1): 2 + y = 3
    g2 = np.where(Th.blabel == 2, 2.0, 0.0)
    g3 = np.where(Th.blabel == 3, 3.0, 0.0)
    assert (f"| g-check {'%.17g' % (g2 * w).sum()} on 2 | g-check {'%.17g' % (g3 * w).sum()} on 3" in out), out[-3000:]


def test_boundary_terms_3d_and_rejections(plugin):
    import numpy as np
    from ffgpu import mesh
    body = r"""
load "msh3"
mesh3 Th=cube(3,3,2);
fespace Vh(Th,P2);
Vh u,v;
varf a(u,v)=int3d(Th)(dx(u)*dx(v)+dy(u)*dy(v)+dz(u)*dz(v)) + int2d(Th,2)(2.*u*v) + on(4,u=0);
matrix A=a(Vh,Vh);
"""
    r, out = run_script(plugin, "bt3.edp", body)
    Th = mesh.cube(3, 3, 2)
    w = np.arange(Th.nbe) % 7 + 1
    rob = np.where(Th.blabel == 2, 2.0, 0.0)
    assert "ffgpu: device assembly P2 dim 3" in out and f"| robin-check {'%.17g' % (rob * w).sum()} on 2" in out
    body2 = r"""
mesh Th=square(6,6);
fespace Vh(Th,P1);
Vh u,v;
varf a(u,v)=int2d(Th)(dx(u)*dx(v)+dy(u)*dy(v)) + int1d(Th,2)(dx(u)*v) + on(1,4,u=0);
matrix A=a(Vh,Vh);
cout << "nnzA " << A.nnz << endl;
varf a2(u,v)=int2d(Th)(dx(u)*dx(v)+dy(u)*dy(v)) + int1d(Th,2,qfe=qf1pE)(u*v) + on(1,4,u=0);
matrix A2=a2(Vh,Vh);
cout << "nnzA2 " << A2.nnz << endl;
"""
    r, out = run_script(plugin, "bt4.edp", body2)
    assert r.returncode == 0, out[-2000:]
    assert "ffgpu: form assembled by FreeFEM on the CPU (boundary term other than c*u*v)" in out
    assert "ffgpu: form assembled by FreeFEM on the CPU (boundary quadrature not exact)" in out


def test_p2_with_a_mass_term_goes_to_the_device(plugin):
    body = r"""
mesh Th=square(5,5);
fespace Vh(Th,P2);
Vh u,v;
varf a(u,v)=int2d(Th)(dx(u)*dx(v)+dy(u)*dy(v)+2.5*u*v) + on(1,2,3,4,u=0);
matrix A=a(Vh,Vh);
"""
    r, out = run_script(plugin, "p2m.edp", body)
    assert "ffgpu: device assembly P2 dim 2 nt 50" in out and " mass 2.5 " in out, out[-2000:]
    if not gpu_present():
        assert r.returncode != 0 and "ffgpu: no usable CUDA device" in out


@pytest.mark.parametrize("dim", [2, 3])
def test_mass_coefficient_functions_go_to_the_device_at_the_rule_points(plugin, tmp_path, dim):
    """A mass coefficient that depends on the point (a function, or P0) is handed to the device
    by FreeFEM's own values at the points of the form's rule; constant mass terms join them."""
    if dim == 2:
        body = r"""
mesh Th=square(5,4);
fespace Vh(Th,P2);
Vh u,v;
varf a(u,v)=int2d(Th)(dx(u)*dx(v)+dy(u)*dy(v)) + int2d(Th)((1+x*y)*u*v) + int2d(Th)(0.25*u*v) + on(1,u=0);
matrix A=a(Vh,Vh,solver=GPUCG);
"""
        c = lambda x, y: 1 + x * y + 0.25
    else:
        body = r"""
load "msh3"
mesh3 Th=cube(2,2,2);
fespace Vh(Th,P1);
Vh u,v;
varf a(u,v)=int3d(Th)(dx(u)*dx(v)+dy(u)*dy(v)+dz(u)*dz(v)) + int3d(Th)(exp(z)*u*v) + on(1,u=0);
matrix A=a(Vh,Vh,solver=GPUCG);
"""
        c = lambda x, y, z: np.exp(z)
    d1 = tmp_path / "mq"
    d1.mkdir()
    r, out = run_script(plugin, "mq.edp", body, {"FFGPU_PLUGIN_DUMP": str(d1)})
    nq = 7 if dim == 2 else 14
    assert f"mass at {nq} points, mq-check" in out
    X = np.fromfile(d1 / "coords.bin", np.float64).reshape(-1, dim)
    E = np.fromfile(d1 / "elems.bin", np.int32).reshape(-1, dim + 1)
    mq = np.fromfile(d1 / "mass_qp.bin", np.float64).reshape(E.shape[0], nq)
    from ffgpu import quadrature
    lam, _ = quadrature.rule(None, dim)
    xq = quadrature.points(X, E, lam)
    ref = c(*[xq[..., k] for k in range(dim)])
    assert np.max(np.abs(mq - ref)) <= 1e-14 * np.max(np.abs(ref))
    if not gpu_present():
        assert r.returncode != 0 and "ffgpu: no usable CUDA device" in out


def test_p2_stiffness_function_goes_to_the_device_at_the_rule_points(plugin, tmp_path):
    """A P2 stiffness coefficient that depends on the point goes to the device by FreeFEM's
    values at the rule's points; a P0 part of the same form joins them."""
    body = r"""
mesh Th=square(5,4);
fespace Vh(Th,P2);
fespace Ph(Th,P0);
Ph k0=1+x;
Vh u,v;
varf a(u,v)=int2d(Th)(exp(x-y)*(dx(u)*dx(v)+dy(u)*dy(v))) + int2d(Th)(k0*(dx(u)*dx(v)+dy(u)*dy(v))) + on(1,u=0);
matrix A=a(Vh,Vh,solver=GPUCG);
"""
    d1 = tmp_path / "kq"
    d1.mkdir()
    r, out = run_script(plugin, "kq.edp", body, {"FFGPU_PLUGIN_DUMP": str(d1)})
    assert "stiffness at 7 points, kq-check" in out
    X = np.fromfile(d1 / "coords.bin", np.float64).reshape(-1, 2)
    E = np.fromfile(d1 / "elems.bin", np.int32).reshape(-1, 3)
    kq = np.fromfile(d1 / "stiff_qp.bin", np.float64).reshape(E.shape[0], 7)
    from ffgpu import quadrature
    lam, _ = quadrature.rule(None, 2)
    xq = quadrature.points(X, E, lam)
    centre = X[E].mean(axis=1)[:, 0]                    # the P0 function 1+x, at the centroid
    ref = np.exp(xq[..., 0] - xq[..., 1]) + (1 + centre)[:, None]
    assert np.max(np.abs(kq - ref)) <= 1e-13 * np.max(np.abs(ref))
    if not gpu_present():
        assert r.returncode != 0 and "ffgpu: no usable CUDA device" in out


def test_solve_and_problem_statements_use_the_gpu_solver(plugin):
    """solve / problem with solver=GPUCG go to the registered device solver (FreeFEM assembles
    the problem form itself); set(A, solver=GPUCG) rebinds a matrix to it."""
    body = r"""
mesh Th=square(10,10);
fespace Vh(Th,P1);
Vh u,v;
solve pb(u,v,solver=GPUCG,eps=1e-10)=int2d(Th)(dx(u)*dx(v)+dy(u)*dy(v)) - int2d(Th)(1.*v) + on(1,2,3,4,u=0);
cout << "umax " << u[].max << endl;
"""
    r, out = run_script(plugin, "sv.edp", body)
    if gpu_present():
        assert r.returncode == 0 and "umax " in r.stdout, out[-2000:]
    else:
        assert r.returncode != 0 and "ffgpu: no usable CUDA device" in out, out[-2000:]
        assert not any(line.startswith("umax ") for line in r.stdout.splitlines())
    body2 = r"""
mesh Th=square(10,10);
fespace Vh(Th,P1);
Vh u,v;
varf a(u,v)=int2d(Th)(dx(u)*dx(v)+dy(u)*dy(v)) + int2d(Th)(1.*v) + on(1,2,3,4,u=0);
matrix A=a(Vh,Vh);
set(A,solver=GPUCG,eps=1e-10);
real[int] b=a(0,Vh);
u[]=A^-1*b;
cout << "umax " << u[].max << endl;
"""
    r, out = run_script(plugin, "st.edp", body2)
    if gpu_present():
        assert r.returncode == 0 and "umax " in r.stdout, out[-2000:]
    else:
        assert r.returncode != 0 and "ffgpu: no usable CUDA device" in out, out[-2000:]
