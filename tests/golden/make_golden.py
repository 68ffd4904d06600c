"""Generate the golden fixtures of the assemble-and-solve path by running FreeFEM itself.

The fixtures under ``tests/golden/*.npz`` are outputs of the FreeFEM 4.15 interpreter
(``FreeFem++-nw``, built from the FreeFEM sources) on small seeded inputs.  Each case
writes an ``.edp`` script, runs it, and parses tagged lines from its stdout:

  V  vertex coordinates (and vertex label)      -> ``coords``, ``vlabel``
  T  element vertex indices (mesh order)        -> ``elems``
  B  boundary elements and their labels         -> ``belems``, ``blabel``
  D  element -> global DOF table  (``Vh(k,i)``)  -> ``dof``
  A  sorted COO of the matrix (``[I,J,C]=A``)   -> ``I``, ``J``, ``C``
  b  right-hand side and solution               -> ``b``, ``u``
  S  scalars (iteration counts, norms)           -> ``scalars`` (name -> value)
  G  extra per-element / per-DOF vectors          -> by name

The inputs that are random (P0 coefficients, observation noise, mesh jitter) are drawn
here with numpy ``PCG64`` seeds and written to text files the script reads, so the
fixture holds the exact inputs too.

Run (in a container where FreeFEM is available)::

    FREEFEM_BIN=/path/to/FreeFem++-nw FF_LOADPATH=/path/to/plugin/seq \
        python tests/golden/make_golden.py

The test suite only reads the ``.npz`` files; it never runs FreeFEM.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle"))
from paths import FF_BIN, FF_LOADPATH   # noqa: E402  (oracle/paths.py)

# ---------------------------------------------------------------- edp fragments
DUMP_MESH2 = r"""
for (int i=0;i<Th.nv;i++) cout << "V " << Th(i).x << " " << Th(i).y << " " << Th(i).label << endl;
for (int k=0;k<Th.nt;k++) cout << "T " << Th[k][0] << " " << Th[k][1] << " " << Th[k][2] << endl;
for (int k=0;k<Th.nbe;k++) cout << "B " << Th.be(k)[0] << " " << Th.be(k)[1] << " " << Th.be(k).label << endl;
"""
DUMP_MESH3 = r"""
for (int i=0;i<Th.nv;i++) cout << "V " << Th(i).x << " " << Th(i).y << " " << Th(i).z << " " << Th(i).label << endl;
for (int k=0;k<Th.nt;k++) cout << "T " << Th[k][0] << " " << Th[k][1] << " " << Th[k][2] << " " << Th[k][3] << endl;
for (int k=0;k<Th.nbe;k++) cout << "B " << Th.be(k)[0] << " " << Th.be(k)[1] << " " << Th.be(k)[2] << " " << Th.be(k).label << endl;
"""
DUMP_DOF = r"""
for (int k=0;k<Th.nt;k++){ cout << "D"; for(int i=0;i<Vh.ndofK;i++) cout << " " << Vh(k,i); cout << endl;}
"""
DUMP_A = r"""
{ int[int] I(1),J(1); real[int] C(1); [I,J,C]=A;
  for (int k=0;k<I.n;k++) cout << "A " << I[k] << " " << J[k] << " " << C[k] << endl; }
"""
HEAD = "cout.precision(17);\n"


def read_vec_edp(name: str, fname: str, n: str) -> str:
    return (f"real[int] {name}({n}); {{ ifstream ff(\"{fname}\"); "
            f"for (int k=0;k<{n};k++) ff >> {name}[k]; }}\n")


# ---------------------------------------------------------------- cases
def case_p1_square(n, m=None, qft="qft=qf2pT", solver="CG"):
    m = n if m is None else m
    body = HEAD + f"""
mesh Th=square({n},{m});
fespace Vh(Th,P1);
Vh u,v;
varf a(u,v)=int2d(Th,{qft})(dx(u)*dx(v)+dy(u)*dy(v)) + int2d(Th,{qft})(1.*v) + on(1,2,3,4,u=0);
int nit=0;
matrix A=a(Vh,Vh,solver={solver},eps=1e-10,getnbiteration=nit);
real[int] b=a(0,Vh);
u[]=0; u[]=A^-1*b;
cout << "S nit " << nit << endl;
cout << "S umax " << u[].max << endl;
cout << "S l2 " << sqrt(u[]'*u[]) << endl;
""" + DUMP_MESH2 + DUMP_DOF + DUMP_A + \
        "for (int k=0;k<b.n;k++) cout << \"b \" << b[k] << \" \" << u[][k] << endl;\n"
    return body, {}


def case_p1_square_tgv(n, tgv, solver):
    """P1 Poisson with non-zero Dirichlet data u = x on all sides, for the tgv < 0 variants of
    HashMatrix::SetBC (-1: unit diagonal, row zeroed; -2: also the column; -3: column only)."""
    body = HEAD + f"""
mesh Th=square({n},{n});
fespace Vh(Th,P1);
Vh u,v;
varf a(u,v)=int2d(Th,qft=qf2pT)(dx(u)*dx(v)+dy(u)*dy(v)) + int2d(Th,qft=qf2pT)(1.*v) + on(1,2,3,4,u=x);
int nit=0;
matrix A=a(Vh,Vh,solver={solver},eps=1e-12,tgv={tgv},getnbiteration=nit);
real[int] b=a(0,Vh,tgv={tgv});
u[]=0; u[]=A^-1*b;
cout << "S nit " << nit << endl;
""" + DUMP_MESH2 + DUMP_DOF + DUMP_A + \
        "for (int k=0;k<b.n;k++) cout << \"b \" << b[k] << \" \" << u[][k] << endl;\n"
    return body, {}


def case_p1_square_kappa(n, seed, jitter=0.0):
    """2D P1 diffusion with a P0 lognormal coefficient, default quadrature, optional jitter."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nt = 2 * n * n
    nv = (n + 1) * (n + 1)
    kap = np.exp(rng.standard_normal(nt))
    jit = rng.uniform(-jitter / n, jitter / n, size=(nv, 2))
    ij = np.array([(i, j) for j in range(n + 1) for i in range(n + 1)])
    border = (ij[:, 0] == 0) | (ij[:, 0] == n) | (ij[:, 1] == 0) | (ij[:, 1] == n)
    jit[border] = 0.0
    files = {"kappa.txt": kap, "jx.txt": jit[:, 0], "jy.txt": jit[:, 1]}
    body = HEAD + f"""
mesh Th0=square({n},{n});
fespace Vh0(Th0,P1);
""" + read_vec_edp("jxa", "jx.txt", "Th0.nv") + read_vec_edp("jya", "jy.txt", "Th0.nv") + """
Vh0 jx, jy; jx[]=jxa; jy[]=jya;
mesh Th=movemesh(Th0,[x+jx,y+jy]);
fespace Vh(Th,P1); fespace Ph(Th,P0);
""" + read_vec_edp("kapa", "kappa.txt", "Th.nt") + """
Ph kappa; kappa[]=kapa;
Vh u,v;
varf a(u,v)=int2d(Th)(kappa*(dx(u)*dx(v)+dy(u)*dy(v))) + int2d(Th)(1.*v) + on(1,2,3,4,u=0);
int nit=0;
matrix A=a(Vh,Vh,solver=CG,eps=1e-10,getnbiteration=nit);
real[int] b=a(0,Vh);
u[]=0; u[]=A^-1*b;
cout << "S nit " << nit << endl;
for (int k=0;k<Th.nt;k++) cout << "G p0dof " << Ph(k,0) << endl;
""" + DUMP_MESH2 + DUMP_DOF + DUMP_A + \
        "for (int k=0;k<b.n;k++) cout << \"b \" << b[k] << \" \" << u[][k] << endl;\n"
    return body, files


def case_p1_cube_kappa(n, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    nt = 6 * n ** 3
    kap = np.exp(rng.standard_normal(nt))
    body = HEAD + f"""
load "msh3"
mesh3 Th=cube({n},{n},{n});
fespace Vh(Th,P1); fespace Ph(Th,P0);
""" + read_vec_edp("kapa", "kappa.txt", "Th.nt") + """
Ph kappa; kappa[]=kapa;
Vh u,v;
varf a(u,v)=int3d(Th)(kappa*(dx(u)*dx(v)+dy(u)*dy(v)+dz(u)*dz(v))) + int3d(Th)(1.*v) + on(1,2,3,4,5,6,u=0);
int nit=0;
matrix A=a(Vh,Vh,solver=CG,eps=1e-10,getnbiteration=nit);
real[int] b=a(0,Vh);
u[]=0; u[]=A^-1*b;
cout << "S nit " << nit << endl;
for (int k=0;k<Th.nt;k++) cout << "G p0dof " << Ph(k,0) << endl;
""" + DUMP_MESH3 + DUMP_DOF + DUMP_A + \
        "for (int k=0;k<b.n;k++) cout << \"b \" << b[k] << \" \" << u[][k] << endl;\n"
    return body, {"kappa.txt": kap}


def case_p2_cube_scalar(n):
    body = HEAD + f"""
load "msh3"
mesh3 Th=cube({n},{n},{n});
fespace Vh(Th,P2);
Vh u,v;
varf a(u,v)=int3d(Th)(dx(u)*dx(v)+dy(u)*dy(v)+dz(u)*dz(v)) + int3d(Th)(1.*v) + on(1,2,3,4,5,6,u=0);
int nit=0;
matrix A=a(Vh,Vh,solver=CG,eps=1e-10,getnbiteration=nit);
real[int] b=a(0,Vh);
u[]=0; u[]=A^-1*b;
cout << "S nit " << nit << endl;
""" + DUMP_MESH3 + DUMP_DOF + DUMP_A + \
        "for (int k=0;k<b.n;k++) cout << \"b \" << b[k] << \" \" << u[][k] << endl;\n"
    return body, {}


def case_p2_elasticity_materials(nx, ny, nz, seed):
    """[P2,P2,P2] elasticity with per-element E and nu (two materials, seeded): P0 Lame
    coefficients mu = E/(2(1+nu)), lambda = E nu/((1+nu)(1-2nu))."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nt = 6 * nx * ny * nz
    Ea = np.where(rng.random(nt) < 0.5, 1.0, 10.0)
    na = np.where(rng.random(nt) < 0.5, 0.25, 0.35)
    files = {"E.txt": Ea, "nu.txt": na}
    body = HEAD + f"""
load "msh3"
mesh3 Th=cube({nx},{ny},{nz});
fespace Vh(Th,[P2,P2,P2]);
fespace Ph(Th,P0);
""" + read_vec_edp("Ea", "E.txt", "Th.nt") + read_vec_edp("na", "nu.txt", "Th.nt") + """
Ph Ek, nuk; Ek[]=Ea; nuk[]=na;
Ph mu=Ek/(2*(1+nuk)), lambda=Ek*nuk/((1+nuk)*(1-2*nuk));
Vh [u1,u2,u3],[v1,v2,v3];
real s2=sqrt(2.);
macro epsilon(u1,u2,u3) [dx(u1),dy(u2),dz(u3),(dz(u2)+dy(u3))/s2,(dz(u1)+dx(u3))/s2,(dy(u1)+dx(u2))/s2] // EOM
macro div(u1,u2,u3) (dx(u1)+dy(u2)+dz(u3)) // EOM
varf a([u1,u2,u3],[v1,v2,v3])=int3d(Th)(lambda*div(u1,u2,u3)*div(v1,v2,v3)+2.*mu*(epsilon(u1,u2,u3)'*epsilon(v1,v2,v3))) + int3d(Th)(-1.*v3) + on(4,u1=0,u2=0,u3=0);
int nit=0;
matrix A=a(Vh,Vh,solver=CG,eps=1e-10,getnbiteration=nit);
real[int] b=a(0,Vh);
u1[]=0; u1[]=A^-1*b;
cout << "S nit " << nit << endl;
""" + DUMP_MESH3 + DUMP_DOF + DUMP_A + \
        "for (int k=0;k<b.n;k++) cout << \"b \" << b[k] << \" \" << u1[][k] << endl;\n"
    return body, files


def case_p2_elasticity(nx, ny, nz):
    body = HEAD + f"""
load "msh3"
mesh3 Th=cube({nx},{ny},{nz});
fespace Vh(Th,[P2,P2,P2]);
Vh [u1,u2,u3],[v1,v2,v3];
real E=1, nu=0.3; real mu=E/(2*(1+nu)); real lambda=E*nu/((1+nu)*(1-2*nu));
real s2=sqrt(2.);
macro epsilon(u1,u2,u3) [dx(u1),dy(u2),dz(u3),(dz(u2)+dy(u3))/s2,(dz(u1)+dx(u3))/s2,(dy(u1)+dx(u2))/s2] // EOM
macro div(u1,u2,u3) (dx(u1)+dy(u2)+dz(u3)) // EOM
varf a([u1,u2,u3],[v1,v2,v3])=int3d(Th)(lambda*div(u1,u2,u3)*div(v1,v2,v3)+2.*mu*(epsilon(u1,u2,u3)'*epsilon(v1,v2,v3))) + int3d(Th)(-1.*v3) + on(4,u1=0,u2=0,u3=0);
int nit=0;
matrix A=a(Vh,Vh,solver=CG,eps=1e-10,getnbiteration=nit);
real[int] b=a(0,Vh);
u1[]=0; u1[]=A^-1*b;
cout << "S nit " << nit << endl;
""" + DUMP_MESH3 + DUMP_DOF + DUMP_A + \
        "for (int k=0;k<b.n;k++) cout << \"b \" << b[k] << \" \" << u1[][k] << endl;\n"
    return body, {}


def case_p2_mass(dim, n):
    """P2 stiffness plus a mass term 2.5*u*v (default quadrature, exact for the degree-4 mass)."""
    if dim == 3:
        head = f'load "msh3"\nmesh3 Th=cube({n},{n},{n});\n'
        form = "int3d(Th)(dx(u)*dx(v)+dy(u)*dy(v)+dz(u)*dz(v)+2.5*u*v) + int3d(Th)(1.*v) + on(1,2,3,4,5,6,u=0)"
        dump = DUMP_MESH3
    else:
        head = f"mesh Th=square({n},{n});\n"
        form = "int2d(Th)(dx(u)*dx(v)+dy(u)*dy(v)+2.5*u*v) + int2d(Th)(1.*v) + on(1,2,3,4,u=0)"
        dump = DUMP_MESH2
    body = HEAD + head + f"""
fespace Vh(Th,P2);
Vh u,v;
varf a(u,v)={form};
int nit=0;
matrix A=a(Vh,Vh,solver=CG,eps=1e-10,getnbiteration=nit);
real[int] b=a(0,Vh);
u[]=0; u[]=A^-1*b;
cout << "S nit " << nit << endl;
""" + dump + DUMP_DOF + DUMP_A + \
        "for (int k=0;k<b.n;k++) cout << \"b \" << b[k] << \" \" << u[][k] << endl;\n"
    return body, {}


def case_p2_square_scalar(n):
    """2D P2: FreeFEM renumbers the P2 nodes (Gibbs); the fixture carries its DOF table."""
    body = HEAD + f"""
mesh Th=square({n},{n});
fespace Vh(Th,P2);
Vh u,v;
varf a(u,v)=int2d(Th)(dx(u)*dx(v)+dy(u)*dy(v)) + int2d(Th)(1.*v) + on(1,2,3,4,u=0);
int nit=0;
matrix A=a(Vh,Vh,solver=CG,eps=1e-10,getnbiteration=nit);
real[int] b=a(0,Vh);
u[]=0; u[]=A^-1*b;
cout << "S nit " << nit << endl;
""" + DUMP_MESH2 + DUMP_DOF + DUMP_A + \
        "for (int k=0;k<b.n;k++) cout << \"b \" << b[k] << \" \" << u[][k] << endl;\n"
    return body, {}


P2NUM_MESHES = {
    # structured, unstructured (Delaunay), with a hole, two components, a truncated square
    "sq7x3": "mesh Th=square(7,3);",
    "disk": "border C(t=0,2*pi){x=cos(t);y=sin(t);label=1;}\nmesh Th=buildmesh(C(24));",
    "annulus": ("border a(t=0,2*pi){x=2*cos(t);y=2*sin(t);label=1;}\n"
                "border c(t=0,2*pi){x=cos(t);y=sin(t);label=2;}\nmesh Th=buildmesh(a(30)+c(-15));"),
    "two": "mesh Th1=square(3,3);\nmesh Th2=square(2,4,[x+2,y]);\nmesh Th=Th1+Th2;",
    "lshape": "mesh Th=trunc(square(8,8),(x<0.5)|(y<0.5));",
    "disk80": "border C(t=0,2*pi){x=cos(t);y=sin(t);label=1;}\nmesh Th=buildmesh(C(80));",
}


def case_p2_numbering(which):
    """FreeFEM's 2D P2 DOF table (ConstructDataFElement::Make + Gibbs renumbering) on a mesh."""
    body = HEAD + P2NUM_MESHES[which] + "\nfespace Vh(Th,P2);\n" + DUMP_MESH2 + DUMP_DOF
    return body, {}


# sources given as functions of the coordinates (taken at the points of the form's rule)
SOURCE_CASES = {
    "sq_p1": ("mesh Th=square(6,5);", "P1", "int2d(Th)", "sin(3*x)*cos(2*y)+x*y", None),
    "sq_p1_qf2": ("mesh Th=square(5,4);", "P1", "int2d(Th,qft=qf2pT)", "exp(x)*(1+y*y)", None),
    "sq_p2": ("mesh Th=square(4,3);", "P2", "int2d(Th)", "exp(x)*y-cos(5*y)", None),
    "cube_p1": ("mesh3 Th=cube(3,2,2);", "P1", "int3d(Th)", "x*y*z+sin(2*z)", None),
    "cube_p2": ("mesh3 Th=cube(2,2,1);", "P2", "int3d(Th)", "cos(x+2*y)*z", None),
    "cube_el": ("mesh3 Th=cube(2,1,1);", "P2vec", "int3d(Th)", None, ("x", "y*z", "-1+x*x")),
}


def case_source_function(which):
    """b = a(0,Vh) for a source that is a function of the coordinates: FreeFEM evaluates it at
    the points of the rule (Element_rhs)."""
    mesh_line, kind, dom, f, fv = SOURCE_CASES[which]
    dump = DUMP_MESH3 if "mesh3" in mesh_line else DUMP_MESH2
    if kind == "P2vec":
        body = HEAD + "load \"msh3\"\n" + mesh_line + f"""
fespace Vh(Th,[P2,P2,P2]);
Vh [u1,u2,u3],[v1,v2,v3];
varf a([u1,u2,u3],[v1,v2,v3])={dom}(({fv[0]})*v1+({fv[1]})*v2+({fv[2]})*v3);
real[int] b=a(0,Vh);
"""
    else:
        load = "load \"msh3\"\n" if "mesh3" in mesh_line else ""
        body = HEAD + load + mesh_line + f"""
fespace Vh(Th,{kind});
Vh u,v;
varf a(u,v)={dom}(({f})*v);
real[int] b=a(0,Vh);
"""
    body += dump + DUMP_DOF + "for (int k=0;k<b.n;k++) cout << \"b \" << b[k] << \" 0\" << endl;\n"
    return body, {}


# mass coefficients that are functions of the point (taken at the points of the form's rule)
MASS_CASES = {
    "sq_p1": ("mesh Th=square(5,4);", "P1", "int2d(Th)", "1+x*y", "1"),
    "sq_p2": ("mesh Th=square(4,3);", "P2", "int2d(Th)", "exp(x+y)", "1,2"),
    "cube_p1": ("mesh3 Th=cube(2,2,2);", "P1", "int3d(Th)", "1+z*x", "1"),
    "cube_p2": ("mesh3 Th=cube(2,1,1);", "P2", "int3d(Th)", "2+cos(x)*y", "1"),
}


# stiffness coefficients that are functions of the point
STIFF_CASES = {
    "sq_p1": ("mesh Th=square(5,4);", "P1", "int2d(Th)", "1+x*x*y", "1,3"),
    "sq_p2": ("mesh Th=square(4,3);", "P2", "int2d(Th)", "exp(x-y)", "1,2"),
    "cube_p2": ("mesh3 Th=cube(2,2,1);", "P2", "int3d(Th)", "1+x*y*z", "1,2"),
}


def case_stiff_function(which):
    """-div(k grad u) = 1 with k a function of the point: FreeFEM's matrix, b and u."""
    mesh_line, kind, dom, k, labels = STIFF_CASES[which]
    three = "mesh3" in mesh_line
    grad = "dx(u)*dx(v)+dy(u)*dy(v)" + ("+dz(u)*dz(v)" if three else "")
    body = HEAD + ("load \"msh3\"\n" if three else "") + mesh_line + f"""
fespace Vh(Th,{kind});
Vh u,v;
varf a(u,v)={dom}(({k})*({grad})) + {dom}(1.*v) + on({labels},u=0);
int nit=0;
matrix A=a(Vh,Vh,solver=CG,eps=1e-12,getnbiteration=nit);
real[int] b=a(0,Vh);
u[]=0; u[]=A^-1*b;
cout << "S nit " << nit << endl;
""" + (DUMP_MESH3 if three else DUMP_MESH2) + DUMP_DOF + DUMP_A + \
        "for (int k=0;k<b.n;k++) cout << \"b \" << b[k] << \" \" << u[][k] << endl;\n"
    return body, {}


def case_mass_function(which):
    """-div grad u + c(x) u = 1 with c a function of the point: FreeFEM's matrix, b and u."""
    mesh_line, kind, dom, c, labels = MASS_CASES[which]
    three = "mesh3" in mesh_line
    grad = "dx(u)*dx(v)+dy(u)*dy(v)" + ("+dz(u)*dz(v)" if three else "")
    body = HEAD + ("load \"msh3\"\n" if three else "") + mesh_line + f"""
fespace Vh(Th,{kind});
Vh u,v;
varf a(u,v)={dom}({grad}) + {dom}(({c})*u*v) + {dom}(1.*v) + on({labels},u=0);
int nit=0;
matrix A=a(Vh,Vh,solver=CG,eps=1e-12,getnbiteration=nit);
real[int] b=a(0,Vh);
u[]=0; u[]=A^-1*b;
cout << "S nit " << nit << endl;
""" + (DUMP_MESH3 if three else DUMP_MESH2) + DUMP_DOF + DUMP_A + \
        "for (int k=0;k<b.n;k++) cout << \"b \" << b[k] << \" \" << u[][k] << endl;\n"
    return body, {}


def case_adjoint_p1(n, seed):
    """FP64 adjoint of L = 1/2 (u-uobs)' M (u-uobs) for -div(kappa grad u) = f, written as
    a FreeFEM script: forward CG solve, transpose solve A'^-1, P0 sensitivities by a varf."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nt = 2 * n * n
    nv = (n + 1) * (n + 1)
    kap = np.exp(0.3 * rng.standard_normal(nt))
    fsrc = 1.0 + 0.5 * rng.standard_normal(nt)
    uobs = 0.05 * rng.standard_normal(nv)
    files = {"kappa.txt": kap, "f.txt": fsrc, "uobs.txt": uobs}
    body = HEAD + f"""
mesh Th=square({n},{n});
fespace Vh(Th,P1); fespace Ph(Th,P0);
""" + read_vec_edp("kapa", "kappa.txt", "Th.nt") + read_vec_edp("fa", "f.txt", "Th.nt") + \
        read_vec_edp("uoa", "uobs.txt", "Th.nv") + """
Ph kappa, fs; kappa[]=kapa; fs[]=fa;
Vh uobs; uobs[]=uoa;
Vh u,v;
varf a(u,v)=int2d(Th)(kappa*(dx(u)*dx(v)+dy(u)*dy(v))) + int2d(Th)(fs*v) + on(1,2,3,4,u=0);
int nit=0;
matrix A=a(Vh,Vh,solver=CG,eps=1e-14,getnbiteration=nit);
real[int] b=a(0,Vh);
u[]=0; u[]=A^-1*b;
cout << "S nit " << nit << endl;
varf m(u,v)=int2d(Th)(u*v);
matrix M=m(Vh,Vh);
real[int] r=u[]; r-=uobs[];
real[int] Mr=M*r;
real L=0.5*(r'*Mr);
cout << "S loss " << L << endl;
Vh lam; lam[]=0; lam[]=A'^-1*Mr;
varf gk(unused,w)=int2d(Th)(-(dx(lam)*dx(u)+dy(lam)*dy(u))*w);
varf gf(unused,w)=int2d(Th)(lam*w);
Ph gkap, gfs; gkap[]=gk(0,Ph); gfs[]=gf(0,Ph);
for (int k=0;k<Th.nt;k++) cout << "G gkappa " << gkap[][k] << endl;
for (int k=0;k<Th.nt;k++) cout << "G gf " << gfs[][k] << endl;
for (int k=0;k<Th.nv;k++) cout << "G lam " << lam[][k] << endl;
{ int[int] I(1),J(1); real[int] C(1); [I,J,C]=M;
  for (int k=0;k<I.n;k++) cout << "G MI " << I[k] << endl;
  for (int k=0;k<I.n;k++) cout << "G MJ " << J[k] << endl;
  for (int k=0;k<I.n;k++) cout << "G MC " << C[k] << endl; }
""" + DUMP_MESH2 + DUMP_DOF + DUMP_A + \
        "for (int k=0;k<b.n;k++) cout << \"b \" << b[k] << \" \" << u[][k] << endl;\n"
    return body, files


def case_heat_p1(n, nsteps, dt, seed):
    """Implicit Euler for u_t - div(kappa grad u) = 1, u(0)=0, u=0 on the boundary."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nt = 2 * n * n
    kap = np.exp(0.3 * rng.standard_normal(nt))
    body = HEAD + f"""
mesh Th=square({n},{n});
fespace Vh(Th,P1); fespace Ph(Th,P0);
""" + read_vec_edp("kapa", "kappa.txt", "Th.nt") + f"""
Ph kappa; kappa[]=kapa;
real dt={dt!r};
Vh u,v,uold;
varf a(u,v)=int2d(Th)(u*v/dt + kappa*(dx(u)*dx(v)+dy(u)*dy(v))) + on(1,2,3,4,u=0);
varf m(u,v)=int2d(Th)(u*v/dt);
varf f(u,v)=int2d(Th)(1.*v) + on(1,2,3,4,u=0);
matrix A=a(Vh,Vh,solver=CG,eps=1e-14);
matrix M=m(Vh,Vh);
real[int] F=f(0,Vh);
u[]=0;
for (int s=0;s<{nsteps};s++) {{
  uold[]=u[];
  real[int] rhs=M*uold[]; rhs+=F;
  u[]=A^-1*rhs;
}}
for (int k=0;k<Th.nv;k++) cout << "G uT " << u[][k] << endl;
""" + DUMP_MESH2 + DUMP_DOF + DUMP_A
    return body, {"kappa.txt": kap}


def case_text_io(n):
    """FreeFEM's own text forms of a matrix and a vector (``f << A``, ``f << b``) next to the
    sorted COO and the values, for the readers of those forms."""
    body = HEAD + f"""
mesh Th=square({n},{n});
fespace Vh(Th,P1);
Vh u,v;
varf a(u,v)=int2d(Th)(dx(u)*dx(v)+dy(u)*dy(v)) + int2d(Th)((1+x)*v) + on(1,2,u=0);
matrix A=a(Vh,Vh);
real[int] b=a(0,Vh);
{{ ofstream f("A_coo.txt"); f << A; }}
{{ ofstream f("b.txt"); f << b; }}
""" + DUMP_A + "for (int k=0;k<b.n;k++) cout << \"b \" << b[k] << \" \" << b[k] << endl;\n"
    return body, {}


BT_VARF2 = {
    "P1": "int2d(Th)(dx(u)*dx(v)+dy(u)*dy(v)) + int1d(Th,3)(2.5*u*v) + int2d(Th)(1.*v) + int1d(Th,2)(gk*v) + int1d(Th,3)(-0.75*v) + on(1,4,u=0)",
}
BT_VARF3 = ("int3d(Th)(dx(u)*dx(v)+dy(u)*dy(v)+dz(u)*dz(v)) + int2d(Th,2)(2.*u*v) + int3d(Th)(1.*v) "
            "+ int2d(Th,1,3)(gk*v) + int2d(Th,6)(0.5*v) + on(4,u=0)")


def case_bterms(kind, dims, seed):
    """Boundary terms: Robin c*u*v and Neumann g*v on labelled boundary edges/faces (int1d in 2D,
    int2d on the boundary in 3D), g a constant or a P0 function (value of the adjacent element),
    next to the volume terms and on(...)."""
    rng = np.random.default_rng(seed)
    dim = len(dims)
    nt = 2 * dims[0] * dims[1] if dim == 2 else 6 * dims[0] * dims[1] * dims[2]
    gk = rng.uniform(0.5, 2.0, nt)
    if dim == 2:
        head = f"mesh Th=square({dims[0]},{dims[1]});\n"
        dump = DUMP_MESH2
    else:
        head = f'load "msh3"\nmesh3 Th=cube({dims[0]},{dims[1]},{dims[2]});\n'
        dump = DUMP_MESH3
    if kind == "P2vec":
        body = HEAD + head + """
fespace Vh(Th,[P2,P2,P2]); fespace Ph(Th,P0);
""" + read_vec_edp("gka", "gk.txt", "Th.nt") + """
Ph gk; gk[]=gka;
Vh [u1,u2,u3],[v1,v2,v3];
real E=1, nu=0.3; real mu=E/(2*(1+nu)); real lambda=E*nu/((1+nu)*(1-2*nu));
real s2=sqrt(2.);
macro epsilon(u1,u2,u3) [dx(u1),dy(u2),dz(u3),(dz(u2)+dy(u3))/s2,(dz(u1)+dx(u3))/s2,(dy(u1)+dx(u2))/s2] // EOM
macro div(u1,u2,u3) (dx(u1)+dy(u2)+dz(u3)) // EOM
varf a([u1,u2,u3],[v1,v2,v3])=int3d(Th)(lambda*div(u1,u2,u3)*div(v1,v2,v3)+2.*mu*(epsilon(u1,u2,u3)'*epsilon(v1,v2,v3)))
  + int2d(Th,6)(0.1*(u1*v1+u2*v2+u3*v3)) + int3d(Th)(-1.*v3) + int2d(Th,2)(0.25*v1-0.5*v3) + on(4,u1=0,u2=0,u3=0);
int nit=0;
matrix A=a(Vh,Vh,solver=CG,eps=1e-10,getnbiteration=nit);
real[int] b=a(0,Vh);
u1[]=0; u1[]=A^-1*b;
cout << "S nit " << nit << endl;
for (int k=0;k<Th.nt;k++) cout << "G p0dof " << Ph(k,0) << endl;
""" + dump + DUMP_DOF + DUMP_A + \
            "for (int k=0;k<b.n;k++) cout << \"b \" << b[k] << \" \" << u1[][k] << endl;\n"
        return body, {"gk.txt": gk}
    varf = BT_VARF2["P1"] if dim == 2 else BT_VARF3
    body = HEAD + head + f"""
fespace Vh(Th,{kind}); fespace Ph(Th,P0);
""" + read_vec_edp("gka", "gk.txt", "Th.nt") + f"""
Ph gk; gk[]=gka;
Vh u,v;
varf a(u,v)={varf};
int nit=0;
matrix A=a(Vh,Vh,solver=CG,eps=1e-10,getnbiteration=nit);
real[int] b=a(0,Vh);
u[]=0; u[]=A^-1*b;
cout << "S nit " << nit << endl;
for (int k=0;k<Th.nt;k++) cout << "G p0dof " << Ph(k,0) << endl;
""" + dump + DUMP_DOF + DUMP_A + \
        "for (int k=0;k<b.n;k++) cout << \"b \" << b[k] << \" \" << u[][k] << endl;\n"
    return body, {"gk.txt": gk}


CASES = {
    "p1sq_n2": lambda: case_p1_square(2),
    "p1sq_n5": lambda: case_p1_square(5),
    "p1sq_n16": lambda: case_p1_square(16),
    "p1sq_7x3": lambda: case_p1_square(7, 3),
    "p1sq_n8_T5": lambda: case_p1_square(8, qft="qft=qf5pT"),
    "p1sq_n12_gmres": lambda: case_p1_square(12, solver="GMRES"),
    "p1sqk_n8_jit": lambda: case_p1_square_kappa(8, seed=11, jitter=0.2),
    "p1sqk_n6": lambda: case_p1_square_kappa(6, seed=12, jitter=0.0),
    "p1cubek_n2": lambda: case_p1_cube_kappa(2, seed=21),
    "p1cubek_n4": lambda: case_p1_cube_kappa(4, seed=22),
    "p2cube_n2": lambda: case_p2_cube_scalar(2),
    "p2el_n1": lambda: case_p2_elasticity(1, 1, 1),
    "p2el_n2": lambda: case_p2_elasticity(2, 2, 2),
    "p2el_3x2x1": lambda: case_p2_elasticity(3, 2, 1),
    "p2sq_n4": lambda: case_p2_square_scalar(4),
    **{f"p2num_{w}": (lambda w=w: case_p2_numbering(w)) for w in P2NUM_MESHES},
    **{f"src_{w}": (lambda w=w: case_source_function(w)) for w in SOURCE_CASES},
    **{f"mq_{w}": (lambda w=w: case_mass_function(w)) for w in MASS_CASES},
    **{f"kq_{w}": (lambda w=w: case_stiff_function(w)) for w in STIFF_CASES},
    "p2elmat_2x2x1": lambda: case_p2_elasticity_materials(2, 2, 1, seed=61),
    "p1sq_n6_tgvm1": lambda: case_p1_square_tgv(6, -1, "GMRES"),
    "p1sq_n6_tgvm2": lambda: case_p1_square_tgv(6, -2, "CG"),
    "p1sq_n6_tgvm3": lambda: case_p1_square_tgv(6, -3, "GMRES"),
    "p1sq_n6_tgvp": lambda: case_p1_square_tgv(6, 1e30, "CG"),
    "adj_p1_n8": lambda: case_adjoint_p1(8, seed=31),
    "heat_p1_n6": lambda: case_heat_p1(6, 10, 1e-2, seed=41),
    "io_p1sq_n4": lambda: case_text_io(4),
    "p2cubem_n2": lambda: case_p2_mass(3, 2),
    "p2sqm_n4": lambda: case_p2_mass(2, 4),
    "bt_p1sq_6x5": lambda: case_bterms("P1", (6, 5), seed=51),
    "bt_p2sq_5x4": lambda: case_bterms("P2", (5, 4), seed=52),
    "bt_p1cube_3x3x2": lambda: case_bterms("P1", (3, 3, 2), seed=53),
    "bt_p2cube_2x2x2": lambda: case_bterms("P2", (2, 2, 2), seed=54),
    "bt_p2el_2x2x2": lambda: case_bterms("P2vec", (2, 2, 2), seed=55),
}


def parse(out: str) -> dict:
    rows: dict[str, list] = {}
    scal: dict[str, float] = {}
    extra: dict[str, list] = {}
    for line in out.splitlines():
        t = line.split()
        if not t:
            continue
        tag = t[0]
        if tag == "S":
            scal[t[1]] = float(t[2])
        elif tag == "G":
            extra.setdefault(t[1], []).append(float(t[2]))
        elif tag in ("V", "T", "B", "D", "A", "b"):
            rows.setdefault(tag, []).append(t[1:])
    res = {}
    if "V" in rows:
        v = np.array(rows["V"], dtype=np.float64)
        res["coords"] = v[:, :-1]
        res["vlabel"] = v[:, -1].astype(np.int64)
    if "T" in rows:
        res["elems"] = np.array(rows["T"], dtype=np.int64).astype(np.int32)
    if "B" in rows:
        bb = np.array(rows["B"], dtype=np.int64)
        res["belems"] = bb[:, :-1].astype(np.int32)
        res["blabel"] = bb[:, -1].astype(np.int32)
    if "D" in rows:
        res["dof"] = np.array(rows["D"], dtype=np.int64).astype(np.int32)
    if "A" in rows:
        a = rows["A"]
        res["I"] = np.array([r[0] for r in a], dtype=np.int32)
        res["J"] = np.array([r[1] for r in a], dtype=np.int32)
        res["C"] = np.array([r[2] for r in a], dtype=np.float64)
    if "b" in rows:
        bu = np.array(rows["b"], dtype=np.float64)
        res["b"] = bu[:, 0]
        res["u"] = bu[:, 1]
    for k, vals in extra.items():
        res["g_" + k] = np.array(vals, dtype=np.float64)
    res["scalar_names"] = np.array(sorted(scal), dtype="U32")
    res["scalar_values"] = np.array([scal[k] for k in sorted(scal)], dtype=np.float64)
    return res


def run_case(name: str) -> None:
    body, files = CASES[name]()
    with tempfile.TemporaryDirectory() as td:
        for fn, arr in files.items():
            np.savetxt(os.path.join(td, fn), np.asarray(arr), fmt="%.17g")
        script = os.path.join(td, name + ".edp")
        with open(script, "w") as f:
            f.write(body)
        env = dict(os.environ, FF_LOADPATH=FF_LOADPATH)
        p = subprocess.run([FF_BIN, "-nw", script, "-v", "0"], cwd=td, env=env,
                           capture_output=True, text=True, timeout=600)
        if p.returncode != 0:
            raise RuntimeError(f"{name}: FreeFEM failed\n{p.stdout[-2000:]}\n{p.stderr[-2000:]}")
        res = parse(p.stdout)
        for fn in ("A_coo.txt", "b.txt"):
            if os.path.exists(os.path.join(td, fn)):
                with open(os.path.join(td, fn)) as f:
                    res["text_" + fn.split(".")[0]] = np.array(f.read())
        for fn, arr in files.items():
            res["in_" + fn.split(".")[0]] = np.asarray(arr, dtype=np.float64)
        res["edp"] = np.array(body)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **res)
    print(f"{name}: " + ", ".join(f"{k}{tuple(np.shape(v))}" for k, v in res.items()
                                  if k != "edp"))


if __name__ == "__main__":
    names = sys.argv[1:] or list(CASES)
    for nm in names:
        run_case(nm)
