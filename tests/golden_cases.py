"""The golden cases: each FreeFEM fixture with the inputs needed to rebuild it here."""
import os

import numpy as np

from ffgpu import mesh

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    sc = dict(zip([str(s) for s in d["scalar_names"]], d["scalar_values"]))
    return d, sc


def case(name):
    """-> dict(Th, kind, form, kappa, f, labels, quad, solver, eps)"""
    d, sc = load(name)
    c = dict(name=name, d=d, sc=sc, kappa=None, f=1.0, form="diffusion", quad=None,
             solver="CG", eps=1e-10, components=None)
    if name.startswith("p1sq_"):
        parts = name.split("_")
        if "x" in parts[1]:
            nx, ny = map(int, parts[1].split("x"))
        else:
            nx = ny = int(parts[1][1:])
        c.update(Th=mesh.square(nx, ny), kind="P1", labels=(1, 2, 3, 4),
                 quad="qf5pT" if "T5" in name else "qf2pT",
                 solver="GMRES" if "gmres" in name else "CG")
    elif name.startswith("p1sqk_"):
        n = int(name.split("_")[1][1:])
        c.update(Th=mesh.movemesh(mesh.square(n), d["coords"]), kind="P1", labels=(1, 2, 3, 4),
                 kappa=d["in_kappa"])
    elif name.startswith("p1cubek_"):
        n = int(name.split("_")[1][1:])
        c.update(Th=mesh.cube(n), kind="P1", labels=(1, 2, 3, 4, 5, 6), kappa=d["in_kappa"])
    elif name.startswith("p2cube_"):
        n = int(name.split("_")[1][1:])
        c.update(Th=mesh.cube(n), kind="P2", labels=(1, 2, 3, 4, 5, 6))
    elif name.startswith("p2el_"):
        s = name.split("_")[1]
        dims = (int(s[1:]),) * 3 if s.startswith("n") else tuple(map(int, s.split("x")))
        c.update(Th=mesh.cube(*dims), kind="P2vec", labels=(4,), form="elasticity", f=(0.0, 0.0, -1.0))
    elif name.startswith("p2sq_"):
        n = int(name.split("_")[1][1:])
        c.update(Th=mesh.square(n), kind="P2", labels=(1, 2, 3, 4), dof=d["dof"])
    elif name.startswith("p2cubem_"):
        n = int(name.split("_")[1][1:])
        c.update(Th=mesh.cube(n), kind="P2", labels=(1, 2, 3, 4, 5, 6), mass=2.5)
    elif name.startswith("p2sqm_"):
        n = int(name.split("_")[1][1:])
        c.update(Th=mesh.square(n), kind="P2", labels=(1, 2, 3, 4), dof=d["dof"], mass=2.5)
    else:
        raise KeyError(name)
    return c


MATRIX_CASES = ["p1sq_n2", "p1sq_n5", "p1sq_n16", "p1sq_7x3", "p1sq_n8_T5", "p1sq_n12_gmres",
                "p1sqk_n8_jit", "p1sqk_n6", "p1cubek_n2", "p1cubek_n4", "p2cube_n2", "p2el_n1",
                "p2el_n2", "p2el_3x2x1", "p2sq_n4", "p2cubem_n2", "p2sqm_n4"]


def value_errors(v, ref, rowptr):
    """Per-entry relative error with a floor of 1e-3 x the row's largest non-tgv entry:
    |v - ref| / max(|ref|, 1e-3 * s_row).  (Entries FreeFEM computes as round-off residue of
    a cancelling sum have no meaningful relative error of their own.)"""
    n = rowptr.size - 1
    a = np.abs(ref)
    a_nt = np.where(a >= 1e20, 0.0, a)
    rows = np.repeat(np.arange(n), np.diff(rowptr))
    s = np.zeros(n)
    np.maximum.at(s, rows, a_nt)
    den = np.maximum(a, 1e-3 * s[rows])
    den = np.where(den == 0, 1.0, den)
    return np.abs(v - ref) / den


# Boundary-term cases (tests/golden/make_golden.py: case_bterms): volume terms as the other
# cases, then the boundary terms in varf order.  "gk" = the P0 function of the fixture, taken
# on each boundary element from its adjacent element.
BT_CASES = {
    "bt_p1sq_6x5": dict(kind="P1", dims=(6, 5), on=(1, 4), robin=[((3,), 2.5)],
                        neumann=[((2,), "gk"), ((3,), -0.75)]),
    "bt_p2sq_5x4": dict(kind="P2", dims=(5, 4), on=(1, 4), robin=[((3,), 2.5)],
                        neumann=[((2,), "gk"), ((3,), -0.75)]),
    "bt_p1cube_3x3x2": dict(kind="P1", dims=(3, 3, 2), on=(4,), robin=[((2,), 2.0)],
                            neumann=[((1, 3), "gk"), ((6,), 0.5)]),
    "bt_p2cube_2x2x2": dict(kind="P2", dims=(2, 2, 2), on=(4,), robin=[((2,), 2.0)],
                            neumann=[((1, 3), "gk"), ((6,), 0.5)]),
    "bt_p2el_2x2x2": dict(kind="P2vec", dims=(2, 2, 2), on=(4,), robin=[((6,), 0.1)],
                          neumann=[((2,), (0.25, 0.0, -0.5))]),
}


def bt_case(name):
    """-> dict(Th, kind, d, sc, spec, gk_elem): gk_elem[k] = the P0 value on element k."""
    d, sc = load(name)
    spec = BT_CASES[name]
    dims = spec["dims"]
    Th = mesh.square(*dims) if len(dims) == 2 else mesh.cube(*dims)
    gk_elem = d["in_gk"][d["g_p0dof"].astype(np.int64)]
    return dict(name=name, d=d, sc=sc, spec=spec, Th=Th, kind=spec["kind"], gk_elem=gk_elem,
                dof=d["dof"] if spec["kind"] == "P2" and len(dims) == 2 else None)
