"""FreeFEM's volume quadrature rules, for sources given as functions of the coordinates.

A source f(x, y[, z]) that is not constant on elements enters b = a(0,Vh) through its values
at the points of the form's rule (Element_rhs, src/fflib/problem.cpp:7839-7911 and 7917-7990):
b_i += |K| sum_q w_q f(x_q) phi_i(lambda_q).  The rules are the published ones FreeFEM uses
(src/femlib/QuadratureFormular.cpp): points in the coordinates of the reference element,
weights relative to the element measure.

* ``qf2pT``: the 3 edge midpoints (degree 2);
* ``qf5pT``: the 7-point degree-5 rule of Radon (FreeFEM's default for ``int2d``);
* ``tet2``: the 4-point degree-2 rule on tetrahedra;
* ``tet5``: the 14-point degree-5 rule on tetrahedra (three orbits of 4, 4 and 6 points;
  FreeFEM's default for ``int3d``).
"""
from __future__ import annotations

import numpy as np


def _t5():
    s15 = np.sqrt(15.0)
    t = 1.0 / 3.0
    r, s, B = (6 - s15) / 21, (9 + 2 * s15) / 21, (155 - s15) / 1200
    u, v, Cw = (6 + s15) / 21, (9 - 2 * s15) / 21, (155 + s15) / 1200
    P = [(t, t), (r, r), (r, s), (s, r), (u, u), (u, v), (v, u)]
    W = [0.225, B, B, B, Cw, Cw, Cw]
    return np.array(P), np.array(W)


def _tet5():
    a1, b1 = 0.7217942490673263207930282587889082, 0.0927352503108912264023239137370306
    a2, b2 = 0.067342242210098170607962798709629, 0.310885919263300609797345733763457
    a3, b3 = 0.454496295874350350508119473720660, 0.045503704125649649491880526279339
    w1 = 0.0122488405193936582572850342477212 * 6.0
    w2 = 0.0187813209530026417998642753888810 * 6.0
    w3 = 7.09100346284691107301157135337624e-3 * 6.0
    P = [(a1, b1, b1), (b1, a1, b1), (b1, b1, a1), (b1, b1, b1),
         (a2, b2, b2), (b2, a2, b2), (b2, b2, a2), (b2, b2, b2),
         (a3, a3, b3), (a3, b3, a3), (b3, a3, a3), (b3, b3, a3), (b3, a3, b3), (a3, b3, b3)]
    return np.array(P), np.array([w1] * 4 + [w2] * 4 + [w3] * 6)


def _rule(name):
    if name == "qf2pT":
        return np.array([(0.5, 0.5), (0.0, 0.5), (0.5, 0.0)]), np.full(3, 1.0 / 3.0)
    if name == "qf5pT":
        return _t5()
    if name == "tet2":
        a, b = 0.58541019662496845446137605030968, 0.138196601125010515179541316563436
        return np.array([(a, b, b), (b, a, b), (b, b, a), (b, b, b)]), np.full(4, 0.25)
    if name == "tet5":
        return _tet5()
    raise ValueError(f"unknown quadrature rule {name!r} (qf2pT, qf5pT, tet2, tet5)")


def rule(name: str | None, dim: int):
    """(lambda (nq, dim+1), weights (nq,)) of a rule; None = FreeFEM's default for the dimension.
    lambda[q, i] is the barycentric coordinate of local vertex i: lambda_0 = 1 - sum of the
    reference coordinates, lambda_i = the i-th reference coordinate."""
    name = name or ("qf5pT" if dim == 2 else "tet5")
    P, W = _rule(name)
    if P.shape[1] != dim:
        raise ValueError(f"rule {name} is not a {dim}D rule")
    lam = np.concatenate([1.0 - P.sum(axis=1, keepdims=True), P], axis=1)
    return np.ascontiguousarray(lam), np.ascontiguousarray(W)


def points(coords, elems, lam):
    """Physical quadrature points (nt, nq, dim): x_q = sum_i lambda_q,i X_{v_i}."""
    X = np.asarray(coords, np.float64)[np.asarray(elems)]          # (nt, dim+1, dim)
    return np.einsum("qi,tid->tqd", lam, X)
