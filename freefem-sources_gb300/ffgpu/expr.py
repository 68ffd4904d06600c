"""Coefficient and source expressions evaluated on the device at the quadrature points.

The FreeFEM way to write a varf term's coefficient -- a function of the point built from
x, y, z, constants, FE functions (by their DOF values) and their derivatives:

    from ffgpu.expr import x, y, exp, sqrt, fe, dx
    kappa = 1 + x * y                      # int2d(Th)((1+x*y)*grad(u)'*grad(v))
    uh = fe("P1", values)                  # an FE function u[] of a P1 space
    f = exp(-uh) + dx(uh) ** 2

An Expr compiles to the postfix program of ffgpu_expr (include/ffgpu.h): the device runs it at
every quadrature point of every element (FreeFEM's Element_Op / Element_rhs evaluate the term's
expression point by point: problem.cpp:6117-6132, 7880-7900).  Python numbers combine with
expressions as constants.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

OPS = {"const": 1, "x": 2, "y": 3, "z": 4, "fe": 5, "dx": 6, "dy": 7, "dz": 8,
       "add": 16, "sub": 17, "mul": 18, "div": 19, "pow": 20, "min": 21, "max": 22,
       "neg": 32, "exp": 33, "log": 34, "sqrt": 35, "sin": 36, "cos": 37, "tan": 38, "abs": 39,
       "tanh": 40, "atan": 41}
_NP = {"add": np.add, "sub": np.subtract, "mul": np.multiply, "div": np.divide, "pow": np.power,
       "min": np.minimum, "max": np.maximum, "neg": np.negative, "exp": np.exp, "log": np.log,
       "sqrt": np.sqrt, "sin": np.sin, "cos": np.cos, "tan": np.tan, "abs": np.abs, "tanh": np.tanh,
       "atan": np.arctan}


class FEFunction:
    """An FE function of the mesh given by its DOF values: kind "P0" (one value per element),
    "P1" (per vertex) or "P2" (per DOF of `dof`, an nt x 6|10 table in FreeFEM's local order;
    None: the assembled space's own table)."""

    def __init__(self, kind, values, dof=None):
        self.kind = {"P0": _lib.FE_P0, "P1": _lib.FE_P1, "P2": _lib.FE_P2}[kind]
        self.kind_name = kind
        self.values = values if hasattr(values, "data_ptr") else np.ascontiguousarray(values, np.float64)
        self.dof = None if dof is None else (dof if hasattr(dof, "data_ptr") else np.ascontiguousarray(dof, np.int32))


class Expr:
    def __init__(self, op, args=(), value=None):
        self.op, self.args, self.value = op, tuple(args), value

    # arithmetic
    def _bin(self, o, op, rev=False):
        o = o if isinstance(o, Expr) else Expr("const", value=float(o))
        return Expr(op, (o, self) if rev else (self, o))

    def __add__(self, o): return self._bin(o, "add")
    def __radd__(self, o): return self._bin(o, "add", True)
    def __sub__(self, o): return self._bin(o, "sub")
    def __rsub__(self, o): return self._bin(o, "sub", True)
    def __mul__(self, o): return self._bin(o, "mul")
    def __rmul__(self, o): return self._bin(o, "mul", True)
    def __truediv__(self, o): return self._bin(o, "div")
    def __rtruediv__(self, o): return self._bin(o, "div", True)
    def __pow__(self, o): return self._bin(o, "pow")
    def __rpow__(self, o): return self._bin(o, "pow", True)
    def __neg__(self): return Expr("neg", (self,))

    def compile(self):
        """-> (ops int32, consts float64, FE functions) of the postfix program."""
        ops, consts, fes = [], [], []

        def emit(e):
            if e.op == "const":
                ops.extend([OPS["const"], len(consts)])
                consts.append(e.value)
            elif e.op in ("x", "y", "z"):
                ops.append(OPS[e.op])
            elif e.op in ("fe", "dx", "dy", "dz"):
                f = e.value
                k = next((i for i, g in enumerate(fes) if g is f), None)
                if k is None:
                    k = len(fes)
                    fes.append(f)
                ops.extend([OPS[e.op], k])
            else:
                for a in e.args:
                    emit(a)
                ops.append(OPS[e.op])

        emit(self)
        return np.asarray(ops, np.int32), np.asarray(consts if consts else [0.0], np.float64), fes

    def evaluate(self, xq, fe_values=None):
        """Host evaluation (numpy) at points xq[..., d]; FE functions need fe_values[id(f)]
        (their values at the same points).  Used to check the device evaluation."""
        if self.op == "const":
            return self.value
        if self.op in ("x", "y", "z"):
            return xq[..., "xyz".index(self.op)]
        if self.op in ("fe", "dx", "dy", "dz"):
            return fe_values[(id(self.value), self.op)]
        return _NP[self.op](*[a.evaluate(xq, fe_values) for a in self.args])


x = Expr("x")
y = Expr("y")
z = Expr("z")


def const(v):
    return Expr("const", value=float(v))


def fe(kind, values, dof=None):
    """The FE function u[] of a P0/P1/P2 space as an expression (its value at the point)."""
    return Expr("fe", value=FEFunction(kind, values, dof))


def _fe_of(e):
    if not (isinstance(e, Expr) and e.op == "fe"):
        raise TypeError("dx/dy/dz apply to an FE function (ffgpu.expr.fe)")
    return e.value


def dx(e): return Expr("dx", value=_fe_of(e))
def dy(e): return Expr("dy", value=_fe_of(e))
def dz(e): return Expr("dz", value=_fe_of(e))


def _un(op):
    def f(a):
        if not isinstance(a, Expr):
            return float(_NP[op](a))
        return Expr(op, (a,))
    f.__name__ = op
    return f


exp, log, sqrt, sin, cos, tan, tanh, atan = (_un(o) for o in ("exp", "log", "sqrt", "sin", "cos", "tan", "tanh", "atan"))
fabs = _un("abs")


def fmin(a, b):
    a = a if isinstance(a, Expr) else const(a)
    return a._bin(b, "min")


def fmax(a, b):
    a = a if isinstance(a, Expr) else const(a)
    return a._bin(b, "max")


def c_expr(e: Expr, keep: list) -> _lib.ExprC:
    """The ffgpu_expr struct of an expression (arrays kept alive in `keep`)."""
    ops, consts, fes = e.compile()
    ex = _lib.ExprC()
    ex.nops = ops.size
    ex.ops = ops.ctypes.data_as(C.c_void_p).value
    ex.consts = consts.ctypes.data_as(C.c_void_p).value
    ex.nfe = len(fes)
    keep += [ops, consts]
    if fes:
        arr = (_lib.FEFuncC * len(fes))()
        for k, f in enumerate(fes):
            arr[k].kind = f.kind
            arr[k].values = f.values.data_ptr() if hasattr(f.values, "data_ptr") else f.values.ctypes.data
            arr[k].dof = None if f.dof is None else (f.dof.data_ptr() if hasattr(f.dof, "data_ptr") else f.dof.ctypes.data)
            keep += [f.values, f.dof]
        keep.append(arr)
        ex.fe = C.cast(arr, C.c_void_p).value
    else:
        ex.fe = None
    return ex
