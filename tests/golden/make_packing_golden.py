"""Golden vectors of the incircle packing, produced by the reference's own code.

Runs get_incenter_mesh_loc from the reference's exp_dict.py, imported from the reference checkout
(PERIGRAIN_REFERENCE, else the development container's checkout; this script runs there only, its
outputs are committed).
The reference's third-party imports that are absent here are replaced by stand-ins:
  genmesh   returns the test mesh (PackMesh from perigrain_gb300.packing: seeded structured
            meshes of a rectangle / cube) in the layout genmesh.py:160-291 returns
  GEKKO     records the model the reference builds per node (variables, initial values,
            equations, objective) and solves it with scipy's SLSQP, with exact gradients from
            forward-mode differentiation of the recorded expressions
  pathos    ProcessingPool.map is the serial map
  h5py, matplotlib, pygmsh, meshio, gmsh: empty modules (not called on this path)

Usage: python tests/golden/make_packing_golden.py  -> tests/golden/pack*.npz
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("PERIGRAIN_REFERENCE") or "/root/reference"
sys.path.insert(0, ROOT)

from perigrain_gb300.packing import cube_mesh, rect_mesh  # noqa: E402

CASES = {
    "pack2d_plain": dict(mesh=lambda: rect_mesh(12, 8, width=1.0, height=0.6, jitter=0.2, seed=1),
                         modify=False, gen_bdry=False, dim=2),
    "pack2d_interior": dict(mesh=lambda: rect_mesh(12, 8, width=1.0, height=0.6, jitter=0.25, seed=2),
                            modify=True, gen_bdry=False, dim=2),
    "pack2d_bdry": dict(mesh=lambda: rect_mesh(10, 7, width=0.8, height=0.5, jitter=0.25, seed=3),
                        modify=True, gen_bdry=True, dim=2),
    "pack3d_plain": dict(mesh=lambda: cube_mesh(4, size=1.0, jitter=0.15, seed=4), modify=False,
                         gen_bdry=False, dim=3),
}


# ---- forward-mode expressions for the GEKKO stand-in ---------------------------------------------
class Expr:
    """f(v) -> (value, gradient) over the model's variables v."""

    def __init__(self, fn):
        self.fn = fn

    @staticmethod
    def lift(x):
        if isinstance(x, Expr):
            return x
        c = float(np.asarray(x).ravel()[0]) if np.ndim(x) else float(x)
        return Expr(lambda v, c=c: (c, np.zeros(len(v))))

    def ev(self, v):
        return self.fn(v)

    def _bin(self, other, op, rev=False):
        a, b = (Expr.lift(other), self) if rev else (self, Expr.lift(other))

        def fn(v):
            (x, gx), (y, gy) = a.ev(v), b.ev(v)
            if op == "+":
                return x + y, gx + gy
            if op == "-":
                return x - y, gx - gy
            if op == "*":
                return x * y, x * gy + y * gx
            if op == "/":
                return x / y, (gx * y - x * gy) / (y * y)
            raise ValueError(op)

        return Expr(fn)

    def __add__(self, o):
        return self._bin(o, "+")

    def __radd__(self, o):
        return self._bin(o, "+", True)

    def __sub__(self, o):
        return self._bin(o, "-")

    def __rsub__(self, o):
        return self._bin(o, "-", True)

    def __mul__(self, o):
        return self._bin(o, "*")

    def __rmul__(self, o):
        return self._bin(o, "*", True)

    def __truediv__(self, o):
        return self._bin(o, "/")

    def __rtruediv__(self, o):
        return self._bin(o, "/", True)

    def __neg__(self):
        return Expr(lambda v: tuple(-t for t in self.ev(v)))

    def __pow__(self, p):
        p = float(p)

        def fn(v):
            x, g = self.ev(v)
            return x ** p, p * x ** (p - 1) * g

        return Expr(fn)

    def __abs__(self):
        def fn(v):
            x, g = self.ev(v)
            return abs(x), np.sign(x) * g

        return Expr(fn)

    def __ge__(self, o):
        return Constraint(self - o)

    def __le__(self, o):
        return Constraint(Expr.lift(o) - self)

    def __array_ufunc__(self, ufunc, method, *inputs, **kw):
        if method != "__call__":
            return NotImplemented
        name = ufunc.__name__
        if name == "absolute":
            return abs(inputs[0])
        if name == "negative":
            return -inputs[0]
        binary = {"add": "+", "subtract": "-", "multiply": "*", "true_divide": "/", "divide": "/"}
        if name in binary:
            a, b = inputs
            return Expr.lift(a)._bin(b, binary[name])
        if name == "less_equal":
            return Expr.lift(inputs[0]).__le__(inputs[1])
        if name == "greater_equal":
            return Expr.lift(inputs[0]).__ge__(inputs[1])
        return NotImplemented


class Var(Expr):
    def __init__(self, k, value=0.0):
        self.k = k
        self.value = value
        super().__init__(self._fn)

    def _fn(self, v):
        g = np.zeros(len(v))
        g[self.k] = 1.0
        return v[self.k], g


class Constraint:
    def __init__(self, g):
        self.g = g  # g(v) >= 0


SOLVES = []


class GEKKO:
    def __init__(self, remote=True, **kw):
        self.options = types.SimpleNamespace()
        self._vars, self._cons, self._obj = [], [], None

    def Var(self, value=0.0, **kw):
        v = Var(len(self._vars), value)
        self._vars.append(v)
        return v

    def Array(self, f, dim, **kw):
        a = np.empty(dim, dtype=object)
        for k in range(dim):
            a[k] = f()
        return a

    def Maximize(self, e):
        self._obj = (-1.0, Expr.lift(e))

    def Minimize(self, e):
        self._obj = (1.0, Expr.lift(e))

    def Equation(self, c):
        self._cons.append(c)

    def solve(self, disp=True, **kw):
        from scipy.optimize import minimize

        sgn, obj = self._obj
        x0 = np.array([float(np.ravel(v.value)[0]) for v in self._vars])
        cons = [{"type": "ineq", "fun": lambda v, c=c: c.g.ev(v)[0], "jac": lambda v, c=c: c.g.ev(v)[1]}
                for c in self._cons]

        def f(v):
            val, g = obj.ev(v)
            return sgn * val, sgn * g

        res = minimize(f, x0, jac=True, constraints=cons, method="SLSQP", options={"ftol": 1e-15, "maxiter": 1000})
        SOLVES.append(bool(res.success))
        for v, x in zip(self._vars, res.x):
            v.value = [float(x)]
        self._variables = [v.value for v in self._vars]


# ---- the other stand-ins ---------------------------------------------------------------------------
CURRENT = {}


class MeshResult:
    def __init__(self, m):
        self.pos, self.T, self.vol = m.pos, m.T, m.vol[:, None]
        self.bdry_nodes = [int(b) for b in m.bdry_nodes]
        self.bdry_edges = m.bdry_edges


def _genmesh(P_bdry=None, meshsize=None, msh_file=None, dimension=2, **kw):
    return MeshResult(CURRENT["mesh"])


class ProcessingPool:
    def map(self, f, items):
        return [f(x) for x in items]


def install_stubs():
    for name in ("h5py", "matplotlib", "matplotlib.pyplot", "matplotlib.collections", "pygmsh", "meshio", "gmsh",
                 "mpl_toolkits", "mpl_toolkits.mplot3d", "pathos", "pathos.multiprocessing", "gekko", "genmesh"):
        sys.modules[name] = types.ModuleType(name)
    sys.modules["matplotlib.collections"].LineCollection = object
    sys.modules["mpl_toolkits.mplot3d"].Axes3D = object
    sys.modules["pathos.multiprocessing"].ProcessingPool = ProcessingPool
    sys.modules["gekko"].GEKKO = GEKKO
    sys.modules["genmesh"].genmesh = _genmesh


def main(names=None):
    install_stubs()
    sys.path.insert(0, REF)
    import exp_dict

    for name, spec in CASES.items():
        if names and name not in names:
            continue
        m = spec["mesh"]()
        CURRENT["mesh"] = m
        SOLVES.clear()
        out = exp_dict.get_incenter_mesh_loc(None, None, dimension=spec["dim"], msh_file="stand-in",
                                             modify_nodal_circles=spec["modify"], gen_bdry=spec["gen_bdry"])
        fn = os.path.join(HERE, name + ".npz")
        np.savez_compressed(fn, pos=m.pos, T=m.T, bdry_nodes=m.bdry_nodes, bdry_edges=m.bdry_edges,
                            modify=spec["modify"], gen_bdry=spec["gen_bdry"],
                            incenter=np.asarray(out.incenter, np.float64),
                            incircle_rad=np.asarray(out.incircle_rad, np.float64),
                            solver_ok=np.array(SOLVES, bool))
        print(name, "circles", len(out.incircle_rad), "SLSQP solves", len(SOLVES), "failed", SOLVES.count(False))


if __name__ == "__main__":
    main(sys.argv[1:])
