"""The packing oracle against golden vectors made by the reference's own get_incenter_mesh_loc
(tests/golden/make_packing_golden.py), and the test meshes themselves. CPU only."""
import math
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
import packing_oracle as PO  # noqa: E402

from perigrain_gb300.packing import cube_mesh, element_volume, rect_mesh  # noqa: E402

CASES = ["pack2d_plain", "pack2d_interior", "pack2d_bdry", "pack3d_plain"]
# maximin circles: the reference's model has several local maxima around many nodes, so the
# golden (SLSQP standing in for APOPT) and the oracle may stop at different ones; where they reach
# the same one they agree to AGREE_TOL, and on at least AGREE_FRAC of the nodes they do.
AGREE_TOL = 1e-9
AGREE_FRAC = 0.75


def load(name):
    return np.load(os.path.join(HERE, "golden", name + ".npz"))


def node_model(g, i, boundary):
    """The node's constraints: circles (centre, radius), lines (e1, u) and the box."""
    pos, T = g["pos"], g["T"]
    inc, rad = PO.element_circles(pos, T)
    e = [k for k in range(len(T)) if i in set(int(v) for v in T[k])]
    circles = [(inc[k], rad[k][0]) for k in e]
    lines = []
    xs, ys = list(inc[e][:, 0]), list(inc[e][:, 1])
    if boundary:
        for a, b in g["bdry_edges"]:
            if i in (int(a), int(b)):
                lines.append((pos[a], pos[b] - pos[a]))
        xs.append(pos[i][0])
        ys.append(pos[i][1])
    return circles, lines, (min(xs), min(ys)), (max(xs), max(ys))


def value(x, circles, lines):
    v = min(math.hypot(x[0] - p[0], x[1] - p[1]) - r for p, r in circles)
    for e1, u in lines:
        v = min(v, abs(u[0] * (x[1] - e1[1]) - u[1] * (x[0] - e1[0])) / math.hypot(u[0], u[1]))
    return v


def is_local_max(x, circles, lines, lo, hi, eps):
    """No point of the box on a ring of radius eps (and eps / 8) around x is higher."""
    f = value(x, circles, lines)
    for rr in (eps, eps / 8):
        for k in range(32):
            a = 2 * math.pi * k / 32
            y = (min(max(x[0] + rr * math.cos(a), lo[0]), hi[0]), min(max(x[1] + rr * math.sin(a), lo[1]), hi[1]))
            if value(y, circles, lines) > f + 1e-12:
                return False
    return True


@pytest.mark.parametrize("name", CASES)
def test_element_circles_bit_identical_to_reference(name):
    g = load(name)
    inc, rad = PO.element_circles(g["pos"], g["T"])
    m = len(g["T"])
    assert np.array_equal(inc, g["incenter"][:m]) and np.array_equal(rad, g["incircle_rad"][:m])


@pytest.mark.parametrize("name", ["pack2d_plain", "pack3d_plain"])
def test_plain_nodal_circles_bit_identical_to_reference(name):
    g = load(name)
    inc, rad, ok = PO.incenter_mesh_loc(g["pos"], g["T"], g["bdry_nodes"], g["bdry_edges"], False, False)
    assert np.array_equal(inc, g["incenter"]) and np.array_equal(rad, g["incircle_rad"]) and ok.all()


@pytest.mark.parametrize("name", ["pack2d_interior", "pack2d_bdry"])
def test_maximin_nodal_circles_solve_the_reference_model(name):
    g = load(name)
    gen = bool(g["gen_bdry"])
    inc, rad, ok = PO.incenter_mesh_loc(g["pos"], g["T"], g["bdry_nodes"], g["bdry_edges"], True, gen)
    assert ok.all()
    m = len(g["T"])
    assert inc.shape == g["incenter"].shape
    bset = set(int(b) for b in g["bdry_nodes"])
    nodes = [i for i in range(len(g["pos"])) if gen or i not in bset]
    agree = n_ok = 0
    for j, i in enumerate(nodes):
        circles, lines, lo, hi = node_model(g, i, i in bset)
        scale = max(hi[0] - lo[0], hi[1] - lo[1])
        x, r = inc[m + j], rad[m + j, 0]
        # the oracle's circle: tight (its radius is the model's value there), in the box, a local
        # maximum, and no smaller than the value at the initial guess
        assert abs(value(x, circles, lines) - r) <= 1e-12 * scale
        assert lo[0] - 1e-12 <= x[0] <= hi[0] + 1e-12 and lo[1] - 1e-12 <= x[1] <= hi[1] + 1e-12
        assert is_local_max(x, circles, lines, lo, hi, 1e-6 * scale), i
        x0 = g["pos"][i] if i not in bset else (np.mean(np.append([c[0][0] for c in circles], g["pos"][i][0])),
                                                 np.mean(np.append([c[0][1] for c in circles], g["pos"][i][1])))
        assert r >= value(x0, circles, lines) - 1e-12 * scale
        if g["solver_ok"][j]:
            n_ok += 1
            gx, gr = g["incenter"][m + j], g["incircle_rad"][m + j, 0]
            if abs(gr - r) <= AGREE_TOL * scale and np.abs(gx - x).max() <= 100 * AGREE_TOL * scale:
                agree += 1
    assert agree >= AGREE_FRAC * n_ok, (agree, n_ok)


def test_mesh_generators():
    m = rect_mesh(9, 5, width=0.9, height=0.5, jitter=0.25, seed=7)
    assert (element_volume(m.pos, m.T) > 0).all()
    assert abs(m.vol.sum() - 0.45) < 1e-12
    assert len(m.bdry_edges) == 2 * (9 + 5) and len(m.bdry_nodes) == 2 * (9 + 5)
    c = cube_mesh(3, size=2.0, jitter=0.2, seed=8)
    assert (element_volume(c.pos, c.T) > 0).all()
    assert abs(c.vol.sum() - 8.0) < 1e-12
    assert len(c.T) == 6 * 27 and len(c.bdry_nodes) == 4 ** 3 - 2 ** 3
