"""GPU incircle packing (pg_pack_incenters) against the oracle and the reference's golden vectors:
element and plain nodal circles bit-identical to the reference's own numpy code; maximin nodal
circles bit-identical to the oracle's restatement of the same ascent and exact solve."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
import packing_oracle as PO  # noqa: E402

from perigrain_gb300 import _native as N  # noqa: E402
from perigrain_gb300.packing import PackMesh, cube_mesh, get_incenter_mesh_loc, rect_mesh  # noqa: E402

pytestmark = pytest.mark.gpu


def golden_mesh(name):
    g = np.load(os.path.join(HERE, "golden", name + ".npz"))
    return g, PackMesh(g["pos"], g["T"], g["bdry_nodes"], g["bdry_edges"])


@pytest.mark.parametrize("name", ["pack2d_plain", "pack2d_interior", "pack2d_bdry", "pack3d_plain"])
def test_golden_meshes(name):
    g, m = golden_mesh(name)
    modify, gen = bool(g["modify"]), bool(g["gen_bdry"])
    out = get_incenter_mesh_loc(m, modify_nodal_circles=modify, gen_bdry=gen)
    ne = len(m.T)
    assert out.count() == len(g["incircle_rad"])
    # element circles: the reference's own code, bit for bit
    assert np.array_equal(out.incenter[:ne], g["incenter"][:ne])
    assert np.array_equal(out.incircle_rad[:ne], g["incircle_rad"][:ne])
    if not modify:
        assert np.array_equal(out.incenter, g["incenter"]) and np.array_equal(out.incircle_rad, g["incircle_rad"])
    inc, rad, ok = PO.incenter_mesh_loc(m.pos, m.T, m.bdry_nodes, m.bdry_edges, modify, gen)
    assert np.array_equal(out.incenter, inc) and np.array_equal(out.incircle_rad, rad)
    assert out.unpolished == 0 and ok.all()


@pytest.mark.parametrize("modify,gen", [(False, False), (True, False), (True, True)])
def test_larger_2d_mesh(modify, gen):
    m = rect_mesh(48, 30, width=2.0, height=1.25, jitter=0.3, seed=11)
    out = get_incenter_mesh_loc(m, modify_nodal_circles=modify, gen_bdry=gen)
    inc, rad, ok = PO.incenter_mesh_loc(m.pos, m.T, m.bdry_nodes, m.bdry_edges, modify, gen)
    assert np.array_equal(out.incenter, inc) and np.array_equal(out.incircle_rad, rad)
    assert out.unpolished == int((~ok).sum()) == 0
    # nodal circles clear the incircles of their elements
    ne = len(m.T)
    nbd = PO.node_elements(m.T, len(m.pos))
    bset = set(int(b) for b in m.bdry_nodes)
    nodes = [i for i in range(len(m.pos)) if i not in bset or (modify and gen)]
    for j, i in enumerate(nodes):
        c, r = out.incenter[ne + j], out.incircle_rad[ne + j, 0]
        d = np.sqrt(np.sum((inc[nbd[i]] - c) ** 2, axis=1)) - rad[nbd[i], 0]
        assert r > 0 and (d >= r - 1e-12).all()
    assert 0.5 < out.packing_ratio() < 1.0


def test_3d_mesh():
    m = cube_mesh(9, size=1.0, jitter=0.2, seed=12)
    out = get_incenter_mesh_loc(m, modify_nodal_circles=False, gen_bdry=False)
    inc, rad, _ = PO.incenter_mesh_loc(m.pos, m.T, m.bdry_nodes, m.bdry_edges, False, False)
    assert np.array_equal(out.incenter, inc) and np.array_equal(out.incircle_rad, rad)


def test_errors():
    m = rect_mesh(4, 3, seed=1)
    bad = PackMesh(m.pos, np.where(m.T == 5, len(m.pos) + 3, m.T), m.bdry_nodes, m.bdry_edges)
    with pytest.raises(N.PerigrainError) as e:
        get_incenter_mesh_loc(bad, modify_nodal_circles=False, gen_bdry=False)
    assert e.value.code == N.PG_EINVAL
    c = cube_mesh(2, seed=1)
    with pytest.raises(N.PerigrainError) as e:
        get_incenter_mesh_loc(c, modify_nodal_circles=True, gen_bdry=False)
    assert e.value.code == N.PG_EINVAL


def test_trim():
    m = rect_mesh(10, 6, seed=3)
    out = get_incenter_mesh_loc(m, modify_nodal_circles=True, gen_bdry=True)
    lo, hi = np.quantile(out.incircle_rad, [0.2, 0.8])
    n = out.count()
    out.trim(min_rad=lo, max_rad=hi)
    r = out.incircle_rad.ravel()
    assert (r >= lo).all() and (r <= hi).all() and out.count() < n and len(out.incenter) == out.count()
