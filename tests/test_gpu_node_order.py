"""The node layout inside the grains (pg_config.node_order) changes where nodes sit on the device,
never a result: every output -- fields, the alive-bond set and break steps in CSR order, the
contact-pair log, wall reactions, snapshots, post-processing, gradients -- is bit-identical between
the input's order, a seeded shuffle (every node moved) and the cell order grouped by bond count
(whole grain and 256-node windows), in FP64 and mixed precision. The reference's own orders are kept through the input indices: bond
rows in NbdArr order, contact candidates in the reference's visit order, wall reactions replayed in
node order, sums over a grain in node order. A shuffled layout is also bit-exact against the oracle."""
import numpy as np
import pytest

import _oracle as O
from perigrain_gb300 import Simulation, grad, setups

pytestmark = pytest.mark.gpu

ORDERS = ("input", "shuffle", "cell_degree", "cell_block_degree")
FIELDS = ("CurrPos", "vel", "acc", "force", "disp")


def _run(s, order, steps, hook=None, **kw):
    g = Simulation(s, record_pairs=True, pair_log_capacity=steps, node_order=order, **kw)
    if hook:
        hook(g, steps)
    else:
        g.step(steps)
    out = {f: g.field(f) for f in FIELDS}
    out["alive"] = g.bond_alive()
    out["break_step"] = g.break_step()
    out["pairs"] = g.pair_log(steps)
    out["reaction"] = g.reaction()
    out["wall"] = g.wall()
    out["status"] = g.device_status()
    snap = g.snapshot(("CurrPos", "vel", "acc", "force", "disp", "bond_alive", "wall", "reaction")).wait()
    out.update({"snap_" + k: v for k, v in snap.items() if isinstance(v, np.ndarray)})
    post = g.postprocess(node_damage=True)
    out.update({"post_" + k: v for k, v in post.items()})
    out["layout"] = g.node_order()
    g.close()
    return out


def _same(a, b):
    for k in a:
        if k == "layout":
            continue
        x, y = a[k], b[k]
        if isinstance(x, tuple):
            for u, v in zip(x, y):
                assert np.array_equal(np.asarray(u), np.asarray(v), equal_nan=True), k
        else:
            assert np.array_equal(np.asarray(x), np.asarray(y), equal_nan=True), k


def _check(s, steps, **kw):
    runs = {o: _run(s, o, steps, **kw) for o in ORDERS}
    assert runs["shuffle"]["layout"] == ("shuffle", True)
    assert runs["input"]["layout"] == ("input", False)
    for o in ORDERS[1:]:
        _same(runs["input"], runs[o])
    return runs["input"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("dim", [2, 3])
def test_walls_clamps_extforce(precision, dim):
    s = setups.small_pair(dim=dim, r=2.5e-4 if dim == 2 else 1.6e-4, wall=True, extforce=True, clamp=True)
    r = _check(s, 200, dt=2e-8, enable_fracture=1, precision=precision)
    assert np.abs(r["reaction"]).max() > 0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fracture_selfcontact_torque(precision):
    s = setups.small_pair(dim=2, speed=60.0, clamp=True, torque=True, extforce=True)
    r = _check(s, 300, dt=2e-8, enable_fracture=1, enable_torque=1, gradient_extforce=1, extforce_maxstep=150,
               precision=precision)
    assert (r["break_step"] > 0).sum() > 0 and r["pairs"][0].sum() > 0


def test_nl_bdry_only_and_grid_search():
    s = setups.small_pair(dim=2, speed=50.0)
    _check(s, 250, dt=2e-8, enable_fracture=1, nl_bdry_only=1, contact_skin=0.0)


def test_worm_loop():
    s = setups.small_pair(dim=2, speed=20.0, extforce=True)
    _check(s, 150, dt=2e-8, enable_fracture=1, timeloop="worm")


def test_hooks_and_host_writes():
    s = setups.small_pair(dim=2, speed=40.0, wall=True)

    def hook(g, steps):
        g.step(steps // 3)
        g.set_grain_flags(1, movable=0)
        g.step(steps // 3)
        g.set_grain_flags(1, movable=1, stoppable=1)
        v = g.field("vel")
        g.set_field("vel", v * 0.5)
        g.step(steps - 2 * (steps // 3))

    for precision in ("fp64", "mixed"):
        _check(s, 150, hook=hook, dt=2e-8, enable_fracture=1, precision=precision)


def test_batched_mixed_ensemble():
    s = setups.concat([setups.small_pair(dim=2, seed=81 + k, wall=k % 2 == 1, speed=35.0 + 5 * k) for k in range(4)])
    _check(s, 200, dt=2e-8, enable_fracture=1, precision="mixed", contact_skin=0.25)


def test_shuffled_layout_bitexact_against_oracle():
    s = setups.two_disk_collision()
    kw = dict(dt=2e-8, enable_fracture=1)
    g = Simulation(s, record_pairs=True, pair_log_capacity=400, node_order="shuffle", **kw)
    r = O.OracleSim(s, **kw)
    g.step(400)
    r.step(400)
    for f in ("CurrPos", "vel", "acc", "force"):
        assert np.array_equal(g.field(f), r.field(f)), f
    assert np.array_equal(g.bond_alive(), r.bond_alive())
    assert np.array_equal(g.break_step(), r.break_step())
    c, h = g.pair_log(400)
    rc, rh = r.pair_log_all()
    assert np.array_equal(c, rc) and np.array_equal(h, rh) and rc.sum() > 0


def test_gradient_independent_of_layout():
    s = setups.compaction_2d(n_grains=6, r=0.3e-3, nodes_per_grain=120, seed=11)
    gs = []
    for order in ("input", "shuffle"):
        sim = Simulation(s, dt=2e-8, enable_fracture=1, precision="mixed", node_order=order)
        run = grad.GradRun(sim, 200, checkpoint_every=50)
        r0, ke0 = run.forward()
        wr = np.ones_like(r0) / max(np.abs(r0).max(), 1e-30)
        vb = np.linspace(-1.0, 1.0, s.n_nodes * s.dim).reshape(s.n_nodes, s.dim)
        gs.append(run.backward(reaction_bar=wr, ke_bar=1.0 / ke0, vel_bar=vb))
        sim.close()
    assert np.abs(gs[0]).max() > 0
    assert np.array_equal(gs[0], gs[1])
