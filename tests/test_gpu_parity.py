"""GPU engine vs the oracle (CPU restatement pinned bit-for-bit to the reference).

Bar: bit-exact for everything that involves only IEEE +, -, *, / and sqrt (bond force, bond
breaking, node-node contact with damping and friction, integrator): positions, velocities,
accelerations, forces, the alive-bond set, the step at which each bond broke and the per-step
contact-pair log (count and order-independent hash). Wall contact calls pow/asin, whose CUDA and
libm results may differ in the last ulp, so wall cases are compared with a relative tolerance.
"""
import numpy as np
import pytest

from perigrain_gb300 import Simulation, setups
import _oracle as O

pytestmark = pytest.mark.gpu

FIELDS = ("CurrPos", "vel", "acc", "force")
# relative position / velocity tolerance for runs that touch a wall (libm vs CUDA pow/asin)
WALL_RTOL = 1e-9


def _pair(s, steps, **kw):
    g = Simulation(s, record_pairs=True, pair_log_capacity=max(steps, 1), **kw)
    r = O.OracleSim(s, **kw)
    g.step(steps)
    r.step(steps)
    return g, r


def _assert_bitexact(g, r, steps):
    for f in FIELDS:
        a, b = g.field(f), r.field(f)
        assert np.array_equal(a, b), "%s differs: max |diff| %g" % (f, np.abs(a - b).max())
    assert np.array_equal(g.bond_alive(), r.bond_alive())
    assert np.array_equal(g.break_step(), r.break_step())
    c, h = g.pair_log(steps)
    rc, rh = r.pair_log_all()
    assert np.array_equal(c, rc[-steps:]) and np.array_equal(h, rh[-steps:])
    st, tc = g.device_status()
    assert st == 0
    assert tc == r.too_close()


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("dim", [2, 3])
def test_bitexact_no_wall(dim):
    s = setups.small_pair(dim=dim, r=2.5e-4 if dim == 2 else 1.6e-4, speed=40.0)
    g, r = _pair(s, 300, dt=2e-8, enable_fracture=1)
    _assert_bitexact(g, r, 300)
    assert r.pair_log_all()[0].sum() > 0  # contact happened


def test_bitexact_fracture_selfcontact_torque_clamp_extforce():
    s = setups.small_pair(dim=2, speed=60.0, clamp=True, torque=True, extforce=True)
    g, r = _pair(s, 400, dt=2e-8, enable_fracture=1, enable_torque=1, gradient_extforce=1, extforce_maxstep=150)
    _assert_bitexact(g, r, 400)
    assert (r.break_step() > 0).sum() > 0  # bonds broke


@pytest.mark.parametrize("flags", [dict(allow_damping=0), dict(allow_friction=0), dict(self_contact=0),
                                   dict(nl_bdry_only=1), dict(enable_fracture=0)])
def test_bitexact_flag_variants(flags):
    s = setups.small_pair(dim=2, speed=50.0)
    kw = dict(dt=2e-8, enable_fracture=1)
    kw.update(flags)
    g, r = _pair(s, 250, **kw)
    _assert_bitexact(g, r, 250)


@pytest.mark.parametrize("dim", [2, 3])
def test_wall_within_tolerance(dim):
    s = setups.small_pair(dim=dim, r=2.5e-4 if dim == 2 else 1.6e-4, wall=True, extforce=True)
    kw = dict(dt=2e-8, enable_fracture=1)
    g, r = Simulation(s, **kw), O.OracleSim(s, **kw)
    touched = 0
    for _ in range(30):
        g.step(10)
        r.step(10)
        for f in ("CurrPos", "vel"):
            assert _rel(g.field(f), r.field(f)) <= WALL_RTOL, f
        rr = r.reaction()
        assert np.abs(g.reaction() - rr).max() <= 1e-7 * max(np.abs(rr).max(), 1e-30)
        touched += int(np.abs(rr).max() > 0)
        assert np.array_equal(g.wall(), r.wall())
    assert np.array_equal(g.bond_alive(), r.bond_alive())
    assert touched > 0  # the wall was hit


def test_collision_1000_steps_bitexact():
    """Two-disk collision (2 x 1249 nodes): contact neighbour lists and broken-bond set match
    bit-exactly over the first 1000 steps."""
    s = setups.two_disk_collision()
    g, r = _pair(s, 1000, dt=2e-8, enable_fracture=1)
    _assert_bitexact(g, r, 1000)
    assert r.pair_log_all()[0].sum() > 0


def test_batched_equals_independent():
    """Instances batched in one handle evolve exactly as when run alone."""
    parts = [setups.small_pair(dim=2, seed=11 + k, speed=30.0 + 10 * k) for k in range(3)]
    batch = setups.concat(parts)
    gb = Simulation(batch, dt=2e-8, enable_fracture=1)
    gb.step(200)
    off = 0
    cur = gb.field("CurrPos")
    for p in parts:
        gi = Simulation(p, dt=2e-8, enable_fracture=1)
        gi.step(200)
        assert np.array_equal(cur[off:off + p.n_nodes], gi.field("CurrPos"))
        off += p.n_nodes


def test_grain_flag_hooks():
    s = setups.small_pair(dim=2, speed=40.0)
    s.movable[1] = 0
    kw = dict(dt=2e-8, enable_fracture=1)
    g, r = _pair(s, 100, **kw)
    g.set_grain_flags(1, movable=1)
    r.set_grain_flags(1, movable=1)
    g.step(100)
    r.step(100)
    for f in FIELDS:
        assert np.array_equal(g.field(f), r.field(f))


def _lists_case(kind):
    if kind == "collide":
        return setups.two_disk_collision(), dict(dt=2e-8, enable_fracture=1), 600
    if kind == "walls":
        return setups.concat([setups.small_pair(dim=2, seed=61 + k, wall=True, speed=40.0, clamp=(k == 0))
                              for k in range(3)]), dict(dt=2e-8, enable_fracture=1), 400
    if kind == "walls3d":
        return setups.small_pair(dim=3, r=1.6e-4, wall=True, speed=30.0), dict(dt=2e-8, enable_fracture=1), 300
    if kind == "nlbdry":
        return setups.small_pair(dim=2, speed=50.0, seed=62), dict(dt=2e-8, enable_fracture=1, nl_bdry_only=1), 400
    if kind == "worm":
        s = setups.small_pair(dim=2, speed=30.0, extforce=True, seed=63)
        s.stoppable[1] = 0
        return s, dict(dt=2e-8, enable_fracture=1, timeloop="worm"), 1200
    raise ValueError(kind)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("kind", ["collide", "walls", "walls3d", "nlbdry", "worm"])
def test_candidate_lists_do_not_change_results(kind, precision):
    """Contact candidate lists with a skin (rebuilt only when a node has moved 0.45 skin) give the
    same run as the per-step grid search, bit for bit, including the pair log."""
    s, kw, steps = _lists_case(kind)
    runs = []
    for skin in (0.0, 0.3, 1.0):
        g = Simulation(s, precision=precision, contact_skin=skin, record_pairs=True, pair_log_capacity=steps, **kw)
        g.step(steps)
        runs.append(g)
    a = runs[0]
    ca, ha = a.pair_log(steps)
    assert ca.sum() > 0
    for b in runs[1:]:
        for f in FIELDS:
            assert np.array_equal(a.field(f), b.field(f)), f
        assert np.array_equal(a.bond_alive(), b.bond_alive())
        assert np.array_equal(a.reaction(), b.reaction())
        cb, hb = b.pair_log(steps)
        assert np.array_equal(ca, cb) and np.array_equal(ha, hb)
        assert b.device_status()[0] == 0
