"""Mixed precision (FP32 bond/contact forces, FP64 state) against the FP64 oracle.

The reference's contact dynamics are chaotic (tests/test_dynamics_sensitivity.py: a 1e-12
change of one node's velocity reaches 1e-3 relative position difference within ~250 steps of
contact, in pure FP64). A pointwise bound therefore holds only where the dynamics do not amplify
differences; there the stated tolerance is POS_RTOL = 1e-6 relative position error,
max|x - x_ref| / max|x_ref|. Over full collisions the checks are invariants (momentum) and
bit-identity of batched vs independent runs."""
import numpy as np
import pytest

import _oracle as O
from perigrain_gb300 import Simulation, setups

pytestmark = pytest.mark.gpu
POS_RTOL = 1e-6


def _pos_err(g, r):
    x, xr = g.field("CurrPos"), r.field("CurrPos")
    return np.abs(x - xr).max() / np.abs(xr).max()


def test_mixed_elastic_waves_1000_steps():
    """One grain with a shear velocity field: bonds stretch and compress, no contact."""
    s = setups.two_disk_collision()
    keep = int(s.grain_node_offset[1])
    one = setups.concat([s])  # copy, then cut to grain 0
    one = s.copy()
    D = 2
    one.grain_instance = s.grain_instance[:1]
    one.grain_node_offset = s.grain_node_offset[:2]
    for f in ("pos", "disp", "vel", "acc", "extforce"):
        setattr(one, f, getattr(s, f)[: keep * D].copy())
    one.vol = s.vol[:keep].copy()
    one.bond_offset = s.bond_offset[: keep + 1].copy()
    one.bond_local = s.bond_local[: int(s.bond_offset[keep])].copy()
    one.bdry_offset = s.bdry_offset[:2].copy()
    one.bdry_nodes = s.bdry_nodes[: int(s.bdry_offset[1])].copy()
    one.clamped_offset = s.clamped_offset[:2].copy()
    one.clamped_nodes = s.clamped_nodes[:0].copy()
    for f in ("delta", "rho", "cnot", "snot", "movable", "breakable", "stoppable", "break_bonds", "torque_axis",
              "torque_val"):
        setattr(one, f, getattr(s, f)[:1].copy())
    p = one.pos.reshape(-1, 2)
    v = np.zeros_like(p)
    v[:, 0] = 5.0 * np.sin(2 * np.pi * (p[:, 1] - p[:, 1].min()) / 1e-3)
    one.vel = v.reshape(-1)
    kw = dict(dt=2e-8, enable_fracture=1)
    g = Simulation(one, precision="mixed", **kw)
    r = O.OracleSim(one, **kw)
    for _ in range(10):
        g.step(100)
        r.step(100)
        assert _pos_err(g, r) <= POS_RTOL
    u = r.field("CurrPos") - one.pos.reshape(-1, 2)
    assert np.abs(u).max() > 1e-7  # the grain really deformed


def test_mixed_collision_through_contact_onset():
    """Two-disk collision up to 40 steps after first contact (contact starts near step 88)."""
    s = setups.two_disk_collision()
    kw = dict(dt=2e-8, enable_fracture=1)
    g = Simulation(s, precision="mixed", record_pairs=True, **kw)
    r = O.OracleSim(s, **kw)
    g.step(128)
    r.step(128)
    assert _pos_err(g, r) <= POS_RTOL
    c, _ = g.pair_log(128)
    assert c.sum() > 0 and np.array_equal(c, r.pair_log_all()[0])


def test_mixed_momentum_conserved_over_collision():
    """No wall, equal node volumes and densities: the reference's pair forces are equal and
    opposite, so total momentum is conserved; mixed precision must keep it within 1e-6 of the
    total momentum magnitude sum over 1000 steps of a fracturing collision."""
    s = setups.two_disk_collision()
    g = Simulation(s, precision="mixed", dt=2e-8, enable_fracture=1)
    m = (s.vol * np.repeat(s.rho, np.diff(s.grain_node_offset)))[:, None]
    v0 = s.vel.reshape(-1, 2)
    scale = (m * np.abs(v0)).sum()
    p0 = (m * v0).sum(0)
    for _ in range(10):
        g.step(100)
        p = (m * g.field("vel")).sum(0)
        assert np.abs(p - p0).max() <= 1e-6 * scale


@pytest.mark.parametrize("dim", [2, 3])
def test_mixed_small_with_walls(dim):
    s = setups.small_pair(dim=dim, r=2.5e-4 if dim == 2 else 1.6e-4, wall=True, extforce=True, clamp=True)
    kw = dict(dt=2e-8, enable_fracture=1)
    g = Simulation(s, precision="mixed", **kw)
    r = O.OracleSim(s, **kw)
    for _ in range(4):
        g.step(25)
        r.step(25)
        assert _pos_err(g, r) <= POS_RTOL
    assert np.array_equal(g.wall(), r.wall())
    rr = r.reaction()
    assert np.abs(g.reaction() - rr).max() <= 1e-4 * max(np.abs(rr).max(), 1e-30) + 1e-30


def test_mixed_batched_equals_independent():
    parts = [setups.small_pair(dim=2, seed=31 + k, speed=35.0 + 5 * k) for k in range(3)]
    batch = setups.concat(parts)
    gb = Simulation(batch, dt=2e-8, enable_fracture=1, precision="mixed")
    gb.step(200)
    cur = gb.field("CurrPos")
    off = 0
    for p in parts:
        gi = Simulation(p, dt=2e-8, enable_fracture=1, precision="mixed")
        gi.step(200)
        assert np.array_equal(cur[off:off + p.n_nodes], gi.field("CurrPos"))
        off += p.n_nodes


def test_mixed_settling_with_gravity_and_walls():
    """A slice of the 2D settling workload: 40 grains falling under gravity in the walled box."""
    s = setups.settling_2d(n_grains=40)
    kw = dict(dt=1e-8, enable_fracture=1)
    g = Simulation(s, precision="mixed", **kw)
    r = O.OracleSim(s, **kw)
    g.step(300)
    r.step(300)
    assert _pos_err(g, r) <= POS_RTOL


def test_mixed_block_size_does_not_change_results():
    """Per-node arithmetic does not depend on the launch shape: block sizes 64 and 128 (different
    shared-memory neighbour windows in 2D, different grids) give identical runs."""
    s = setups.concat([setups.small_pair(dim=2, seed=51 + k, wall=True, speed=35.0) for k in range(3)])
    runs = []
    for b in (64, 128):
        g = Simulation(s, dt=2e-8, enable_fracture=1, precision="mixed", block_size=b)
        g.step(300)
        runs.append(g)
    for f in ("CurrPos", "vel", "acc", "force"):
        assert np.array_equal(runs[0].field(f), runs[1].field(f)), f
    assert np.array_equal(runs[0].bond_alive(), runs[1].bond_alive())


@pytest.mark.parametrize("dim", [2, 3])
def test_mixed_overlapped_graphs_equal_serial_launches(dim):
    """The CUDA graphs run each step's finalize (wall move, grid refit, box reset) beside the next
    step's position update; the serial launch sequence of the timed mode gives identical runs,
    moving walls and list rebuilds included."""
    s = setups.concat([setups.small_pair(dim=dim, seed=61 + k, wall=True, speed=35.0) for k in range(3)])
    runs = []
    for timed in (False, True):
        g = Simulation(s, dt=2e-8, enable_fracture=1, precision="mixed", contact_skin=0.25)
        g.set_timing(timed)
        g.step(160)
        runs.append(g)
    a, b = runs
    for f in ("CurrPos", "vel", "acc", "force", "disp"):
        assert np.array_equal(a.field(f), b.field(f)), f
    assert np.array_equal(a.bond_alive(), b.bond_alive())
    assert np.array_equal(a.reaction(), b.reaction()) and np.array_equal(a.wall(), b.wall())
    assert a.device_status() == b.device_status()
