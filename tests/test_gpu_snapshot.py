"""Asynchronous snapshots (pg_snapshot / pg_wait): every item equals what the synchronous getters
return after the same steps, also when more steps are issued before the wait, into page-locked and
into ordinary host buffers, for both precisions in 2D and 3D."""
import numpy as np
import pytest

from perigrain_gb300 import Simulation, setups

pytestmark = pytest.mark.gpu
ITEMS = ("CurrPos", "vel", "acc", "force", "disp", "bond_alive", "wall", "reaction")


def _sync_state(sim):
    out = {k: sim.field(k) for k in ("CurrPos", "vel", "acc", "force", "disp")}
    out["bond_alive"] = sim.bond_alive()
    out["wall"] = sim.wall()
    out["reaction"] = sim.reaction()
    out["too_close_events"] = sim.device_status()[1]
    return out


def _setup(dim):
    parts = [setups.small_pair(dim=dim, seed=41 + k, wall=True, speed=40.0, clamp=(k == 0)) for k in range(3)]
    return setups.concat(parts)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("pinned", [True, False])
def test_snapshot_equals_getters(precision, dim, pinned):
    s = _setup(dim)
    sim = Simulation(s, dt=2e-8, enable_fracture=1, precision=precision)
    sim.step(150)
    ref = _sync_state(sim)
    out = sim.snapshot_buffers(ITEMS) if pinned else None
    snap = sim.snapshot(ITEMS, out=out)
    sim.step(37)  # issued before the wait: must not leak into the snapshot
    got = snap.wait()
    assert got["last_step"] == 150
    for k in ITEMS:
        assert got[k].shape == ref[k].shape, k
        assert np.array_equal(got[k], ref[k]), k
    assert got["too_close_events"] == ref["too_close_events"]
    if dim == 2:
        assert (got["bond_alive"] == 0).any()  # bonds broke: the alive bytes are not trivially all ones
    # the later steps did run
    assert not np.array_equal(sim.field("CurrPos"), ref["CurrPos"])
    sim.close()


def test_second_snapshot_completes_the_first():
    s = _setup(2)
    sim = Simulation(s, dt=2e-8, enable_fracture=1, precision="mixed")
    sim.step(20)
    a_ref = sim.field("vel")
    a = sim.snapshot(("vel",))
    sim.step(20)
    b = sim.snapshot(("vel", "reaction"))  # completes a first
    ga = a.wait()
    assert np.array_equal(ga["vel"], a_ref) and ga["last_step"] == 20
    gb = b.wait()
    assert gb["last_step"] == 40
    assert np.array_equal(gb["vel"], sim.field("vel"))
    assert np.array_equal(gb["reaction"], sim.reaction())
    sim.close()


def test_snapshot_rejects_bad_buffers():
    s = _setup(2)
    sim = Simulation(s, dt=2e-8, precision="fp64")
    with pytest.raises(ValueError):
        sim.snapshot(("nope",))
    with pytest.raises(ValueError):
        sim.snapshot(("vel",), out={"vel": np.empty((s.n_nodes, 2), np.float32)})
    sim.close()
