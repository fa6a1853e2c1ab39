"""Failure detection without a GPU fault: the cooperative grid build's barrier waits are bounded;
a barrier that cannot complete (its arrival count preset from the host) ends the step with
PG_ETIMEOUT in the status word, the kernel returns and the context stays usable. The timed-out
handle is halted: grid builds already enqueued return at entry and further steps are refused."""
import time

import pytest

from perigrain_gb300 import Simulation, setups
from perigrain_gb300 import _native as N

pytestmark = pytest.mark.gpu


def test_grid_barrier_wait_times_out_into_status():
    s = setups.small_pair(dim=2, seed=71)
    sim = Simulation(s, dt=2e-8, enable_fracture=1, precision="mixed", contact_skin=0.25)
    N.check(N.lib().pg_debug_grid_barrier(sim.h, 1 << 30))
    t0 = time.perf_counter()
    sim.step(1)  # the first step rebuilds the lists: its first grid barrier cannot complete
    # steps enqueued before the host has seen the timeout: their grid builds return at entry (the
    # barrier holds stale arrivals), so none of them can release a barrier early
    sim.step(3)
    with pytest.raises(N.PerigrainError) as e:
        sim.synchronize()
    assert e.value.code == N.PG_ETIMEOUT
    assert time.perf_counter() - t0 < 60.0
    # the host refuses further steps on the halted handle
    with pytest.raises(N.PerigrainError) as e:
        sim.step(2)
    assert e.value.code == N.PG_ETIMEOUT
    assert sim.device_status()[0] == N.PG_ETIMEOUT
    with pytest.raises(N.PerigrainError) as e:
        sim.step(1)
    assert e.value.code == N.PG_ETIMEOUT
    sim.close()
    # the context is intact: a new handle runs and agrees with the one-shot reference state
    a = Simulation(s, dt=2e-8, enable_fracture=1, precision="mixed", contact_skin=0.25)
    a.step(20)
    a.synchronize()
    assert a.device_status()[0] == 0
    a.close()


def test_debug_hook_needs_the_cooperative_build():
    s = setups.small_pair(dim=2, seed=72)
    sim = Simulation(s, dt=2e-8, precision="mixed", contact_skin=0.0)
    assert N.lib().pg_debug_grid_barrier(sim.h, 1) == N.PG_EINVAL
    sim.close()
