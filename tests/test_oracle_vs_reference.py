"""Live differential runs of the oracle against the reference simulator compiled from its own
sources (needs the reference checkout; skipped elsewhere). Wider than the golden fixtures:
more seeds and shapes, and the is_parallel=1 OpenMP path of the reference without walls."""
import os
import tempfile

import numpy as np
import pytest

import _oracle as O
from perigrain_gb300 import setups

# the reference simulator built from its own sources by oracle/Makefile (absent where the reference
# checkout is absent)
O.build_oracle()
pytestmark = pytest.mark.skipif(not all(os.path.exists(O.REF_BIN[k]) for k in (2, 3)),
                                reason="reference build (oracle/_ref) not present")


def _compare(s, conf):
    d = tempfile.mkdtemp(prefix="refcmp_")
    O.make_case_dir(d, s, conf)
    O.run_reference(d, s.dim)
    sim = O.OracleSim(s, **O.engine_kwargs(conf))

    def check(k):
        ref = O.read_tc(d, k, s.n_grains, s.dim)
        for f in ("CurrPos", "vel", "acc", "force"):
            assert np.array_equal(sim.field(f), ref[f]), (k, f)
        assert np.array_equal(sim.reaction()[0], ref["reaction"])
        assert np.array_equal(sim.wall()[0], ref["wall_info"])
        for a, b in zip(O.conn_from_alive(s, sim.bond_alive()), ref["Connectivity"]):
            assert np.array_equal(a, b)

    O.drive(sim, conf, s.n_grains, check)


@pytest.mark.parametrize("seed", [21, 22, 23])
def test_random_pairs_2d(seed):
    rng = np.random.default_rng(seed)
    s = setups.small_pair(dim=2, seed=seed, speed=float(rng.uniform(20, 70)), wall=bool(seed % 2),
                          n_grains=3, extforce=True)
    conf = O.conf_for(s, timesteps=200, modulo=100, dt=2e-8, is_parallel=0, enable_fracture=1)
    _compare(s, conf)


def test_three_d_collision():
    s = setups.small_pair(dim=3, r=1.4e-4, speed=50.0)
    conf = O.conf_for(s, timesteps=150, modulo=75, dt=2e-8, is_parallel=0, enable_fracture=1)
    _compare(s, conf)


def test_reference_openmp_path_no_wall():
    """Without walls the reference's OpenMP grain loop has no shared accumulator, so its parallel
    run must equal the serial oracle too."""
    s = setups.small_pair(dim=2, seed=5, speed=45.0, n_grains=4)
    conf = O.conf_for(s, timesteps=150, modulo=50, dt=2e-8, is_parallel=1, enable_fracture=1)
    _compare(s, conf)


def test_resume_semantics():
    """The reference's resume (timeloop.h:508-550) equals the oracle started from
    resumed_setup(): disp = CurrPos - pos, vel/acc/Connectivity/wall from the files."""
    s = setups.small_pair(dim=2, seed=9, speed=50.0, wall=True, extforce=True)
    conf = O.conf_for(s, timesteps=200, modulo=100, dt=2e-8, is_parallel=0, enable_fracture=1)
    d = tempfile.mkdtemp(prefix="refres_")
    O.make_case_dir(d, s, conf)
    O.run_reference(d, 2)
    tc1 = O.read_tc(d, 1, s.n_grains, 2)
    conf2 = dict(conf, do_resume=1, resume_ind=1, wall_resume=1, timesteps=150)
    O.write_conf(os.path.join(d, "config", "main.conf"), conf2)
    out = O.run_reference(d, 2)
    assert "Resuming from counter 2" in out
    rs = O.resumed_setup(s, tc1, tc1["wall_info"])
    sim = O.OracleSim(rs, **O.engine_kwargs(conf2))
    sim.step(100)
    ref = O.read_tc(d, 2, s.n_grains, 2)
    for f in ("CurrPos", "vel", "acc", "force"):
        assert np.array_equal(sim.field(f), ref[f]), f
    assert np.array_equal(sim.reaction()[0], ref["reaction"])
