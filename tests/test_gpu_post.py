"""On-device post-processing (pg_postprocess) against the reference's numpy formulas applied to the
downloaded state, and the drop-in executable's timestep_data.h5 against the same formulas applied
to its own tc_/wall_ files (what gen_timestep_data.py, gen_damage_data.py and read_force_val in
read_sim_output.py compute). Sums are reduced in a different order than numpy's, so the bound is
relative, REL."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import _oracle as O
from perigrain_gb300 import Simulation, h5, setups

pytestmark = pytest.mark.gpu
REL = 1e-12
BIN = os.path.join(O.ROOT, "perigrain_gb300", "bin")


def _close(a, b, scale=0.0):
    """|a - b| <= REL * max(|b|, scale); sums whose terms cancel (internal forces) pass the sum of
    the terms' magnitudes as scale."""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    assert a.shape == b.shape
    assert np.abs(a - b).max() <= REL * max(np.abs(b).max(), scale, 1e-300), np.abs(a - b).max()


def _damage(setup, alive):
    """total_neighbors (read_sim_output.py:10-21) now against at creation, per node."""
    deg0 = np.diff(setup.bond_offset.astype(np.int64)).astype(np.float64)
    row = np.repeat(np.arange(setup.n_nodes), np.diff(setup.bond_offset.astype(np.int64)))
    deg = np.bincount(row, weights=alive.astype(np.float64), minlength=setup.n_nodes)
    with np.errstate(invalid="ignore", divide="ignore"):
        return (deg0 - deg) / deg0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("dim", [2, 3])
def test_postprocess_matches_numpy(precision, dim):
    parts = [setups.small_pair(dim=dim, seed=31 + k, wall=True, speed=40.0) for k in range(2)]
    s = setups.concat(parts)
    sim = Simulation(s, dt=2e-8, enable_fracture=1, precision=precision)
    sim.step(400)
    p = sim.postprocess(node_damage=True)
    off = np.asarray(s.grain_node_offset, np.int64)
    vel, acc, cur, force = (sim.field(f) for f in ("vel", "acc", "CurrPos", "force"))
    vol = np.asarray(s.vol, np.float64)
    rho = np.asarray(s.rho, np.float64)
    dmg = _damage(s, sim.bond_alive())
    assert np.array_equal(np.isnan(p["node_damage"]), np.isnan(dmg))
    ok = ~np.isnan(dmg)
    _close(p["node_damage"][ok], dmg[ok])
    if dim == 2:
        assert dmg[ok].max() > 0  # some bonds broke (the 3D pair stays intact at this speed)
    inert = np.zeros((s.n_instances, dim))
    inert_abs = 0.0
    vol_inst = np.zeros(s.n_instances)
    for g in range(s.n_grains):
        sl = slice(off[g], off[g + 1])
        _close(p["grain_mean_vel"][g], vel[sl].mean(axis=0))
        _close(p["grain_mean_acc"][g], acc[sl].mean(axis=0))
        _close(p["grain_mean_currpos"][g], cur[sl].mean(axis=0))
        _close(p["grain_force"][g], force[sl].sum(axis=0), np.abs(force[sl]).sum())
        _close(p["grain_damage"][g], np.mean(dmg[sl]))
        k = s.grain_instance[g]
        inert[k] += np.sum((vol[sl] * rho[g])[:, None] * acc[sl], axis=0)
        inert_abs += np.abs((vol[sl] * rho[g])[:, None] * acc[sl]).sum()
        vol_inst[k] += vol[sl].sum()
    _close(p["inertial_force"], inert, inert_abs)
    wi = sim.wall()
    if dim == 2:
        wv = (wi[:, 1] - wi[:, 0]) * (wi[:, 2] - wi[:, 3])
    else:
        wv = (wi[:, 1] - wi[:, 0]) * (wi[:, 3] - wi[:, 2]) * (wi[:, 5] - wi[:, 4])
    _close(p["volume_fraction"], vol_inst / wv)


def test_dropin_timestep_data_matches_output_files():
    s = setups.small_pair(dim=2, wall=True, speed=40.0, seed=41)
    conf = O.conf_for(s, timesteps=600, modulo=100, dt=2e-8, enable_fracture=1, is_parallel=0)
    d = tempfile.mkdtemp(prefix="tsd_")
    O.make_case_dir(d, s, conf)
    env = dict(os.environ, PERIGRAIN_TIMESTEP_DATA="1")
    r = subprocess.run([os.path.join(BIN, "simulate2d")], cwd=d, capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stdout + r.stderr
    fn = os.path.join(d, "output", "hdf5", "timestep_data.h5")
    T, G = 6, s.n_grains
    tm = h5.read(fn, "time").ravel()
    _close(tm, np.arange(1, T + 1) * 2e-8 * 100)
    off = np.asarray(s.grain_node_offset, np.int64)
    vol = np.asarray(s.vol, np.float64)
    rho = np.asarray(s.rho, np.float64)
    fields = {k: h5.read(fn, k) for k in ("wall_loc", "wall_force", "particle_damage", "particle_force",
                                           "particle_mean_vel", "particle_mean_acc", "particle_mean_CurrPos",
                                           "f_sum", "volume_fraction")}
    assert fields["particle_mean_vel"].shape == (T, G, 2)
    for t in range(1, T + 1):
        tc = O.read_tc(d, t, G, 2)
        np.testing.assert_array_equal(fields["wall_loc"][t - 1], tc["wall_info"])
        np.testing.assert_array_equal(fields["wall_force"][t - 1], tc["reaction"])
        fsum = np.zeros(2)
        fabs = 0.0
        for g in range(G):
            sl = slice(off[g], off[g + 1])
            _close(fields["particle_mean_vel"][t - 1, g], tc["vel"][sl].mean(axis=0))
            _close(fields["particle_mean_acc"][t - 1, g], tc["acc"][sl].mean(axis=0))
            _close(fields["particle_mean_CurrPos"][t - 1, g], tc["CurrPos"][sl].mean(axis=0))
            _close(fields["particle_force"][t - 1, g], tc["force"][sl].sum(axis=0), np.abs(tc["force"][sl]).sum())
            n = off[g + 1] - off[g]
            conn = tc["Connectivity"][g]
            deg = np.bincount(conn.ravel().astype(np.int64), minlength=n).astype(np.float64)
            row = np.diff(s.bond_offset.astype(np.int64))[sl].astype(np.float64)
            _close(fields["particle_damage"][t - 1, g], np.mean((row - deg) / row))
            fsum += np.sum((vol[sl] * rho[g])[:, None] * tc["acc"][sl], axis=0)
            fabs += np.abs((vol[sl] * rho[g])[:, None] * tc["acc"][sl]).sum()
        _close(fields["f_sum"][t - 1], fsum, fabs)
        wi = tc["wall_info"]
        _close(fields["volume_fraction"][t - 1], vol.sum() / ((wi[1] - wi[0]) * (wi[2] - wi[3])))
