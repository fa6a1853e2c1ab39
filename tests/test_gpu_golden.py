"""The GPU engine against the reference's own outputs (tests/golden/*.npz), in-process through
the C ABI and as the drop-in executables (bin/simulate2d, bin/simulate3d) writing tc_/wall_ files.

Non-wall cases are bit-exact. Wall cases call pow/asin (CUDA vs the reference's libm), so they
are compared with relative tolerance WALL_RTOL on state and 1e-7 on reactions."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import _oracle as O
from golden.make_golden import CASES, case_kwargs, case_setup
from perigrain_gb300 import Simulation, h5

pytestmark = pytest.mark.gpu
WALL_CASES = {"wall2d_full", "wall3d"}
WALL_RTOL = 1e-9
BIN = os.path.join(O.ROOT, "perigrain_gb300", "bin")


def _check_state(name, k, z, fields, reaction, wall, conn):
    exact = name not in WALL_CASES
    for f, a in fields.items():
        b = z["%d/%s" % (k, f)]
        if exact:
            assert np.array_equal(a, b), (name, k, f, np.abs(a - b).max())
        else:
            assert np.abs(a - b).max() <= WALL_RTOL * max(np.abs(b).max(), 1e-300), (name, k, f)
    zr = z["%d/reaction" % k]
    if exact:
        assert np.array_equal(reaction, zr)
    else:
        assert np.abs(reaction - zr).max() <= 1e-7 * max(np.abs(zr).max(), 1e-30)
    assert np.array_equal(wall, z["%d/wall_info" % k])
    for g, c in enumerate(conn or []):
        assert np.array_equal(c, z["%d/conn%d" % (k, g)]), (name, k, g)


@pytest.mark.parametrize("name", sorted(CASES))
def test_engine_matches_reference_outputs(name):
    z, meta = O.load_golden(name)
    s = case_setup(CASES[name])
    conf = meta["conf"]
    sim = Simulation(s, **case_kwargs(CASES[name], conf))
    worm = CASES[name].get("timeloop") == "worm"

    def check(k):
        fields = {f: sim.field(f) for f in ("CurrPos", "vel", "acc", "force")}
        conn = None if worm else O.conn_from_alive(s, sim.bond_alive())
        _check_state(name, k, z, fields, sim.reaction()[0], sim.wall()[0], conn)

    O.drive(sim, conf, s.n_grains, check)


@pytest.mark.parametrize("name", sorted(CASES))
def test_dropin_executable_matches_reference_files(name):
    z, meta = O.load_golden(name)
    s = case_setup(CASES[name])
    conf = meta["conf"]
    d = tempfile.mkdtemp(prefix="dropin_")
    O.make_case_dir(d, s, conf)
    exe = os.path.join(BIN, "simulate%dd" % s.dim)
    worm = CASES[name].get("timeloop") == "worm"
    env = dict(os.environ, PERIGRAIN_TIMELOOP="worm") if worm else None
    r = subprocess.run([exe], cwd=d, capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "Runtime:" in r.stdout
    out = os.path.join(d, "output", "hdf5")
    flc = h5.read(os.path.join(out, "plotinfo.h5"), "f_l_counter", np.uint32).ravel()
    assert flc.tolist() == [1, conf["timesteps"] // conf["modulo"]]
    assert h5.read(os.path.join(out, "plotinfo.h5"), "dimension", np.uint32).ravel()[0] == s.dim
    for k in range(1, conf["timesteps"] // conf["modulo"] + 1):
        tc = O.read_tc(d, k, s.n_grains, s.dim, connectivity=not worm)
        fields = {f: tc[f] for f in ("CurrPos", "vel", "acc", "force")}
        _check_state(name, k, z, fields, tc["reaction"], tc["wall_info"], tc.get("Connectivity"))
    rt = h5.read(os.path.join(out, "run_time.h5"), "t_ind", np.float64).ravel()
    assert rt.tolist() == [float(conf["modulo"] * (k + 1)) for k in range(len(rt))]


def test_dropin_resume():
    """do_resume + wall_resume: restart from tc_00002.h5 / wall_00002.h5 and continue; the
    result equals the oracle started from the state the reference rebuilds on resume."""
    name = "wall2d_full"
    z, meta = O.load_golden(name)
    s = case_setup(CASES[name])
    conf = dict(meta["conf"])
    d = tempfile.mkdtemp(prefix="resume_")
    O.make_case_dir(d, s, conf)
    exe = os.path.join(BIN, "simulate2d")
    assert subprocess.run([exe], cwd=d, capture_output=True, timeout=300).returncode == 0
    tc2 = O.read_tc(d, 2, s.n_grains, s.dim)
    conf2 = dict(conf, do_resume=1, resume_ind=2, wall_resume=1, timesteps=100)
    O.write_conf(os.path.join(d, "config", "main.conf"), conf2)
    r = subprocess.run([exe], cwd=d, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:]
    assert "Resuming from counter 3" in r.stdout
    rs = O.resumed_setup(s, tc2, tc2["wall_info"])
    sim = O.OracleSim(rs, **O.engine_kwargs(conf2))
    sim.step(conf2["modulo"])
    tc3 = O.read_tc(d, 3, s.n_grains, s.dim)
    for f in ("CurrPos", "vel"):
        assert np.abs(tc3[f] - sim.field(f)).max() <= WALL_RTOL * np.abs(sim.field(f)).max(), f
    for a, b in zip(tc3["Connectivity"], O.conn_from_alive(rs, sim.bond_alive())):
        assert np.array_equal(a, b)
