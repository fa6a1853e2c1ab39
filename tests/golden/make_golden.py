"""Generate the golden fixtures: outputs of the reference simulator itself.

Each case builds a small seeded setup (perigrain_gb300.setups), writes data/hdf5/all.h5 and
config/main.conf, runs the reference (debdeepbh/perigrain's own src/ headers and run/ drivers,
compiled unmodified against the project's Eigen/HDF5 API shims by oracle/Makefile) and stores
every tc_%05u.h5 / wall_%05u.h5 it writes into tests/golden/<case>.npz.

Needs the reference build of oracle/Makefile (the reference checkout is named by PERIGRAIN_REFERENCE
or the recipe's default). Run from the repository root:
    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from perigrain_gb300 import setups  # noqa: E402
import _oracle as O  # noqa: E402

BASE = dict(dt=2e-8, is_parallel=0, enable_fracture=1, save_file=1)

CASES = {
    "collide2d": dict(setup=dict(dim=2, speed=40.0), conf=dict(timesteps=300, modulo=100)),
    "wall2d_full": dict(setup=dict(dim=2, wall=True, clamp=True, torque=True, extforce=True),
                        conf=dict(timesteps=300, modulo=50, enable_torque=1, gradient_extforce=1,
                                  extforce_maxstep=150)),
    "wall3d": dict(setup=dict(dim=3, r=1.6e-4, wall=True, extforce=True), conf=dict(timesteps=200, modulo=50)),
    "nlbdry2d": dict(setup=dict(dim=2, speed=50.0), conf=dict(timesteps=250, modulo=125, nl_bdry_only=1)),
    "hooks2d": dict(setup=dict(dim=2, speed=40.0), movable={1: 0}, stoppable={0: 0},
                    conf=dict(timesteps=300, modulo=100, set_movable_index=1, set_movable_timestep=120,
                              set_stoppable_index=0, set_stoppable_timestep=80, allow_damping=0)),
    "nofracture2d": dict(setup=dict(dim=2, speed=60.0), conf=dict(timesteps=200, modulo=100, enable_fracture=0,
                                                                  allow_friction=0)),
    # run_timeloop_worm (timeloop.h:1018-1369): both gait phases (t < 1000 and t >= 1000), external
    # force gated by the phase, and a grain that is not stoppable still in contact
    "worm2d": dict(setup=dict(dim=2, speed=30.0, extforce=True), stoppable={1: 0}, timeloop="worm",
                   conf=dict(timesteps=1200, modulo=200)),
}


def case_setup(spec):
    s = setups.small_pair(**spec["setup"])
    for g, v in spec.get("movable", {}).items():
        s.movable[g] = v
    for g, v in spec.get("stoppable", {}).items():
        s.stoppable[g] = v
    return s


def case_kwargs(spec, conf):
    """Engine / oracle keyword arguments of a case (the time-loop variant is not a config key)."""
    kw = O.engine_kwargs(conf)
    if spec.get("timeloop") == "worm":
        kw["timeloop"] = 1
    return kw


def case_conf(spec, s):
    c = dict(BASE)
    c.update(spec["conf"])
    return O.conf_for(s, **c)


def setup_digest(s):
    h = hashlib.sha256()
    for k in ("pos", "vol", "bond_offset", "bond_local", "bdry_nodes", "vel", "extforce"):
        h.update(np.ascontiguousarray(getattr(s, k)).tobytes())
    return h.hexdigest()


def main(names=None):
    O.build_oracle()
    for name, spec in CASES.items():
        if names and name not in names:
            continue
        s = case_setup(spec)
        conf = case_conf(spec, s)
        d = tempfile.mkdtemp(prefix="golden_")
        O.make_case_dir(d, s, conf)
        O.run_reference(d, s.dim, timeloop=spec.get("timeloop"))
        out = {"meta": np.frombuffer(json.dumps(dict(conf=conf, spec=spec, digest=setup_digest(s))).encode(),
                                     np.uint8)}
        nsnap = conf["timesteps"] // conf["modulo"]
        worm = spec.get("timeloop") == "worm"  # the worm loop writes no Connectivity
        for k in range(1, nsnap + 1):
            tc = O.read_tc(d, k, s.n_grains, s.dim, connectivity=not worm)
            for f in ("CurrPos", "vel", "acc", "force", "wall_info", "reaction"):
                out["%d/%s" % (k, f)] = tc[f]
            for g, c in enumerate(tc.get("Connectivity", [])):
                out["%d/conn%d" % (k, g)] = c
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, s.n_nodes, "nodes", nsnap, "snapshots")


if __name__ == "__main__":
    main(sys.argv[1:])
