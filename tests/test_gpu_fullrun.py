"""The two-disk collision (two 1249-node disks, +-20 m/s head-on, fracture and self-contact on, no
wall) over its whole configured run of 20,000 steps (the disks meet once and rebound).

The FP64 GPU path against the oracle (the CPU restatement pinned bit for bit to the reference):
everything in this configuration is IEEE +, -, *, / and sqrt, so the bar is bit-exact for the
whole run, not only the first 1000 steps -- positions, velocities, accelerations and forces every
1000 steps; the alive-bond set and the step at which each bond broke; the per-step contact-pair
log (count and hash) of all 20,000 steps; the "nodes too close" count; a clean device status.

The mixed-precision path over the same whole run: momentum conservation and the energy bound of
this wall-free collision, and its statistics against an ensemble of FP64 runs perturbed at FP32
resolution (the tolerance is stated below)."""
import numpy as np
import pytest

import _oracle as O
from perigrain_gb300 import Simulation, setups

pytestmark = pytest.mark.gpu

STEPS = setups.WORKLOADS[0]["steps"]  # 20,000
DT = setups.WORKLOADS[0]["dt"]
FIELDS = ("CurrPos", "vel", "acc", "force")


def test_collision_whole_run_fp64_bitexact():
    s = setups.two_disk_collision()
    kw = dict(dt=DT, enable_fracture=1)
    g = Simulation(s, record_pairs=True, pair_log_capacity=STEPS, **kw)
    r = O.OracleSim(s, **kw)
    for k in range(STEPS // 1000):
        g.step(1000)
        r.step(1000)
        for f in FIELDS:
            a, b = g.field(f), r.field(f)
            assert np.array_equal(a, b), "step %d: %s differs, max |diff| %g" % ((k + 1) * 1000, f,
                                                                                 np.abs(a - b).max())
    assert np.array_equal(g.bond_alive(), r.bond_alive())
    bs = r.break_step()
    assert np.array_equal(g.break_step(), bs)
    c, h = g.pair_log(STEPS)
    rc, rh = r.pair_log_all()
    assert len(rc) == STEPS
    assert np.array_equal(c, rc) and np.array_equal(h, rh)
    st, tc = g.device_status()
    assert st == 0 and tc == r.too_close()
    # the run is a real collision (the disks meet once, within the first 1000 steps, and rebound;
    # at +-20 m/s no bond reaches the critical stretch)
    assert (rc > 0).sum() > 50


# Whole-run tolerance of the mixed path. The collision's outcome is chaotic in FP64 itself: FP64
# runs whose initial velocities differ at round-off level already separate by several percent
# after the disks part. The mixed run is therefore compared with an ensemble of FP64 runs whose
# initial velocities are moved by 2^-24 max|v0| (FP32 resolution, seeded random signs): each
# statistic of the mixed run must differ from the FP64 run by at most max(2 x the ensemble's
# largest difference, STAT_FLOOR). Momentum and the energy bound are laws, checked directly.
MOMENTUM_TOL = 1e-6
STAT_FLOOR = 1e-3
MEMBERS = 6


def _perturbed(s, seed):
    p = s.copy()
    rng = np.random.default_rng(1000 + seed)
    p.vel = s.vel + 2.0 ** -24 * max(np.abs(s.vel).max(), 1.0) * rng.choice([-1.0, 1.0], size=s.vel.shape)
    return p


def test_collision_whole_run_mixed_statistics():
    s = setups.two_disk_collision()
    kw = dict(dt=DT, enable_fracture=1)
    runs = {"mixed": Simulation(s, precision="mixed", **kw), "fp64": Simulation(s, precision="fp64", **kw)}
    for k in range(MEMBERS):
        runs["ens%d" % k] = Simulation(_perturbed(s, k), precision="fp64", **kw)
    D = s.dim
    gsize = np.diff(s.grain_node_offset.astype(np.int64))
    m = (s.vol * np.repeat(s.rho, gsize))[:, None]
    starts = s.grain_node_offset[:-1].astype(np.int64)
    v0 = s.vel.reshape(-1, D)
    p0 = (m * v0).sum(0)
    pscale = (m * np.abs(v0)).sum()
    ke0 = 0.5 * (m[:, 0] * (v0 * v0).sum(1)).sum()
    ke = {p: [] for p in runs}
    for _ in range(STEPS // 500):
        for sim in runs.values():
            sim.step(500)
        for p, sim in runs.items():
            v = sim.field("vel")
            # no wall, equal and opposite pair forces: momentum is conserved; no energy source:
            # kinetic energy never exceeds the initial (all-kinetic) energy
            assert np.abs((m * v).sum(0) - p0).max() <= MOMENTUM_TOL * pscale, p
            ke[p].append(0.5 * (m[:, 0] * (v * v).sum(1)).sum())
            assert ke[p][-1] <= ke0 * (1 + 1e-6), p
    kes = {p: np.array(v) for p, v in ke.items()}
    gv = {p: np.add.reduceat(m * sim.field("vel"), starts, axis=0) / np.add.reduceat(m, starts, axis=0)
          for p, sim in runs.items()}
    gx = {p: np.add.reduceat(m * sim.field("CurrPos"), starts, axis=0) / np.add.reduceat(m, starts, axis=0)
          for p, sim in runs.items()}

    def rel(a, b):
        return np.abs(a - b).max() / np.abs(b).max()

    ens = ["ens%d" % k for k in range(MEMBERS)]
    for name, series in (("kinetic energy", kes), ("grain mean velocity", gv), ("grain centroid", gx)):
        err = rel(series["mixed"], series["fp64"])
        spread = max(rel(series[e], series["fp64"]) for e in ens)
        assert err <= max(2 * spread, STAT_FLOOR), (name, err, spread)
    for sim in runs.values():
        assert sim.bond_alive().all()  # at +-20 m/s no bond breaks, in any run
