"""Benchmark: node-steps/s of the PeriDEM time step on one GB300 (or N, one process per GPU).

Default workload: the batched ensemble -- 256 independent two-grain collisions (disk / n-gon,
radius U(0.5, 1.5) mm, 200-1800 nodes per grain, impact speed U(5, 40) m/s, angle U(0, 60) deg),
all advanced together in one handle. A "step" is one time step of every instance.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload 0..4] [--precision fp64|mixed]
    python bench.py --impl reference ...   # the reference's CPU algorithm on the host cores

Prints one JSON line (rank 0). `value` is the mixed-precision batched path (FP32 forces, FP64
state), device-timed (CUDA events on the engine's stream, state resident in HBM, inputs larger
than L2), with block size and grid density picked by the project autotuner, over the workload's
whole configured run by default (10,000 steps for the ensemble: the cost of a step grows as the
collisions bring grains into contact). Beside it: the plain
FP64 path on the same batch (`plain_fp64`), 256 sequential single-instance FP64 runs
(`sequential_fp64`, timed on a sample of instances), and mixed-vs-FP64 errors of positions,
velocities and wall reactions over the whole configured run of every workload beside the spread of
FP64 runs perturbed at FP32 resolution (`accuracy`; the dynamics are chaotic). `e2e` goes
through the C ABI from host buffers: setup upload + the timed steps + a tc_-snapshot download
(CurrPos, vel, acc, force) every 100 steps.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "node-steps/s"
COMPARE_STEPS = 1000  # both paths are also timed over the first steps on their own
# Algorithmic bytes of the dominant kernel (the fused bond + contact + wall + integrate kernel),
# counting each array once per launch and treating neighbour gathers as cache-served:
#   FP64:  per node  reads disp, xpos, cur, vel, acc, extforce (8*dim B each), vol (8), grain id
#          and degree (4 + 4); writes acc, vel, force (8*dim each) -> 72*dim + 16 B
#          per bond  neighbour id (4 B) + xi_norm (8 B) + one alive bit          -> 12.125 B
#   mixed: per node  reads the FP32 hi/lo record of disp and xpos (16*dim), hi/lo cur (8*dim), FP64
#          vel (8*dim), FP32 acc and extforce (4*dim each), grain id (4); writes FP32 acc (4*dim),
#          FP64 vel (8*dim), FP32 force (4*dim)                                  -> 56*dim + 4 B
#          per bond  neighbour id (4 B) + one alive bit                          -> 4.125 B


def node_bytes(dim, precision="fp64"):
    return 72 * dim + 16 if precision == "fp64" else 56 * dim + 4


def bond_bytes(precision="fp64"):
    return 12.125 if precision == "fp64" else 4.125


def node_step_bytes(n_nodes, n_bonds, dim, precision="fp64"):
    """Algorithmic bytes of one step by the scope table's per-unit figure: per node
    B = B_node + 12.125 deg + 16 (node stream, bond stream of index + xi_norm + alive bit, contact
    search), B_node = (8 dim + 1) 8 for FP64 and 52 dim + 4 for mixed; summed over the nodes
    (sum of deg = directed bonds)."""
    b_node = (8 * dim + 1) * 8 if precision == "fp64" else 52 * dim + 4
    return n_nodes * (b_node + 16) + n_bonds * 12.125


def fp64_flops_per_bond(dim):
    # (dj - di) + (xj - xi): 3*dim, |e|^2: 2*dim-1, sqrt 1, stretch 2, scale 2, unit*scale+acc: 3*dim
    return 3 * dim + (2 * dim - 1) + 1 + 2 + 2 + 3 * dim


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """Sample SM clocks and throttle reasons while the timed region runs."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0:
                    self.samples.append([x.strip() for x in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[2 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def profiled_traffic(key):
    """dram__bytes_read.sum + dram__bytes_write.sum of one k_force launch, from the ncu summaries
    committed under profiles/ (lines `bench-key: <workload>/<precision>` and
    `traffic_bytes_per_launch: <bytes>`)."""
    import glob
    import re

    for fn in sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md"))):
        txt = open(fn).read()
        if re.search(r"^bench-key:\s*%s\s*$" % re.escape(key), txt, re.M):
            m = re.search(r"^traffic_bytes_per_launch:\s*(\d+)", txt, re.M)
            if m:
                return int(m.group(1))
    return None


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    return int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")), ws


def reduce_over_ranks(dist, ms, n_nodes, device):
    """The job's timed milliseconds (max over ranks) and nodes (sum over ranks: every rank runs its
    own ensemble, so node counts differ); one process per GPU under torchrun."""
    if not dist:
        return ms, n_nodes
    import torch

    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    n = torch.tensor([float(n_nodes)], dtype=torch.float64, device=device)
    dist.all_reduce(n, op=dist.ReduceOp.SUM)
    return float(t.item()), int(round(n.item()))


def build_workload(k, rank):
    from perigrain_gb300 import setups

    spec = setups.WORKLOADS[k]
    kw = {}
    if k == 3:
        kw["seed"] = 3 + 1000 * rank  # weak scaling: every rank runs its own ensemble
    return setups.workload(k, **kw), spec


def engine_kwargs(spec, precision):
    return dict(dt=spec["dt"], enable_fracture=1, precision=precision)


def instance_subset(setup, first, count):
    """Single setup made of instances [first, first + count) of a batched setup."""
    D = setup.dim
    g0 = int(np.searchsorted(setup.grain_instance, first))
    g1 = int(np.searchsorted(setup.grain_instance, first + count))
    n0, n1 = int(setup.grain_node_offset[g0]), int(setup.grain_node_offset[g1])
    b0, b1 = int(setup.bond_offset[n0]), int(setup.bond_offset[n1])
    sub = setup.copy()
    sub.grain_instance = setup.grain_instance[g0:g1] - np.uint32(first)
    sub.grain_node_offset = setup.grain_node_offset[g0:g1 + 1] - np.uint32(n0)
    for f in ("pos", "disp", "vel", "acc", "extforce"):
        setattr(sub, f, getattr(setup, f)[n0 * D:n1 * D].copy())
    sub.vol = setup.vol[n0:n1].copy()
    sub.bond_offset = setup.bond_offset[n0:n1 + 1] - np.uint64(b0)
    sub.bond_local = setup.bond_local[b0:b1].copy()
    d0, d1 = int(setup.bdry_offset[g0]), int(setup.bdry_offset[g1])
    sub.bdry_offset = setup.bdry_offset[g0:g1 + 1] - np.uint32(d0)
    sub.bdry_nodes = setup.bdry_nodes[d0:d1].copy()
    c0, c1 = int(setup.clamped_offset[g0]), int(setup.clamped_offset[g1])
    sub.clamped_offset = setup.clamped_offset[g0:g1 + 1] - np.uint32(c0)
    sub.clamped_nodes = setup.clamped_nodes[c0:c1].copy()
    for f in ("delta", "rho", "cnot", "snot", "movable", "breakable", "stoppable", "break_bonds", "torque_axis",
              "torque_val"):
        setattr(sub, f, getattr(setup, f)[g0:g1].copy())
    for f in ("contact_radius", "normal_stiffness", "friction_coefficient", "damping_ratio", "allow_wall"):
        setattr(sub, f, getattr(setup, f)[first:first + count].copy())
    sub.wall_geom = setup.wall_geom[first * 2 * D:(first + count) * 2 * D].copy()
    sub.wall_speed = setup.wall_speed[first * 2 * D:(first + count) * 2 * D].copy()
    return sub


def cpu_model():
    """The host CPU's model name (lscpu on Arm, /proc/cpuinfo on x86), or the machine type."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform

    return platform.machine()


def _cpu_rate(sub, spec, steps, threads, budget_s):
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import _oracle as O

    sim = O.OracleSim(sub, dt=spec["dt"], enable_fracture=1)
    sim.set_mode(1, threads)
    t0 = time.perf_counter()
    done = 0
    while done < steps:
        sim.step(1)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return sub.n_nodes * done / dt, done, dt


def cpu_reference(setup, spec, steps, threads, budget_s=12.0, one_thread_s=4.0):
    """The reference's CPU algorithm, timed on a bounded sample of the workload: the oracle port
    in reference-structured mode (the reference's node-pair loops, bit-identical arithmetic),
    independent instances run concurrently on `threads` host threads (one instance per thread, the
    reference's OpenMP loop over grains gives no more parallelism than that for two-grain
    instances), for up to `steps` steps or until `budget_s` seconds of work have been done. The
    instances are independent, so the rate of the sample is the rate of the whole ensemble on these
    cores (work grows linearly with the number of instances). Beside it: one instance on one thread
    for up to `one_thread_s` seconds."""
    take = min(setup.n_instances, max(1, threads))
    sub = instance_subset(setup, 0, take)
    v, done, dt = _cpu_rate(sub, spec, steps, threads, budget_s)
    one = instance_subset(setup, 0, 1)
    v1, done1, dt1 = _cpu_rate(one, spec, steps, 1, one_thread_s)
    return v, dict(kind="port", cores=threads, steps=done, instances=take, nodes=sub.n_nodes, seconds=round(dt, 3),
                   cpu_model=cpu_model(), nproc=os.cpu_count(),
                   one_thread={"value": v1, "unit": METRIC, "instances": 1, "nodes": one.n_nodes, "steps": done1,
                               "seconds": round(dt1, 3)},
                   scaling="%d of %d independent instances, one per thread; the ensemble's CPU time grows "
                           "linearly with its instances, so this rate is the whole ensemble's rate on %d threads"
                           % (take, setup.n_instances, threads))


GRAD_HORIZONS = (200, 500, 1000, 2000, 5000)  # steps at which the gradient checks are repeated
GRAD_TOL = 1e-2  # a check holds at a horizon when its error is within this of the largest sensitivity


def _grad_checks(s, spec, n_steps, checkpoint_every=100, n_fd=4, times=False):
    """One differentiable run of n_steps steps of setup s: the mixed-precision gradient of
    J = top-wall reaction (y) / |value| + kinetic energy / value with respect to the per-grain
    parameters, the FP64 reference gradient (FP64 replay of the same masks, FP64 reverse step) and
    central differences of the frozen FP64 map for the n_fd largest sensitivities at h = 1e-4 and
    1e-6 (relative). Errors are relative to the largest reference sensitivity theta dJ/dtheta."""
    from perigrain_gb300 import Simulation, grad

    sim = Simulation(s, dt=spec["dt"], precision="mixed")
    run = grad.GradRun(sim, n_steps, checkpoint_every)
    r0, ke0 = run.forward()
    top = float(r0[0, 2, 1])
    wr = np.zeros_like(r0)
    wr[0, 2, 1] = 1.0 / abs(top) if top else 0.0
    wk = 1.0 / ke0
    out = {"steps": n_steps}
    if times:
        run.backward(reaction_bar=wr, ke_bar=wk)  # the first call captures the segment graphs
        run.forward()
    g = run.backward(reaction_bar=wr, ke_bar=wk)
    if times:
        out["times"] = run.times()
    th = run.params()
    tv = np.stack([th[k] for k in grad.PARAMS], 1)
    sens = g * tv
    m = run.record_masks()
    run.forward(m)
    g_ref = run.backward(reaction_bar=wr, ke_bar=wk) * tv
    scale = float(np.abs(g_ref).max())
    idx = np.argsort(-np.abs(g_ref).ravel())[:n_fd]
    fd_err = {}
    for h in (1e-4, 1e-6):
        e = 0.0
        for fi in idx:
            gi, a = divmod(int(fi), 4)
            vals = []
            for sg in (1, -1):
                p = {k: th[k].copy() for k in grad.PARAMS}
                p[grad.PARAMS[a]][gi] *= 1 + sg * h
                run.set_params(**p)
                r, ke = run.forward(m)
                vals.append(float((wr * r).sum() + (wk * ke).sum()))
            run.set_params(**{k: th[k] for k in grad.PARAMS})
            e = max(e, abs((vals[0] - vals[1]) / (2 * h) - g_ref[gi, a]))
        fd_err["h=%g" % h] = e / scale
    m.close()
    sim.close()
    out.update({"max_abs_sensitivity": float(np.abs(sens).max()),
                "mixed_vs_fp64_reference_grad_gap": float(np.abs(sens - g_ref).max() / scale),
                "fd_vs_fp64_adjoint_top%d" % n_fd: fd_err})
    return out


def adjoint_bench(n_steps=5000, checkpoint_every=100, n_fd=4, horizons=GRAD_HORIZONS):
    """Cost and checks of the gradient path on the differentiable compaction (50 grains, 5000
    steps, mixed-precision forward): backward (recompute from checkpoints + reverse steps) time
    over forward (with checkpointing) time at the configured 5000 steps, and at each horizon the
    gap between the mixed-precision gradient and the FP64 reference gradient and central
    differences of the frozen FP64 map for the largest sensitivities. The compaction is chaotic
    (FP64 runs perturbed at FP32 resolution separate), so the checks hold up to a horizon; the line
    names the longest horizon at which all of them are within GRAD_TOL."""
    from perigrain_gb300 import setups

    spec = setups.WORKLOADS[4]
    s = setups.workload(4)
    full = _grad_checks(s, spec, n_steps, checkpoint_every, n_fd, times=True)
    t = full.pop("times")
    checks = [_grad_checks(s, spec, h, checkpoint_every, n_fd) for h in horizons if h < n_steps] + [full]
    fdk = "fd_vs_fp64_adjoint_top%d" % n_fd
    for c in checks:
        c["hold"] = bool(c["mixed_vs_fp64_reference_grad_gap"] <= GRAD_TOL and c[fdk]["h=1e-06"] <= GRAD_TOL
                         and c[fdk]["h=0.0001"] <= GRAD_TOL)
    held = [c["steps"] for c in checks if c["hold"]]
    through = 0
    for c in checks:  # the horizon through which every check holds at every shorter horizon too
        if not c["hold"]:
            break
        through = c["steps"]
    return {"workload": spec["name"], "steps": n_steps, "checkpoint_every": checkpoint_every, "nodes": s.n_nodes,
            "params": 4 * s.n_grains, "objective": "top-wall reaction (y) / |value| + kinetic energy / value",
            "forward_ms": t["forward_ms"], "backward_ms": t["backward_ms"],
            "backward_over_forward": t["backward_ms"] / t["forward_ms"],
            "forward_launches": t["forward_launches"], "backward_launches": t["backward_launches"],
            "checks": checks, "checks_hold_through_step": through, "checks_hold_at": held, "tolerance": GRAD_TOL,
            "note": "each check is relative to the largest FP64 reference sensitivity; beyond the stated horizon the "
                    "compaction's chaotic dynamics separate the mixed and FP64 trajectories (and their gradients) and "
                    "push h=1e-4 differences out of the linear regime"}


def bonds_bench(n_target=200_000, repeats=5):
    """GPU bond-list builder (pg_build_bonds) on one jittered 2D disk grain of ~200k nodes with the
    horizon delta = 3h: grain nodes per second with positions resident on the device, end to end
    from a host array, and the reference's algorithm (all n(n-1)/2 pairs through
    itertools.combinations, exp_dict.py:199-222) in Python on a 1,200-node grain. The reference's
    cost grows with n^2, so its rate on the large grain would be far lower still."""
    import itertools
    import math

    import ctypes as C
    import torch

    from perigrain_gb300 import _native as N
    from perigrain_gb300 import bonds, setups

    h = 1e-5
    rng = np.random.default_rng(5)
    p, _ = setups.grid_nodes("disk", h * math.sqrt(n_target / math.pi), h, 2, 6, 0.1, rng, 0.0)
    p = np.ascontiguousarray(p, np.float64)
    delta = 3 * h
    n = len(p)
    d_pos = torch.from_numpy(p).cuda()
    cap = n * 32
    d_pairs = torch.empty((cap, 2), dtype=torch.int32, device="cuda")
    npairs = C.c_uint64()
    L = N.lib()

    def build():
        N.check(L.pg_build_bonds(C.c_void_p(d_pos.data_ptr()), n, 2, delta, C.c_void_p(d_pairs.data_ptr()), cap,
                                 C.byref(npairs), None))

    build()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(repeats):
        build()
    dev_s = (time.perf_counter() - t0) / repeats
    t0 = time.perf_counter()
    pairs = bonds.build_bonds(p, delta, capacity=cap)
    e2e_s = time.perf_counter() - t0
    # the reference's rule on a small grain, in Python
    ps, _ = setups.grid_nodes("disk", h * math.sqrt(1200 / math.pi), h, 2, 6, 0.1, np.random.default_rng(6), 0.0)
    ps = [tuple(map(float, q)) for q in ps]
    t0 = time.perf_counter()
    found = 0
    for a, b in itertools.combinations(range(len(ps)), 2):
        if math.sqrt((ps[b][0] - ps[a][0]) ** 2 + (ps[b][1] - ps[a][1]) ** 2) <= delta:
            found += 1
    cpu_s = time.perf_counter() - t0
    return {"workload": "one 2D disk grain, %d nodes, delta = 3h, %d bonds" % (n, len(pairs)),
            "metric": "grain nodes/s", "value": n / dev_s, "ms": dev_s * 1e3, "bonds": int(npairs.value),
            "e2e": {"value": n / e2e_s, "unit": "grain nodes/s", "note": "host positions -> device, build, pairs -> host"},
            "cpu_baseline": {"value": len(ps) / cpu_s, "unit": "grain nodes/s", "cores": 1, "kind": "port",
                             "sample": "the reference's all-pairs rule in Python on a %d-node grain (%d bonds), %.2f s"
                                       % (len(ps), found, cpu_s)}}


def postprocess_bench(sim, setup, repeats=20):
    """On-device post-processing (pg_postprocess) of the workload's state: snapshots per second,
    against the reference scripts' numpy formulas (read_sim_output.py) applied on the host to
    the same fields already in host memory (file reading excluded)."""
    sim.synchronize()
    sim.postprocess()
    t0 = time.perf_counter()
    for _ in range(repeats):
        sim.postprocess(node_damage=True)
    dev_s = (time.perf_counter() - t0) / repeats
    fields = {f: sim.field(f) for f in ("vel", "acc", "CurrPos", "force")}
    alive = sim.bond_alive()
    off = np.asarray(setup.grain_node_offset, np.int64)
    vol = np.asarray(setup.vol, np.float64)
    rho = np.asarray(setup.rho, np.float64)
    t0 = time.perf_counter()
    deg0 = np.diff(setup.bond_offset.astype(np.int64)).astype(np.float64)
    row = np.repeat(np.arange(setup.n_nodes), np.diff(setup.bond_offset.astype(np.int64)))
    deg = np.bincount(row, weights=alive.astype(np.float64), minlength=setup.n_nodes)
    dmg = (deg0 - deg) / deg0
    for g in range(setup.n_grains):
        sl = slice(off[g], off[g + 1])
        fields["vel"][sl].mean(axis=0)
        fields["acc"][sl].mean(axis=0)
        fields["CurrPos"][sl].mean(axis=0)
        fields["force"][sl].sum(axis=0)
        np.mean(dmg[sl])
        np.sum((vol[sl] * rho[g])[:, None] * fields["acc"][sl], axis=0)
    cpu_s = time.perf_counter() - t0
    return {"workload": "state of the bench workload, %d nodes, %d grains" % (setup.n_nodes, setup.n_grains),
            "metric": "snapshots/s", "value": 1.0 / dev_s, "ms": dev_s * 1e3,
            "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "snapshots/s", "cores": 1, "kind": "port",
                             "sample": "numpy formulas of read_sim_output.py on the same state in host memory, %.3f s"
                                       % cpu_s}}


class _QuietStdout:
    """Sends file descriptor 1 to /dev/null (the drop-in driver prints its progress table there)."""

    def __enter__(self):
        sys.stdout.flush()
        self.fd = os.dup(1)
        self.nul = os.open(os.devnull, os.O_WRONLY)
        os.dup2(self.nul, 1)

    def __exit__(self, *exc):
        import ctypes
        ctypes.CDLL(None).fflush(None)
        os.dup2(self.fd, 1)
        os.close(self.fd)
        os.close(self.nul)


def dropin_bench(steps=2000, modulo=100):
    """The drop-in process contract (pg_run_simulation: config/main.conf and data/hdf5/all.h5 in,
    output/hdf5/ out, as bin/simulate2d runs it) in-process on the 2D settling workload, mixed
    precision: node-steps/s with output off (save_file = 0) and with tc_/wall_ files every `modulo`
    steps. The fixed cost of a run (reading all.h5, creating the engine, plotinfo.h5, run_time.h5)
    is timed by 0-step runs and taken out."""
    import shutil
    import tempfile

    from perigrain_gb300 import run_simulation, setups

    spec = setups.WORKLOADS[1]
    s = spec["build"]()
    d = tempfile.mkdtemp(prefix="pg_dropin_")
    try:
        for sub in ("config", os.path.join("data", "hdf5"), os.path.join("output", "hdf5")):
            os.makedirs(os.path.join(d, sub), exist_ok=True)
        s.save_h5(os.path.join(d, "data", "hdf5", "all.h5"))

        def run(T, save):
            conf = {"timesteps": T, "modulo": modulo, "dt": spec["dt"], "save_file": save, "enable_fracture": 1,
                    "allow_damping": 1, "allow_friction": 1, "self_contact": 1, "is_parallel": 1}
            with open(os.path.join(d, "config", "main.conf"), "w") as f:
                for k, v in conf.items():
                    f.write("%s = %r\n" % (k, v))
            t0 = time.perf_counter()
            with _QuietStdout():
                run_simulation(d, 2, "mixed")
            return time.perf_counter() - t0

        run(0, 0)
        fixed = min(run(0, 0) for _ in range(2))
        off = run(steps, 0)
        on = run(steps, 1)
        out = os.path.join(d, "output", "hdf5")
        tc_bytes = os.path.getsize(os.path.join(out, "tc_00001.h5")) + os.path.getsize(os.path.join(out, "wall_00001.h5"))
        n_out = steps // modulo
        return {"workload": "%s: %d grains, %d nodes, %d bonds, through all.h5 and config/main.conf"
                            % (spec["name"], s.n_grains, s.n_nodes, s.n_bonds),
                "precision": "mixed", "steps": steps, "modulo": modulo, "fixed_ms": fixed * 1e3,
                "no_output": {"value": s.n_nodes * steps / (off - fixed), "unit": METRIC, "ms": (off - fixed) * 1e3},
                "with_output": {"value": s.n_nodes * steps / (on - fixed), "unit": METRIC, "ms": (on - fixed) * 1e3,
                                "outputs": n_out, "bytes_per_output": tc_bytes},
                "note": "files of one output are written while the GPU runs the next segment (pg_snapshot)"}
    except Exception as e:  # reported in the line, the headline stands
        return {"error": "%s: %s" % (type(e).__name__, e)}
    finally:
        shutil.rmtree(d, ignore_errors=True)


def packing_bench(nx=800, ny=500, repeats=3):
    """Incircle packing (pg_pack_incenters) of a jittered 800 x 500-cell triangulated rectangle with
    the reference's default options (maximin nodal circles, boundary nodes included): circles per
    second with the mesh resident in HBM, end to end from host arrays, and the oracle's scalar CPU
    port on a bounded sample (the reference solves each node's model with GEKKO, not installed)."""
    import torch

    from perigrain_gb300 import packing

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import packing_oracle as PO

    m = packing.rect_mesh(nx, ny, width=nx * 1e-4, height=ny * 1e-4, jitter=0.25, seed=21)
    d_pos = torch.from_numpy(m.pos).cuda()
    d_T, d_bn, d_be = packing._u32(m.T), packing._u32(m.bdry_nodes), packing._u32(m.bdry_edges)
    packing.pack_device(d_pos, d_T, d_bn, d_be)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(repeats):
        cen, rad, unp = packing.pack_device(d_pos, d_T, d_bn, d_be)
    dev_s = (time.perf_counter() - t0) / repeats
    n_circ = int(rad.shape[0])
    t0 = time.perf_counter()
    out = packing.get_incenter_mesh_loc(m)
    e2e_s = time.perf_counter() - t0
    sm = packing.rect_mesh(40, 25, width=40e-4, height=25e-4, jitter=0.25, seed=22)
    t0 = time.perf_counter()
    _, crad, _ = PO.incenter_mesh_loc(sm.pos, sm.T, sm.bdry_nodes, sm.bdry_edges, True, True)
    cpu_s = time.perf_counter() - t0
    return {"workload": "rect mesh %d x %d cells, %d nodes, %d triangles, maximin nodal circles with boundary nodes"
                        % (nx, ny, len(m.pos), len(m.T)),
            "metric": "circles/s", "value": n_circ / dev_s, "ms": dev_s * 1e3, "circles": n_circ,
            "unpolished": unp, "packing_ratio": float(out.packing_ratio()),
            "e2e": {"value": n_circ / e2e_s, "unit": "circles/s",
                    "note": "host mesh -> device, pg_pack_incenters, circles -> host"},
            "cpu_baseline": {"value": len(crad) / cpu_s, "unit": "circles/s", "cores": 1, "kind": "port",
                             "sample": "oracle scalar port on a 40 x 25-cell mesh (%d circles), %.2f s"
                                       % (len(crad), cpu_s)}}


ACC_HORIZONS = (10, 100, 1000, 10000)  # pointwise comparisons (and the configured run's last step)
ACC_WINDOWS = 10  # wall-reaction time series compared as means over this many windows of the run
ACC_EPS = 2.0 ** -24  # FP32 unit round-off: size of the FP64 ensemble's velocity perturbation
ACC_POS_TOL = 1e-6  # pointwise relative position error bound while the dynamics do not amplify
# whole-run statistics: a mixed-vs-FP64 difference passes when it is at most max(2 x the FP64
# ensemble's spread, floor); the floors are relative to the statistic's FP64 scale
ACC_STAT_FLOOR = {"kinetic_energy": 2e-2, "mean_grain_speed": 5e-2, "grain_centroid": 5e-2,
                  "reaction_window_means": 5e-2, "broken_bonds": 1e-1}


def _rel(a, b):
    """max |a - b| / max |b| over all entries (0 when both vanish)."""
    s = float(np.abs(b).max()) if np.size(b) else 0.0
    d = float(np.abs(a - b).max()) if np.size(b) else 0.0
    return d / s if s > 0 else (0.0 if d == 0 else float("inf"))


def perturbed_velocities(setup, seed, eps=ACC_EPS):
    """Copy of a setup whose initial velocity components are moved by eps * V with seeded random
    signs, V = max(max |v0|, 1 m/s): FP64 inputs known only to FP32 resolution."""
    p = setup.copy()
    rng = np.random.default_rng(1000 + seed)
    V = max(float(np.abs(setup.vel).max()), 1.0)
    p.vel = setup.vel + eps * V * rng.choice([-1.0, 1.0], size=setup.vel.shape)
    return p


def accuracy_config(k, members=2, sample_every=100, horizons=ACC_HORIZONS):
    """Mixed precision against FP64 over the whole configured run of workload k.

    Runs of the same setup advance together: the mixed path, the FP64 path (the reference's
    arithmetic, bit-exact to it in the tests) and an ensemble of `members` FP64 runs whose initial
    velocities differ from the setup's at FP32 resolution (perturbed_velocities). Contact dynamics
    are chaotic -- an FP64 run perturbed by 1e-15 already moves by several percent after a
    collision -- so every mixed-vs-FP64 figure is reported beside the ensemble's spread, the largest
    difference of an ensemble run from the FP64 run in the same measure.

      pointwise  at each horizon: max|dx| / max|x| (CurrPos), max|dv| / max|v| (vel) and
                 max|dR| / max|R| (wall reactions, every instance and side)
      full_run   kinetic energy sum(1/2 rho vol |v|^2) sampled every `sample_every` steps (max
                 difference / max KE), the wall-reaction time series (sampled like the reference's
                 wall_ files every `sample_every` steps) as means over ACC_WINDOWS windows, the mean
                 grain speed at the end, the grain centroids (mass-weighted) at the end as the mean
                 distance from FP64's over the mean distance the grains travelled, the number of
                 bonds broken (relative to FP64's), and the drift of total linear momentum
                 (configurations without walls, where the reference conserves it) relative to
                 sum(m |v0|).
    A whole-run measure passes when the mixed difference is at most max(2 x spread,
    ACC_STAT_FLOOR[measure]); pointwise, the horizon through which the position error stays within
    ACC_POS_TOL is reported.
    """
    from perigrain_gb300 import Simulation, setups

    spec = setups.WORKLOADS[k]
    setup = setups.workload(k)
    steps = spec["steps"]
    t0 = time.perf_counter()
    sims = {"mixed": Simulation(setup, **engine_kwargs(spec, "mixed")),
            "fp64": Simulation(setup, **engine_kwargs(spec, "fp64"))}
    ens = ["ens%d" % i for i in range(members)]
    for i, name in enumerate(ens):
        sims[name] = Simulation(perturbed_velocities(setup, i), **engine_kwargs(spec, "fp64"))
    D = setup.dim
    gsize = np.diff(setup.grain_node_offset.astype(np.int64))
    m = (setup.vol * np.repeat(setup.rho, gsize))[:, None]
    starts = setup.grain_node_offset[:-1].astype(np.int64)
    gmass = np.add.reduceat(m[:, 0], starts)
    v0 = setup.vel.reshape(-1, D)
    p0 = (m * v0).sum(0)
    pscale = max(float((m * np.abs(v0)).sum()), 1e-300)
    walls = bool(np.any(setup.allow_wall))
    hz = sorted(set([h for h in horizons if h < steps] + [steps]))
    ke = {n: [] for n in sims}
    reac = {n: [] for n in sims}
    mom = {n: 0.0 for n in sims}
    point = []
    done = 0
    while done < steps:
        nxt = min([h for h in hz if h > done] + [done + sample_every, steps])
        for sm in sims.values():
            sm.step(nxt - done)
        done = nxt
        vel = {}
        for name, sm in sims.items():
            v = sm.field("vel")
            ke[name].append(0.5 * float((m[:, 0] * (v * v).sum(1)).sum()))
            if walls:
                reac[name].append(sm.reaction())
            else:
                mom[name] = max(mom[name], float(np.abs((m * v).sum(0) - p0).max()) / pscale)
            vel[name] = v
        if done in hz:
            x = {name: sm.field("CurrPos") for name, sm in sims.items()}
            row = {"step": done}
            for key, group in (("mixed", ["mixed"]), ("spread", ens)):
                row[key] = {"pos": max(_rel(x[g], x["fp64"]) for g in group),
                            "vel": max(_rel(vel[g], vel["fp64"]) for g in group)}
                if walls:
                    row[key]["reaction"] = max(_rel(reac[g][-1], reac["fp64"][-1]) for g in group)
            row["pos_within_tol"] = bool(row["mixed"]["pos"] <= ACC_POS_TOL)
            point.append(row)
    fin = {}
    for name, sm in sims.items():
        x, v = sm.field("CurrPos"), sm.field("vel")
        alive = sm.bond_alive()
        gv = np.add.reduceat(m * v, starts, axis=0) / gmass[:, None]
        fin[name] = {"gspeed": float(np.sqrt((gv * gv).sum(1)).mean()),
                     "gpos": np.add.reduceat(m * x, starts, axis=0) / gmass[:, None],
                     "broken": int(setup.n_bonds - int(alive.sum()))}
        sm.close()
    x0 = setup.pos.reshape(-1, D) + setup.disp.reshape(-1, D)
    gpos0 = np.add.reduceat(m * x0, starts, axis=0) / gmass[:, None]
    travel = max(float(np.sqrt(((fin["fp64"]["gpos"] - gpos0) ** 2).sum(1)).mean()), 1e-300)
    kef = {n: np.array(v) for n, v in ke.items()}
    kscale = float(kef["fp64"].max())
    w = None
    if walls:
        nwin = min(ACC_WINDOWS, len(reac["fp64"]))
        w = np.array_split(np.arange(len(reac["fp64"])), nwin)
    bscale = max(fin["fp64"]["broken"], 1)
    sscale = max(fin["fp64"]["gspeed"], 1e-300)

    def measure(g):
        e = {"kinetic_energy": float(np.abs(kef[g] - kef["fp64"]).max() / kscale) if kscale > 0 else 0.0,
             "mean_grain_speed": abs(fin[g]["gspeed"] - fin["fp64"]["gspeed"]) / sscale,
             "grain_centroid": float(np.sqrt(((fin[g]["gpos"] - fin["fp64"]["gpos"]) ** 2).sum(1)).mean()) / travel,
             "broken_bonds": abs(fin[g]["broken"] - fin["fp64"]["broken"]) / bscale}
        if walls:
            a, b = np.array(reac[g]), np.array(reac["fp64"])
            e["reaction_window_means"] = _rel(np.stack([a[i].mean(0) for i in w]), np.stack([b[i].mean(0) for i in w]))
        return e

    mixed = measure("mixed")
    spread = {key: max(measure(g)[key] for g in ens) for key in mixed} if ens else {key: 0.0 for key in mixed}
    full = {key: {"mixed": mixed[key], "spread": spread[key], "floor": ACC_STAT_FLOOR[key],
                  "pass": bool(mixed[key] <= max(2.0 * spread[key], ACC_STAT_FLOOR[key]))} for key in mixed}
    full["broken_bond_counts"] = {n: fin[n]["broken"] for n in ("mixed", "fp64")}
    full["mean_grain_speed_values"] = {n: fin[n]["gspeed"] for n in ("mixed", "fp64")}
    if not walls:
        full["momentum_drift"] = {"mixed": mom["mixed"], "fp64": mom["fp64"], "pass": bool(mom["mixed"] <= 1e-6)}
    tol_h = [r["step"] for r in point if r["pos_within_tol"]]
    return {"workload": spec["name"], "dim": D, "nodes": setup.n_nodes, "bonds": setup.n_bonds, "steps": steps,
            "dt": spec["dt"], "ensemble": members, "pos_err_le_1e-6_through_step": max(tol_h) if tol_h else 0,
            "pointwise": point, "full_run": full,
            "all_full_run_pass": all(v["pass"] for v in full.values() if isinstance(v, dict) and "pass" in v),
            "seconds": time.perf_counter() - t0}


def accuracy_report(configs=(0, 1, 2, 3, 4), members=2):
    """members: FP64 ensemble runs per workload, an int or a dict workload -> int."""
    mem = members if isinstance(members, dict) else {k: members for k in configs}
    return {"runs": [accuracy_config(k, members=mem[k]) for k in configs],
            "measures": "'mixed': mixed vs FP64; 'spread': the largest difference from FP64 of the workload's "
                        "'ensemble' FP64 runs whose initial velocities are perturbed by 2^-24 max(|v0|, 1 m/s) "
                        "with random signs",
            "tolerance": ACCURACY_TOLERANCE}


ACCURACY_TOLERANCE = (
    "pointwise: relative position error <= 1e-6 up to the step given per workload (the dynamics then amplify "
    "any difference; later horizons are reported beside the FP64 ensemble spread); whole run: each statistic "
    "differs from FP64 by at most max(2 x ensemble spread, floor) -- kinetic-energy series 2e-2; mean grain "
    "speed, grain centroids (relative to the grains' travel) and windowed wall-reaction means 5e-2; broken-bond "
    "count 1e-1 (relative); momentum "
    "drift <= 1e-6 of sum(m|v0|) without walls")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=0,
                    help="timed steps (default: the workload's whole configured run, 10,000 steps for the "
                         "collision ensemble)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--workload", type=int, default=3)
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=400)
    ap.add_argument("--no-adjoint", action="store_true", help="skip the gradient-path measurement")
    ap.add_argument("--no-packing", action="store_true",
                    help="skip the setup-side measurements (packing generator, bond builder, post-processing)")
    ap.add_argument("--profile-adjoint", type=int, default=0, metavar="STEPS",
                    help="only a forward + backward of STEPS steps of the differentiable compaction "
                         "(checkpoint every 100; the command profiled under ncu)")
    ap.add_argument("--profile-packing", type=int, default=0, metavar="NX",
                    help="only incircle packings of an NX x 0.625 NX-cell mesh (the command profiled under ncu)")
    ap.add_argument("--accuracy", default="full", choices=["full", "off"],
                    help="mixed-vs-FP64 error over the whole configured run of every workload (default full)")
    ap.add_argument("--adjoint-only", action="store_true",
                    help="only the gradient-path measurement and its checks at every horizon; one JSON line")
    ap.add_argument("--accuracy-members", type=int, default=2,
                    help="FP64 runs perturbed at FP32 resolution per workload in the accuracy report")
    ap.add_argument("--accuracy-only", default="", metavar="K,K,...",
                    help="only the accuracy report of these workloads (e.g. 0,1,2,3,4); prints one JSON line")
    ap.add_argument("--profile-run", action="store_true",
                    help="only warmup + steps of the engine (the command profiled under ncu)")
    ap.add_argument("--profile-extras", action="store_true",
                    help="with --profile-run: then one asynchronous tc_ snapshot, one on-device post-processing "
                         "call and one bond-list build of a 20k-node grain (their kernels profiled under ncu)")
    a = ap.parse_args()
    a.warmup = max(3, a.warmup)
    import perigrain_gb300.setups as _setups

    if a.steps <= 0:
        a.steps = _setups.WORKLOADS[a.workload]["steps"]
    rank, local_rank, world = dist_env()
    threads = os.cpu_count() or 1

    if a.impl == "reference":
        if rank != 0:
            return
        setup, spec = build_workload(a.workload, 0)
        v, info = cpu_reference(setup, spec, a.cpu_steps + a.warmup, threads)
        line = {"metric": METRIC, "value": v, "unit": METRIC, "impl": "reference", "n_gpus": a.gpus,
                "steps": info["steps"], "warmup": 0, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": spec["name"], "instances_sampled": info["instances"],
                           "nodes_sampled": info["nodes"]},
                "cpu_baseline": dict(value=v, unit=METRIC, kind=info["kind"], cores=info["cores"],
                                     sample="%d instances x %d steps of %s, reference-structured oracle port"
                                            % (info["instances"], info["steps"], spec["name"]),
                                     cpu_model=info["cpu_model"], nproc=info["nproc"], one_thread=info["one_thread"],
                                     scaling=info["scaling"]),
                "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import perigrain_gb300 as pg
    from perigrain_gb300 import Simulation

    if a.adjoint_only:
        pg.engine.select_device(local_rank)
        print(json.dumps(adjoint_bench()), flush=True)
        return

    if a.accuracy_only:
        pg.engine.select_device(local_rank)
        print(json.dumps(accuracy_report([int(x) for x in a.accuracy_only.split(",")], members=a.accuracy_members)),
              flush=True)
        return

    if a.profile_packing:
        import torch

        from perigrain_gb300 import packing

        nx = a.profile_packing
        m = packing.rect_mesh(nx, nx * 5 // 8, width=nx * 1e-4, height=nx * 5 // 8 * 1e-4, jitter=0.25, seed=21)
        d_pos = torch.from_numpy(m.pos).cuda()
        d_T, d_bn, d_be = packing._u32(m.T), packing._u32(m.bdry_nodes), packing._u32(m.bdry_edges)
        for _ in range(a.warmup + a.steps):
            cen, rad, unp = packing.pack_device(d_pos, d_T, d_bn, d_be)
        print("profile packing: %d nodes, %d triangles, %d circles, unpolished %d, %d calls"
              % (len(m.pos), len(m.T), rad.shape[0], unp, a.warmup + a.steps))
        return

    if a.profile_adjoint:
        from perigrain_gb300 import grad, setups

        s = setups.workload(4)
        sim = Simulation(s, dt=setups.WORKLOADS[4]["dt"], precision=a.precision)
        run = grad.GradRun(sim, a.profile_adjoint, checkpoint_every=100)
        r, ke = run.forward()
        g = run.backward(ke_bar=1.0 / ke)
        print("profile adjoint: compaction_2d, %d nodes, %d steps, %s, finite %s"
              % (s.n_nodes, a.profile_adjoint, run.times(), bool(np.isfinite(g).all())))
        return

    pg.engine.select_device(local_rank)
    dist = None
    if world > 1:
        import torch
        import torch.distributed as tdist

        torch.cuda.set_device(local_rank)
        tdist.init_process_group("nccl")
        dist = tdist

    setup, spec = build_workload(a.workload, rank)
    kw = engine_kwargs(spec, a.precision)
    sim = Simulation(setup, autotune=not a.profile_run, **kw)
    tuned = dict(sim.launch_config(), contact_skin=sim.contact_skin(), node_order=sim.node_order()[0])
    sim.step(a.warmup)
    sim.synchronize()
    if a.profile_run:
        sim.step(a.steps)
        sim.synchronize()
        if a.profile_extras:
            import math

            from perigrain_gb300 import bonds, setups as _s

            got = sim.snapshot(("CurrPos", "vel", "acc", "force")).wait()
            post = sim.postprocess(node_damage=True)
            h = 1e-5
            p, _ = _s.grid_nodes("disk", h * math.sqrt(20000 / math.pi), h, 2, 6, 0.1, np.random.default_rng(5), 0.0)
            pairs = bonds.build_bonds(np.ascontiguousarray(p, np.float64), 3 * h)
            print("profile extras: snapshot %d nodes, post-processing of %d grains, %d bonds of a %d-node grain"
                  % (len(got["CurrPos"]), len(post["grain_damage"]), len(pairs), len(p)))
        print("profile run: %s, %d nodes, %d steps" % (spec["name"], setup.n_nodes, a.warmup + a.steps))
        return

    def barrier():
        if dist:
            import torch

            dist.barrier()
            torch.cuda.synchronize()

    barrier()
    # the first COMPARE_STEPS steps are timed on their own as well (the FP64 comparison reports them)
    k_cmp = min(a.steps, COMPARE_STEPS)
    launches = 0
    with Clocks(local_rank) as clk:
        ms_cmp = sim.step_timed(k_cmp)
        launches += sim.launch_count()
        ms = ms_cmp
        if a.steps > k_cmp:
            ms += sim.step_timed(a.steps - k_cmp)
            launches += sim.launch_count()
    barrier()
    ms_max, job_nodes = reduce_over_ranks(dist, ms, setup.n_nodes, "cuda")
    node_steps = job_nodes * a.steps
    value = node_steps / (ms_max / 1e3)

    # dominant kernel time: CUDA events around every k_force launch, over the steps that follow
    sim.set_timing(True)
    sim.step(min(a.steps, 2000))
    force_ms, total_ms, nforce = sim.kernel_times()
    sim.set_timing(False)
    st, _ = sim.device_status()
    if st:
        raise RuntimeError("device status %d after the timed region" % st)
    post_line = None if (a.no_packing or rank != 0) else postprocess_bench(sim, setup)
    sim.close()

    plain = seq = accuracy = None
    if a.precision == "mixed" and rank == 0:
        # the plain FP64 path on the same batch over the same whole run as `value` (FP64 = the
        # reference's arithmetic), its first COMPARE_STEPS steps also on their own: early in the
        # run most bonds are unstretched and the FP64 force kernel skips their force update
        s64 = Simulation(setup, autotune=True, **engine_kwargs(spec, "fp64"))
        tuned64 = dict(s64.launch_config(), contact_skin=s64.contact_skin(), node_order=s64.node_order()[0])
        s64.step(a.warmup)
        ms64_cmp = s64.step_timed(k_cmp)
        ms64 = ms64_cmp
        if a.steps > k_cmp:
            ms64 += s64.step_timed(a.steps - k_cmp)
        s64.set_timing(True)
        s64.step(min(k_cmp, 200))
        f64_ms, t64_ms, n64 = s64.kernel_times()
        s64.close()
        f64_launch_s = f64_ms / max(1, n64) / 1e3
        peak64, peak64_kind = load_peaks()
        hbm64 = node_step_bytes(setup.n_nodes, setup.n_bonds, setup.dim, "fp64") / f64_launch_s / 1e9
        tf64 = setup.n_bonds * fp64_flops_per_bond(setup.dim) / f64_launch_s / 1e12
        plain = {"value": setup.n_nodes * a.steps / (ms64 / 1e3), "unit": METRIC, "ms_per_step": ms64 / a.steps,
                 "steps": a.steps, "mixed_same_steps": setup.n_nodes * a.steps / (ms / 1e3),
                 "first_steps": {"steps": k_cmp, "value": setup.n_nodes * k_cmp / (ms64_cmp / 1e3),
                                 "ms_per_step": ms64_cmp / k_cmp,
                                 "mixed_value": setup.n_nodes * k_cmp / (ms_cmp / 1e3)},
                 "k_force_ms": f64_ms / max(1, n64), "autotuned": tuned64,
                 "roofline": {"kernel": "k_force", "bound": "fp64 pipe",
                              "hbm_achieved": hbm64, "hbm_peak": peak64, "hbm_frac": hbm64 / peak64,
                              "hbm_peak_source": peak64_kind,
                              "bytes_model": "per node-step B = (8 dim + 1) 8 + 12.125 deg + 16",
                              "fp64_tflops": tf64, "fp64_nominal_tflops": 1.25, "fp64_frac_of_nominal": tf64 / 1.25},
                 "fp64_tflops": tf64}
        # 256 sequential single-instance FP64 runs, timed on a sample of instances
        ns = min(8, setup.n_instances)
        k_seq = min(a.steps, 200)
        t_seq, nodes_seq = 0.0, 0
        for i in range(ns):
            one = instance_subset(setup, i, 1)
            si = Simulation(one, **engine_kwargs(spec, "fp64"))
            si.step(a.warmup)
            t_seq += si.step_timed(k_seq)
            nodes_seq += one.n_nodes
            si.close()
        seq = {"value": nodes_seq * k_seq / (t_seq / 1e3), "unit": METRIC,
               "sample": "%d instances run one after another, %d steps each" % (ns, k_seq),
               "est_ms_for_all_instances_per_step": t_seq / k_seq * setup.n_instances / ns}

    # end to end through the C ABI from host buffers
    # a run of at least 1000 steps (config 3 runs 10,000), so that creation is amortised as in use
    e2e_steps = max(a.steps, 1000)
    barrier()
    t0 = time.perf_counter()
    e2e_sim = Simulation(setup, **kw, **tuned)  # the launch configuration the autotuner picked
    t_created = time.perf_counter()
    # a tc_ snapshot (CurrPos, vel, acc, force) every 100 steps, as the drop-in writes them: each is
    # gathered on the device behind its steps and copied to page-locked host buffers while the next
    # 100 steps run (pg_snapshot / pg_wait)
    snap_items = ("CurrPos", "vel", "acc", "force")
    bufs = e2e_sim.snapshot_buffers(snap_items)
    t_bufs = time.perf_counter()
    snaps = 0
    done = 0
    d2h = 0
    t_wait = 0.0
    pending = None
    while done < e2e_steps:
        n = min(100, e2e_steps - done)
        e2e_sim.step(n)
        done += n
        if pending is not None:
            td = time.perf_counter()
            got = pending.wait()
            t_wait += time.perf_counter() - td
            d2h += sum(got[f].nbytes for f in snap_items)
        pending = e2e_sim.snapshot(snap_items, out=bufs)
        snaps += 1
    td = time.perf_counter()
    got = pending.wait()
    t_wait += time.perf_counter() - td
    d2h += sum(got[f].nbytes for f in snap_items)
    e2e_s = time.perf_counter() - t0
    e2e_parts = {"create_ms": (t_created - t0) * 1e3, "buffers_ms": (t_bufs - t_created) * 1e3,
                 "host_wait_ms": t_wait * 1e3}
    e2e_sim.close()
    h2d = sum(getattr(setup, f).nbytes for f in ("pos", "vol", "disp", "vel", "acc", "extforce", "bond_offset",
                                                   "bond_local"))
    e2e_ms, e2e_nodes = reduce_over_ranks(dist, e2e_s * 1e3, setup.n_nodes, "cuda")

    if rank != 0:
        return
    D = setup.dim
    peak, peak_kind = load_peaks()
    force_launch_ms = force_ms / max(1, nforce)
    # achieved: the scope table's per-unit bytes x the nodes one launch of the dominant kernel
    # processes / its average launch time; beside it the kernel's own stream (what it must read and
    # write with xi recomputed from the reference positions), which the DRAM traffic is compared to
    step_bytes = node_step_bytes(setup.n_nodes, setup.n_bonds, D, a.precision)
    achieved = step_bytes / (force_launch_ms / 1e3) / 1e9
    alg_bytes = setup.n_nodes * node_bytes(D, a.precision) + setup.n_bonds * bond_bytes(a.precision)
    achieved_kernel = alg_bytes / (force_launch_ms / 1e3) / 1e9
    fp64_tflops = setup.n_bonds * fp64_flops_per_bond(D) / (force_launch_ms / 1e3) / 1e12
    traffic = profiled_traffic("%s/%s" % (spec["name"], a.precision))
    cpu_v, cpu_info = cpu_reference(setup, spec, a.cpu_steps, threads)
    if a.precision == "mixed" and a.accuracy == "full":
        # mixed vs FP64 over the whole configured run of every workload: two perturbed FP64 runs
        # for the chaotic collisions and compaction, one for the long settling runs (their FP64 runs
        # dominate the bench's time); --accuracy-only with --accuracy-members sets any size
        accuracy = accuracy_report(members={0: 2, 1: 1, 2: 1, 3: 2, 4: 2})
    adjoint = None if a.no_adjoint else adjoint_bench()
    packing_line = None if a.no_packing else packing_bench()
    bonds_line = None if a.no_packing else bonds_bench()
    dropin_line = None if a.no_packing else dropin_bench()
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms_max / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if a.precision == "fp64" else "f32-forces/f64-state", "data": "synthetic (seeded generator)",
        "config": {"workload": spec["name"], "precision": a.precision, "instances": setup.n_instances,
                   "nodes": setup.n_nodes, "bonds": setup.n_bonds, "dim": D, "dt": spec["dt"],
                   "nodes_all_ranks": job_nodes,
                   "parallelism": "instances per GPU" if world == 1 else "dp%d (independent ensembles)" % world,
                   "timed_steps": "steps %d..%d of the run (the workload's configured run is %d steps)"
                                  % (a.warmup + 1, a.warmup + a.steps, spec["steps"]),
                   "l2": "inputs larger than L2 (%.0f MB of node and bond arrays resident)"
                         % ((alg_bytes + setup.n_bonds * 4) / 1e6)},
        "roofline": {"bound": "hbm", "kernel": "k_force" if a.precision == "fp64" else "k_force_mx",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                     "algorithmic_bytes_per_launch": step_bytes,
                     "bytes_model": "per node-step B = B_node + 12.125 deg + 16, B_node = %s"
                                    % ("(8 dim + 1) 8" if a.precision == "fp64" else "52 dim + 4"),
                     "kernel_stream": {"bytes_per_launch": alg_bytes, "achieved": achieved_kernel,
                                       "frac": achieved_kernel / peak,
                                       "model": "per node %s B, per directed bond %s B (xi from the reference "
                                                "positions, no xi_norm stream)"
                                                % ("72 dim + 16" if a.precision == "fp64" else "56 dim + 4",
                                                   bond_bytes(a.precision))},
                     "launch_ms": force_launch_ms,
                     "share_of_step": force_ms / total_ms if total_ms else None,
                     **({"fp64_tflops": fp64_tflops, "fp64_nominal_tflops": 1.25} if a.precision == "fp64" else {})},
        "cpu_baseline": {"value": cpu_v, "unit": METRIC, "cores": cpu_info["cores"], "kind": cpu_info["kind"],
                         "sample": "%d instances x %d steps of %s (%d nodes), reference-structured oracle port, "
                                   "%.1f s" % (cpu_info["instances"], cpu_info["steps"], spec["name"],
                                               cpu_info["nodes"], cpu_info["seconds"]),
                         "cpu_model": cpu_info["cpu_model"], "nproc": cpu_info["nproc"],
                         "one_thread": cpu_info["one_thread"], "scaling": cpu_info["scaling"]},
        "e2e": {"value": e2e_nodes * e2e_steps / (e2e_ms / 1e3), "unit": METRIC, "steps": e2e_steps,
                "h2d_bytes_per_step": h2d / e2e_steps, "d2h_bytes_per_step": d2h / e2e_steps,
                "note": "pg_create from host arrays + %d steps + %d tc_ snapshots (one every 100 steps, copied to "
                        "page-locked host buffers while the next steps run)"
                        % (e2e_steps, snaps),
                **e2e_parts},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "autotuned": tuned,
        "plain_fp64": plain,
        "sequential_fp64": seq,
        "accuracy": accuracy,
        "adjoint": adjoint,
        "packing": packing_line,
        "bond_builder": bonds_line,
        "postprocess": post_line,
        "dropin": dropin_line,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
