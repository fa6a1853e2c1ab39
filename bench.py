"""Benchmark: node-steps/s of the PeriDEM time step on one GB300 (or N, one process per GPU).

Default workload: the batched ensemble -- 256 independent two-grain collisions (disk / n-gon,
radius U(0.5, 1.5) mm, 200-1800 nodes per grain, impact speed U(5, 40) m/s, angle U(0, 60) deg),
all advanced together in one handle. A "step" is one time step of every instance.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload 0..4] [--precision fp64|mixed]
    python bench.py --impl reference ...   # the reference's CPU algorithm on the host cores

Prints one JSON line (rank 0). `value` is device-timed (CUDA events on the engine's stream, state
resident in HBM, inputs larger than L2); `e2e` goes through the C ABI from host buffers: setup
upload + the timed steps + a tc_-snapshot download (CurrPos, vel, acc, force) every 100 steps.
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
# dominant kernel: fused bond + contact + wall + integrate (k_force); per node it reads disp, xpos,
# cur, vel, acc, extforce (dim doubles each), vol, grain id, degree, and writes acc, vel, force;
# per directed bond it reads the neighbour id (4 B), xi_norm (8 B) and one alive bit.
BOND_BYTES = 12.125


def node_bytes(dim):
    return 9 * 8 * dim + 8 + 8


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


def build_workload(k, rank):
    from perigrain_gb300 import setups

    spec = setups.WORKLOADS[k]
    kw = {}
    if k == 3:
        kw["seed"] = 3 + 1000 * rank  # weak scaling: every rank runs its own ensemble
    return setups.workload(k, **kw), spec


def engine_kwargs(spec, precision):
    return dict(dt=spec["dt"], enable_fracture=1, precision=precision)


def cpu_reference(setup, spec, steps, threads, budget_s=20.0):
    """The reference's CPU algorithm, timed on a bounded sample of the workload: the oracle port
    in reference-structured mode (the reference's node-pair loops, bit-identical arithmetic),
    independent instances run concurrently on `threads` host threads."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import _oracle as O
    from perigrain_gb300 import setups

    take = min(setup.n_instances, max(1, threads))
    # sub-setup made of the first `take` instances
    g_end = int(np.searchsorted(setup.grain_instance, take))
    n_end = int(setup.grain_node_offset[g_end])
    sub = setup.copy()
    sub.grain_instance = setup.grain_instance[:g_end]
    sub.grain_node_offset = setup.grain_node_offset[: g_end + 1]
    D = setup.dim
    for f in ("pos", "disp", "vel", "acc", "extforce"):
        setattr(sub, f, getattr(setup, f)[: n_end * D])
    sub.vol = setup.vol[:n_end]
    sub.bond_offset = setup.bond_offset[: n_end + 1]
    sub.bond_local = setup.bond_local[: int(setup.bond_offset[n_end])]
    sub.bdry_offset = setup.bdry_offset[: g_end + 1]
    sub.bdry_nodes = setup.bdry_nodes[: int(setup.bdry_offset[g_end])]
    sub.clamped_offset = setup.clamped_offset[: g_end + 1]
    sub.clamped_nodes = setup.clamped_nodes[: int(setup.clamped_offset[g_end])]
    for f in ("delta", "rho", "cnot", "snot", "movable", "breakable", "stoppable", "break_bonds", "torque_axis",
              "torque_val"):
        setattr(sub, f, getattr(setup, f)[:g_end])
    for f in ("contact_radius", "normal_stiffness", "friction_coefficient", "damping_ratio", "allow_wall"):
        setattr(sub, f, getattr(setup, f)[:take])
    sub.wall_geom = setup.wall_geom[: take * 2 * D]
    sub.wall_speed = setup.wall_speed[: take * 2 * D]
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
    return sub.n_nodes * done / dt, dict(kind="port", cores=threads, steps=done, instances=take,
                                         nodes=sub.n_nodes, seconds=round(dt, 3))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--workload", type=int, default=3)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=5)
    ap.add_argument("--profile-run", action="store_true",
                    help="only warmup + steps of the engine (the command profiled under ncu)")
    a = ap.parse_args()
    a.warmup = max(3, a.warmup)
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
                                            % (info["instances"], info["steps"], spec["name"])),
                "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import perigrain_gb300 as pg
    from perigrain_gb300 import Simulation

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
    sim = Simulation(setup, **kw)
    sim.step(a.warmup)
    sim.synchronize()
    if a.profile_run:
        sim.step(a.steps)
        sim.synchronize()
        print("profile run: %s, %d nodes, %d steps" % (spec["name"], setup.n_nodes, a.warmup + a.steps))
        return

    def barrier():
        if dist:
            import torch

            dist.barrier()
            torch.cuda.synchronize()

    barrier()
    with Clocks(local_rank) as clk:
        ms = sim.step_timed(a.steps)
    launches = sim.launch_count()
    barrier()
    ms_max = ms
    if dist:
        import torch

        t = torch.tensor([ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_max = float(t.item())
    node_steps = setup.n_nodes * a.steps * world
    value = node_steps / (ms_max / 1e3)

    # dominant kernel time: CUDA events around every k_force launch over the same number of steps
    sim.set_timing(True)
    sim.step(a.steps)
    force_ms, total_ms, nforce = sim.kernel_times()
    sim.set_timing(False)
    st, _ = sim.device_status()
    if st:
        raise RuntimeError("device status %d after the timed region" % st)
    sim.close()

    # end to end through the C ABI from host buffers
    t0 = time.perf_counter()
    e2e_sim = Simulation(setup, **kw)
    snaps = 0
    done = 0
    d2h = 0
    while done < a.steps:
        n = min(100, a.steps - done)
        e2e_sim.step(n)
        done += n
        for f in ("CurrPos", "vel", "acc", "force"):
            d2h += e2e_sim.field(f).nbytes
        snaps += 1
    e2e_s = time.perf_counter() - t0
    e2e_sim.close()
    h2d = sum(getattr(setup, f).nbytes for f in ("pos", "vol", "disp", "vel", "acc", "extforce", "bond_offset",
                                                   "bond_local"))

    if rank != 0:
        return
    D = setup.dim
    peak, peak_kind = load_peaks()
    force_launch_ms = force_ms / max(1, nforce)
    alg_bytes = setup.n_nodes * node_bytes(D) + setup.n_bonds * BOND_BYTES
    achieved = alg_bytes / (force_launch_ms / 1e3) / 1e9
    fp64_tflops = setup.n_bonds * fp64_flops_per_bond(D) / (force_launch_ms / 1e3) / 1e12
    traffic = profiled_traffic("%s/%s" % (spec["name"], a.precision))
    cpu_v, cpu_info = cpu_reference(setup, spec, a.cpu_steps, threads)
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms_max / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if a.precision == "fp64" else "f32-forces/f64-state", "data": "synthetic",
        "config": {"workload": spec["name"], "precision": a.precision, "instances": setup.n_instances,
                   "nodes": setup.n_nodes, "bonds": setup.n_bonds, "dim": D, "dt": spec["dt"],
                   "parallelism": "instances per GPU" if world == 1 else "dp%d (independent ensembles)" % world,
                   "l2": "inputs larger than L2 (%.0f MB of node and bond arrays resident)"
                         % ((alg_bytes + setup.n_bonds * 4) / 1e6)},
        "roofline": {"bound": "hbm", "kernel": "k_force", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                     "algorithmic_bytes_per_launch": alg_bytes, "launch_ms": force_launch_ms,
                     "share_of_step": force_ms / total_ms if total_ms else None,
                     "fp64_tflops": fp64_tflops, "fp64_nominal_tflops": 1.25},
        "cpu_baseline": {"value": cpu_v, "unit": METRIC, "cores": cpu_info["cores"], "kind": cpu_info["kind"],
                         "sample": "%d instances x %d steps of %s (%d nodes), reference-structured oracle port, "
                                   "%.1f s" % (cpu_info["instances"], cpu_info["steps"], spec["name"],
                                               cpu_info["nodes"], cpu_info["seconds"])},
        "e2e": {"value": setup.n_nodes * a.steps / e2e_s, "unit": METRIC,
                "h2d_bytes_per_step": h2d / a.steps, "d2h_bytes_per_step": d2h / a.steps,
                "note": "pg_create from host arrays + %d steps + %d tc_ snapshot downloads" % (a.steps, snaps)},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
