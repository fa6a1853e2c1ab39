"""Test helpers around the oracle (oracle/): the C++ restatement (liboracle.so) and the
reference itself compiled against API shims (oracle/_ref/simulate{2,3}d)."""
import ctypes as C
import os
import subprocess

import numpy as np

from perigrain_gb300 import _native as N
from perigrain_gb300 import h5

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE = os.path.join(ROOT, "oracle")
LIBORACLE = os.path.join(ORACLE, "liboracle.so")
REF_BIN = {2: os.path.join(ORACLE, "_ref", "simulate2d"), 3: os.path.join(ORACLE, "_ref", "simulate3d"),
           "worm": os.path.join(ORACLE, "_ref", "simulate2d_worm")}

_lib = None


def build_oracle():
    subprocess.run(["make", "-s", "-C", ORACLE], check=True, capture_output=True)


def oracle_lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIBORACLE):
            build_oracle()
        L = C.CDLL(LIBORACLE)
        L.orc_create.argtypes = [C.POINTER(N.SetupDesc), C.POINTER(N.Config), C.POINTER(C.c_void_p)]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_step.argtypes = [C.c_void_p, C.c_uint32]
        L.orc_get_field.argtypes = [C.c_void_p, C.c_int, N.f64p]
        L.orc_set_field.argtypes = [C.c_void_p, C.c_int, N.f64p]
        L.orc_get_bond_alive.argtypes = [C.c_void_p, N.u8p]
        L.orc_get_bond_break_step.argtypes = [C.c_void_p, N.u32p]
        L.orc_get_reaction.argtypes = [C.c_void_p, N.f64p]
        L.orc_get_wall.argtypes = [C.c_void_p, N.f64p]
        L.orc_set_grain_flags.argtypes = [C.c_void_p, C.c_uint32, C.c_int32, C.c_int32]
        L.orc_pair_log_size.argtypes = [C.c_void_p]
        L.orc_pair_log_size.restype = C.c_uint64
        L.orc_get_pair_log.argtypes = [C.c_void_p, N.u64p, N.u64p]
        L.orc_too_close.argtypes = [C.c_void_p]
        L.orc_too_close.restype = C.c_uint64
        L.orc_set_mode.argtypes = [C.c_void_p, C.c_int, C.c_int]
        _lib = L
    return _lib


class OracleSim:
    """Same interface as perigrain_gb300.Simulation, computed by the CPU oracle."""

    def __init__(self, setup, dt, enable_fracture=1, nl_bdry_only=0, allow_damping=1, allow_friction=1,
                 self_contact=1, enable_torque=0, gradient_extforce=0, extforce_maxstep=0, first_step=1, timeloop=0,
                 **_):
        L = oracle_lib()
        self.setup = setup
        self.dim = setup.dim
        cfg = N.Config()
        cfg.dt = dt
        cfg.enable_fracture = int(enable_fracture)
        cfg.nl_bdry_only = int(nl_bdry_only)
        cfg.allow_damping = int(allow_damping)
        cfg.allow_friction = int(allow_friction)
        cfg.self_contact = int(self_contact)
        cfg.enable_torque = int(enable_torque)
        cfg.gradient_extforce = int(gradient_extforce)
        cfg.extforce_maxstep = int(extforce_maxstep)
        cfg.first_step = int(first_step)
        cfg.timeloop = 1 if timeloop in (1, "worm") else 0
        self._desc = setup.desc()
        h = C.c_void_p()
        assert L.orc_create(C.byref(self._desc), C.byref(cfg), C.byref(h)) == 0
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            oracle_lib().orc_destroy(self.h)
            self.h = None

    def set_mode(self, reference_structured=0, threads=1):
        oracle_lib().orc_set_mode(self.h, int(reference_structured), int(threads))

    def step(self, n=1):
        oracle_lib().orc_step(self.h, int(n))

    def field(self, name):
        out = np.empty((self.setup.n_nodes, self.dim))
        assert oracle_lib().orc_get_field(self.h, N.FIELD[name], N.ptr(out, C.c_double)) == 0
        return out

    def set_field(self, name, a):
        a = np.ascontiguousarray(a, np.float64)
        assert oracle_lib().orc_set_field(self.h, N.FIELD[name], N.ptr(a, C.c_double)) == 0

    def bond_alive(self):
        out = np.empty(max(1, self.setup.n_bonds), np.uint8)
        oracle_lib().orc_get_bond_alive(self.h, N.ptr(out, C.c_uint8))
        return out[: self.setup.n_bonds]

    def break_step(self):
        out = np.empty(max(1, self.setup.n_bonds), np.uint32)
        oracle_lib().orc_get_bond_break_step(self.h, N.ptr(out, C.c_uint32))
        return out[: self.setup.n_bonds]

    def reaction(self):
        out = np.empty((self.setup.n_instances, 2 * self.dim, self.dim))
        oracle_lib().orc_get_reaction(self.h, N.ptr(out, C.c_double))
        return out

    def wall(self):
        out = np.empty((self.setup.n_instances, 2 * self.dim))
        oracle_lib().orc_get_wall(self.h, N.ptr(out, C.c_double))
        return out

    def set_grain_flags(self, grain, movable=-1, stoppable=-1):
        oracle_lib().orc_set_grain_flags(self.h, int(grain), int(movable), int(stoppable))

    def pair_log_all(self):
        L = oracle_lib()
        n = L.orc_pair_log_size(self.h)
        c = np.empty(max(1, n), np.uint64)
        hs = np.empty(max(1, n), np.uint64)
        L.orc_get_pair_log(self.h, N.ptr(c, C.c_uint64), N.ptr(hs, C.c_uint64))
        return c[:n], hs[:n]

    def too_close(self):
        return oracle_lib().orc_too_close(self.h)


def write_conf(path, conf):
    with open(path, "w") as f:
        for k, v in conf.items():
            f.write("%s = %r\n" % (k, v) if isinstance(v, float) else "%s = %s\n" % (k, v))


WALL_SPEED_KEYS = {2: ["speed_wall_left", "speed_wall_right", "speed_wall_top", "speed_wall_bottom"],
                   3: ["speed_wall_x_min", "speed_wall_y_min", "speed_wall_z_min", "speed_wall_x_max",
                       "speed_wall_y_max", "speed_wall_z_max"]}


def conf_for(setup, **conf):
    """main.conf keys for a single-instance setup: the reference reads wall speeds only from the
    config (contact.h:280-298), so they are written there."""
    c = dict(conf)
    for k, v in zip(WALL_SPEED_KEYS[setup.dim], setup.wall_speed[: 2 * setup.dim]):
        if v != 0.0:
            c.setdefault(k, float(v))
    return c


def make_case_dir(tmp, setup, conf):
    os.makedirs(os.path.join(tmp, "config"), exist_ok=True)
    os.makedirs(os.path.join(tmp, "data", "hdf5"), exist_ok=True)
    os.makedirs(os.path.join(tmp, "output", "hdf5"), exist_ok=True)
    setup.save_h5(os.path.join(tmp, "data", "hdf5", "all.h5"))
    write_conf(os.path.join(tmp, "config", "main.conf"), conf)
    return tmp


def run_reference(case_dir, dim, timeout=600, timeloop=None):
    """Run the reference simulator (compiled unmodified against the shims) in case_dir;
    timeloop="worm" runs the reference's run_timeloop_worm (2D)."""
    exe = REF_BIN["worm" if timeloop == "worm" else dim]
    if not os.path.exists(exe):
        build_oracle()
    if not os.path.exists(exe):
        raise FileNotFoundError("reference build unavailable: %s" % exe)
    r = subprocess.run([exe], cwd=case_dir, capture_output=True, text=True, timeout=timeout,
                       env=dict(os.environ, OMP_NUM_THREADS=os.environ.get("PERIGRAIN_REF_THREADS", "2")))
    if r.returncode != 0:
        raise RuntimeError("reference run failed (%d):\n%s\n%s" % (r.returncode, r.stdout[-3000:], r.stderr[-3000:]))
    return r.stdout


def read_tc(case_dir, counter, n_grains, dim, connectivity=True):
    fn = os.path.join(case_dir, "output", "hdf5", "tc_%05d.h5" % counter)
    out = {}
    for key in ("CurrPos", "vel", "acc", "force"):
        out[key] = np.concatenate([h5.read(fn, "P_%05d/%s" % (g, key), np.float64) for g in range(n_grains)])
    if connectivity:
        out["Connectivity"] = [h5.read(fn, "P_%05d/Connectivity" % g, np.uint32).reshape(-1, 2)
                               for g in range(n_grains)]
    fw = os.path.join(case_dir, "output", "hdf5", "wall_%05d.h5" % counter)
    out["wall_info"] = h5.read(fw, "wall_info", np.float64).ravel()
    out["reaction"] = h5.read(fw, "reaction", np.float64)
    return out


def conn_from_alive(setup, alive):
    """Connectivity rows (i < q per grain, row order) from an alive mask in CSR order."""
    from perigrain_gb300.setups import rows_to_conn

    res = []
    for g in range(setup.n_grains):
        n0, n1 = int(setup.grain_node_offset[g]), int(setup.grain_node_offset[g + 1])
        b0, b1 = int(setup.bond_offset[n0]), int(setup.bond_offset[n1])
        off = setup.bond_offset[n0:n1 + 1] - setup.bond_offset[n0]
        loc = setup.bond_local[b0:b1]
        a = alive[b0:b1].astype(bool)
        # drop dead entries, keep order
        keep_counts = np.add.reduceat(a.astype(np.int64), off[:-1].astype(np.int64)) if len(loc) else np.zeros(n1 - n0, np.int64)
        if len(loc):
            empty = np.diff(off.astype(np.int64)) == 0
            keep_counts[empty] = 0
        noff = np.zeros(n1 - n0 + 1, np.uint64)
        noff[1:] = np.cumsum(keep_counts)
        res.append(rows_to_conn(noff, loc[a]).astype(np.uint32))
    return res


def drive(sim, conf, n_grains, on_snapshot):
    """The run_timeloop step loop (timeloop.h:608-1006) around any engine with the Simulation
    interface: hooks at the start of step t, on_snapshot(counter) every `modulo` steps."""
    T, mod = int(conf["timesteps"]), int(conf["modulo"])
    hooks = {}
    if conf.get("set_movable_index", -1) != -1:
        hooks.setdefault(int(conf["set_movable_timestep"]), []).append(("movable", int(conf["set_movable_index"])))
    if conf.get("set_stoppable_index", -1) != -1:
        hooks.setdefault(int(conf["set_stoppable_timestep"]), []).append(("stoppable", int(conf["set_stoppable_index"])))
    counter = 1
    t = 1
    while t <= T:
        for kind, g in hooks.get(t, []):
            if kind == "movable":
                sim.set_grain_flags(g, movable=1)
            else:
                sim.set_grain_flags(g, stoppable=1)
        e = min(T, ((t + mod - 1) // mod) * mod)
        for ht in hooks:
            if t < ht <= e:
                e = ht - 1
        sim.step(e - t + 1)
        t = e + 1
        if conf.get("save_file", 1) and e % mod == 0:
            on_snapshot(counter)
            counter += 1


def engine_kwargs(conf):
    return dict(dt=float(conf["dt"]), enable_fracture=int(conf.get("enable_fracture", 0)),
                nl_bdry_only=int(conf.get("nl_bdry_only", 0)), allow_damping=int(conf.get("allow_damping", 1)),
                allow_friction=int(conf.get("allow_friction", 1)), self_contact=int(conf.get("self_contact", 1)),
                enable_torque=int(conf.get("enable_torque", 0)),
                gradient_extforce=int(conf.get("gradient_extforce", 0)),
                extforce_maxstep=int(conf.get("extforce_maxstep", 0)))


def load_golden(name):
    import json

    z = np.load(os.path.join(ROOT, "tests", "golden", name + ".npz"))
    meta = json.loads(bytes(z["meta"]).decode())
    return z, meta


def resumed_setup(s, tc, wall_info=None, reload_connectivity=True):
    """The state run_timeloop rebuilds on resume (timeloop.h:508-550): disp = CurrPos - pos, vel
    and acc from tc_%05u.h5, neighbour rows from its Connectivity (conn2NArr), wall from wall_."""
    from perigrain_gb300.setups import conn_to_rows

    r = s.copy()
    D = s.dim
    r.disp = (tc["CurrPos"] - s.pos.reshape(-1, D)).reshape(-1)
    r.vel = tc["vel"].reshape(-1).copy()
    r.acc = tc["acc"].reshape(-1).copy()
    if reload_connectivity:
        offs, locs, base = [np.zeros(1, np.uint64)], [], 0
        for g in range(s.n_grains):
            n = int(s.grain_node_offset[g + 1] - s.grain_node_offset[g])
            off, loc = conn_to_rows(tc["Connectivity"][g], n)
            offs.append(off[1:] + np.uint64(base))
            locs.append(loc)
            base += int(off[-1])
        r.bond_offset = np.concatenate(offs).astype(np.uint64)
        r.bond_local = np.concatenate(locs).astype(np.uint32)
    if wall_info is not None:
        r.wall_geom = np.asarray(wall_info, np.float64).ravel().copy()
    return r
