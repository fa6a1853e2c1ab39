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
REF_BIN = {2: os.path.join(ORACLE, "_ref", "simulate2d"), 3: os.path.join(ORACLE, "_ref", "simulate3d")}

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
        _lib = L
    return _lib


class OracleSim:
    """Same interface as perigrain_gb300.Simulation, computed by the CPU oracle."""

    def __init__(self, setup, dt, enable_fracture=1, nl_bdry_only=0, allow_damping=1, allow_friction=1,
                 self_contact=1, enable_torque=0, gradient_extforce=0, extforce_maxstep=0, first_step=1, **_):
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
        self._desc = setup.desc()
        h = C.c_void_p()
        assert L.orc_create(C.byref(self._desc), C.byref(cfg), C.byref(h)) == 0
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            oracle_lib().orc_destroy(self.h)
            self.h = None

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


def run_reference(case_dir, dim, timeout=600):
    """Run the reference simulator (compiled unmodified against the shims) in case_dir."""
    exe = REF_BIN[dim]
    if not os.path.exists(exe):
        build_oracle()
    if not os.path.exists(exe):
        raise FileNotFoundError("reference build unavailable: %s" % exe)
    r = subprocess.run([exe], cwd=case_dir, capture_output=True, text=True, timeout=timeout,
                       env=dict(os.environ, OMP_NUM_THREADS="1"))
    if r.returncode != 0:
        raise RuntimeError("reference run failed (%d):\n%s\n%s" % (r.returncode, r.stdout[-3000:], r.stderr[-3000:]))
    return r.stdout


def read_tc(case_dir, counter, n_grains, dim):
    fn = os.path.join(case_dir, "output", "hdf5", "tc_%05d.h5" % counter)
    out = {}
    for key in ("CurrPos", "vel", "acc", "force"):
        out[key] = np.concatenate([h5.read(fn, "P_%05d/%s" % (g, key), np.float64) for g in range(n_grains)])
    out["Connectivity"] = [h5.read(fn, "P_%05d/Connectivity" % g, np.uint32).reshape(-1, 2) for g in range(n_grains)]
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
