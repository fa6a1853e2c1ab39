"""Python face of the GPU engine (C ABI in include/perigrain.h).

:class:`Simulation` mirrors the reference's in-process entry point
``run_timeloop<dim>(PArr, Timeloop, Contact, RectWall)`` (src/particle/timeloop.h:501-1015):
it owns the grains of one or more independent simulations on the GPU and advances them by
time steps; fields come back in the reference's node order. :func:`run_simulation` is the whole
``bin/simulate2d`` / ``bin/simulate3d`` process contract (config/main.conf + data/hdf5/all.h5 in,
output/hdf5/*.h5 out).
"""
import ctypes as C
import weakref

import numpy as np

from . import _native as N


class Simulation:
    def __init__(self, setup, dt, enable_fracture=1, nl_bdry_only=0, allow_damping=1, allow_friction=1,
                 self_contact=1, enable_torque=0, gradient_extforce=0, extforce_maxstep=0, precision="fp64",
                 record_pairs=False, pair_log_capacity=1024, first_step=1, max_contacts=48, block_size=0,
                 autotune=False, cells_per_node=0, timeloop=0, contact_skin=0.25, node_order=None):
        L = N.lib()
        self.setup = setup
        self.dim = setup.dim
        cfg = N.Config()
        L.pg_config_default(C.byref(cfg))
        cfg.dt = dt
        cfg.enable_fracture = int(enable_fracture)
        cfg.nl_bdry_only = int(nl_bdry_only)
        cfg.allow_damping = int(allow_damping)
        cfg.allow_friction = int(allow_friction)
        cfg.self_contact = int(self_contact)
        cfg.enable_torque = int(enable_torque)
        cfg.gradient_extforce = int(gradient_extforce)
        cfg.extforce_maxstep = int(extforce_maxstep)
        cfg.precision = N.PG_MIXED if precision == "mixed" else N.PG_FP64
        cfg.record_pairs = int(bool(record_pairs))
        cfg.pair_log_capacity = int(pair_log_capacity)
        cfg.first_step = int(first_step)
        cfg.max_contacts = int(max_contacts)
        cfg.block_size = int(block_size)
        cfg.autotune = int(bool(autotune))
        cfg.cells_per_node = int(cells_per_node)
        cfg.timeloop = 1 if timeloop in (1, "worm") else 0
        cfg.contact_skin = float(contact_skin)
        if node_order is not None:
            cfg.node_order = N.NODE_ORDER[node_order] if isinstance(node_order, str) else int(node_order)
        self.cfg = cfg
        self._desc = setup.desc()
        h = C.c_void_p()
        N.check(L.pg_create(C.byref(self._desc), C.byref(cfg), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            N.lib().pg_destroy(self.h)
            self.h = None
            self._pending = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def step(self, n=1):
        N.check(N.lib().pg_step(self.h, int(n)))

    def step_timed(self, n):
        """Advance n steps; returns the device time in ms (CUDA events on the engine's stream)."""
        ms = C.c_double()
        N.check(N.lib().pg_step_timed(self.h, int(n), C.byref(ms)))
        return ms.value

    def synchronize(self):
        N.check(N.lib().pg_synchronize(self.h))

    def next_step(self):
        t = C.c_uint64()
        N.check(N.lib().pg_get_step(self.h, C.byref(t)))
        return t.value

    def field(self, name):
        out = np.empty((self.setup.n_nodes, self.dim), np.float64)
        N.check(N.lib().pg_get_field(self.h, N.FIELD[name], N.ptr(out, C.c_double)))
        return out

    def set_field(self, name, a):
        a = np.ascontiguousarray(a, np.float64).reshape(self.setup.n_nodes, self.dim)
        N.check(N.lib().pg_set_field(self.h, N.FIELD[name], N.ptr(a, C.c_double)))

    def bond_alive(self):
        out = np.empty(max(1, self.setup.n_bonds), np.uint8)
        N.check(N.lib().pg_get_bond_alive(self.h, N.ptr(out, C.c_uint8)))
        return out[: self.setup.n_bonds]

    def set_bond_alive(self, a):
        a = np.ascontiguousarray(a, np.uint8)
        N.check(N.lib().pg_set_bond_alive(self.h, N.ptr(a, C.c_uint8)))

    def break_step(self):
        out = np.empty(max(1, self.setup.n_bonds), np.uint32)
        N.check(N.lib().pg_get_bond_break_step(self.h, N.ptr(out, C.c_uint32)))
        return out[: self.setup.n_bonds]

    def reaction(self):
        ns = 2 * self.dim
        out = np.empty((self.setup.n_instances, ns, self.dim), np.float64)
        N.check(N.lib().pg_get_reaction(self.h, N.ptr(out, C.c_double)))
        return out

    def wall(self):
        out = np.empty((self.setup.n_instances, 2 * self.dim), np.float64)
        N.check(N.lib().pg_get_wall(self.h, N.ptr(out, C.c_double)))
        return out

    SNAPSHOT_ITEMS = ("CurrPos", "vel", "acc", "force", "disp", "bond_alive", "wall", "reaction")

    def snapshot_buffers(self, items=("CurrPos", "vel", "acc", "force")):
        """Page-locked host arrays for :meth:`snapshot` (the copies then go straight into them)."""
        n, d = self.setup.n_nodes, self.dim
        shapes = {"bond_alive": ((max(1, self.setup.n_bonds),), np.uint8),
                  "wall": ((self.setup.n_instances, 2 * d), np.float64),
                  "reaction": ((self.setup.n_instances, 2 * d, d), np.float64)}
        specs = [(k,) + shapes.get(k, ((n, d), np.float64)) for k in items]
        sizes = [(int(np.prod(sh)) * np.dtype(dt).itemsize + 255) // 256 * 256 for _, sh, dt in specs]
        block = pinned_empty((max(1, sum(sizes)),), np.uint8)  # one page-locked allocation for all
        out, at = {}, 0
        for (k, sh, dt), nb in zip(specs, sizes):
            cnt = int(np.prod(sh))
            out[k] = block[at: at + cnt * np.dtype(dt).itemsize].view(dt).reshape(sh)
            at += nb
        return out

    def snapshot(self, items=("CurrPos", "vel", "acc", "force"), out=None):
        """Enqueue an asynchronous snapshot (pg_snapshot) of the state after the steps issued so far
        and return a :class:`Snapshot`; its ``wait()`` returns the arrays. The copies overlap steps
        issued before ``wait()``. ``out`` (e.g. from :meth:`snapshot_buffers`) receives the copies;
        by default new arrays are made."""
        bad = [k for k in items if k not in self.SNAPSHOT_ITEMS]
        if bad:
            raise ValueError("unknown snapshot item(s): %s" % bad)
        n, d = self.setup.n_nodes, self.dim
        arrs = {}
        for k in items:
            if out is not None and k in out:
                arrs[k] = out[k]
            elif k == "bond_alive":
                arrs[k] = np.empty(max(1, self.setup.n_bonds), np.uint8)
            elif k == "wall":
                arrs[k] = np.empty((self.setup.n_instances, 2 * d), np.float64)
            elif k == "reaction":
                arrs[k] = np.empty((self.setup.n_instances, 2 * d, d), np.float64)
            else:
                arrs[k] = np.empty((n, d), np.float64)
        for k, a in arrs.items():
            want = np.uint8 if k == "bond_alive" else np.float64
            if a.dtype != want or not a.flags.c_contiguous:
                raise ValueError("snapshot buffer %s: C-contiguous %s expected" % (k, np.dtype(want).name))
        snap = Snapshot(self, arrs)
        desc = N.SnapshotDesc()
        names = {"CurrPos": "currpos", "vel": "vel", "acc": "acc", "force": "force", "disp": "disp",
                 "bond_alive": "bond_alive", "wall": "wall", "reaction": "reaction"}
        for k, a in arrs.items():
            setattr(desc, names[k], a.ctypes.data)
        desc.too_close_events = C.addressof(snap._too_close)
        desc.last_step = C.addressof(snap._last_step)
        # the engine writes into the buffers of a snapshot in flight until it is waited for (or the
        # next snapshot completes it): keep them alive until then
        prev = getattr(self, "_pending", None)
        N.check(N.lib().pg_snapshot(self.h, C.byref(desc)))
        if prev is not None:
            prev._done = True
        self._pending = snap
        return snap

    def set_grain_flags(self, grain, movable=-1, stoppable=-1):
        N.check(N.lib().pg_set_grain_flags(self.h, int(grain), int(movable), int(stoppable)))

    def pair_log(self, n):
        c = np.empty(n, np.uint64)
        hs = np.empty(n, np.uint64)
        N.check(N.lib().pg_get_pair_log(self.h, int(n), N.ptr(c, C.c_uint64), N.ptr(hs, C.c_uint64)))
        return c, hs

    def postprocess(self, node_damage=False):
        """On-device post-processing of the current state (pg_postprocess): grain means of vel,
        acc and CurrPos, grain force sums, grain and (optionally) node damage, per-instance
        sum of vol*rho*acc and volume fraction."""
        G, I, D, Nn = self.setup.n_grains, self.setup.n_instances, self.dim, self.setup.n_nodes
        out = dict(grain_mean_vel=np.empty((G, D)), grain_mean_acc=np.empty((G, D)),
                   grain_mean_currpos=np.empty((G, D)), grain_force=np.empty((G, D)),
                   grain_damage=np.empty(G), inertial_force=np.empty((I, D)), volume_fraction=np.empty(I))
        if node_damage:
            out["node_damage"] = np.empty(Nn)
        p = N.Post()
        for k, v in out.items():
            setattr(p, k, N.ptr(v, C.c_double))
        N.check(N.lib().pg_postprocess(self.h, C.byref(p)))
        return out

    def device_status(self):
        st = C.c_int32()
        tc = C.c_uint64()
        N.check(N.lib().pg_get_device_status(self.h, C.byref(st), C.byref(tc)))
        return st.value, tc.value

    def node_order(self):
        """(name of the node layout in use, whether it differs from the input's order)."""
        o, p = C.c_int32(), C.c_int32()
        N.check(N.lib().pg_get_node_order(self.h, C.byref(o), C.byref(p)))
        names = {v: k for k, v in N.NODE_ORDER.items()}
        return names.get(o.value, str(o.value)), bool(p.value)

    def contact_skin(self):
        """Candidate-list skin in use (fraction of R_c; 0: grid search every step)."""
        v = C.c_double()
        N.check(N.lib().pg_get_contact_skin(self.h, C.byref(v)))
        return v.value

    def launch_count(self):
        n = C.c_uint64()
        N.check(N.lib().pg_get_launch_count(self.h, C.byref(n)))
        return n.value

    def launch_config(self):
        b, c = C.c_uint32(), C.c_uint32()
        N.check(N.lib().pg_get_launch_config(self.h, C.byref(b), C.byref(c)))
        return dict(block_size=b.value, cells_per_node=c.value)

    def set_timing(self, on):
        N.check(N.lib().pg_set_timing(self.h, int(bool(on))))

    def kernel_times(self):
        f, t, n = C.c_double(), C.c_double(), C.c_uint64()
        N.check(N.lib().pg_get_kernel_times(self.h, C.byref(f), C.byref(t), C.byref(n)))
        return f.value, t.value, n.value


def run_simulation(root=".", dim=2, precision="fp64"):
    """bin/simulate{2,3}d in-process: reads <root>/config/main.conf and <root>/data/hdf5/all.h5,
    writes <root>/output/hdf5/."""
    p = N.PG_MIXED if precision == "mixed" else N.PG_FP64
    N.check(N.lib().pg_run_simulation(str(root).encode(), int(dim), p))


def select_device(device):
    N.check(N.lib().pg_select_device(int(device)))


def device_count():
    n = C.c_int32()
    rc = N.lib().pg_device_count(C.byref(n))
    return n.value if rc == N.PG_OK else 0


class Snapshot:
    """An asynchronous snapshot in flight (pg_snapshot); ``wait()`` (pg_wait) returns a dict of the
    requested arrays plus ``too_close_events`` and ``last_step``. The arrays hold the state after
    the steps issued before the snapshot, whatever was issued after it."""

    def __init__(self, sim, arrays):
        self._sim = sim
        self.arrays = arrays
        self._too_close = C.c_uint64()
        self._last_step = C.c_uint64()
        self._done = False

    def wait(self):
        if not self._done:
            self._done = True
            if getattr(self._sim, "_pending", None) is self:
                self._sim._pending = None
            N.check(N.lib().pg_wait(self._sim.h))
        out = dict(self.arrays)
        if "bond_alive" in out:
            out["bond_alive"] = out["bond_alive"][: self._sim.setup.n_bonds]
        out["too_close_events"] = self._too_close.value
        out["last_step"] = self._last_step.value
        return out


def pinned_empty(shape, dtype=np.float64):
    """A numpy array in page-locked host memory (pg_host_alloc), freed with the array."""
    dtype = np.dtype(dtype)
    nbytes = max(1, int(np.prod(shape)) * dtype.itemsize)
    L = N.lib()
    p = C.c_void_p()
    N.check(L.pg_host_alloc(nbytes, C.byref(p)))
    buf = (C.c_uint8 * nbytes).from_address(p.value)
    weakref.finalize(buf, L.pg_host_free, C.c_void_p(p.value))
    return np.frombuffer(buf, dtype, count=int(np.prod(shape))).reshape(shape)
