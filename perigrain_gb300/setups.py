"""Seeded synthetic PeriDEM setups in the reference's data layout.

A :class:`Setup` holds, for one or more independent simulations ("instances"), exactly what
``data/hdf5/all.h5`` holds for one (writer ``exp_dict.py:705-768``, reader
``src/read/load_hdf5.h:42-201``): per-grain node positions, volumes, bond lists (``Connectivity``
turned into neighbour rows by ``conn2NArr``, ``load_hdf5.h:28-38``), nonlocal boundary nodes,
clamped nodes, initial disp/vel/acc/extforce, material scalars, flags, and the pairwise contact
and wall parameters.

Meshes are generated here instead of by gmsh (absent): nodes on a uniform or seeded jittered
grid inside the shape, node volume = h**dim, bonds between nodes with ``|x_j - x_i| <= delta``
(the rule of ``exp_dict.py:171-222``), nonlocal boundary nodes = nodes within the contact radius
of a mesh-edge node (``exp_dict.py:284-301``). Material constants follow ``peridem`` /
``peridem_3d`` (``material_dict.py:61-82``, ``:186-197``).

The named workloads ``workload(k)`` are the five benchmark configurations (two-disk collision,
2D settling, 3D sphere settling, batched two-grain ensemble, 2D compaction).
"""
import ctypes as C
import math
from dataclasses import dataclass, field
from typing import List

import numpy as np

from . import _native as N

# peridem (material_dict.py:61-82)
BULK = 2.0e9
SHEAR = 1.33e9
RHO = 1200.0
GNOT = 135.0


def peridem_2d(delta, K=BULK, G=SHEAR, Gnot=GNOT):
    nu = (3 * K - 2 * G) / (2 * (3 * K + G))
    E = 9 * K * G / (9 * K + G)
    cnot = 24 * E / ((1 - nu) * np.pi * (delta ** 3))
    snot = np.sqrt(4 * np.pi * Gnot / (9 * E * delta))
    return cnot, snot


def contact_stiffness(delta, power=4, K=BULK):
    """Normal contact stiffness 18 K / (pi delta**power). The reference's experiments use
    power 4 (exp_dict.py:1403, :1991, ...). With power 5 the contact spring is ~1/delta stiffer
    and the explicit step at dt = 2e-8 s is unstable at first contact (omega*dt >> 2)."""
    return 18 * K / (np.pi * delta ** power)


def shape_area(shape, r, nsides=6, dim=2):
    if dim == 3:
        return 4.0 / 3.0 * math.pi * r ** 3
    if shape == "disk":
        return math.pi * r * r
    if shape == "ngon":
        return 0.5 * nsides * r * r * math.sin(2 * math.pi / nsides)
    if shape == "plus":
        return 20.0 / 9.0 * r * r
    if shape == "square":
        return 2.0 * r * r
    raise ValueError(shape)


def peridem_3d(delta, K=BULK, Gnot=GNOT):
    cnot = 18 * K / (np.pi * delta ** 4)
    snot = np.sqrt(5 * Gnot / (9 * K * delta))
    return cnot, snot


# ---------------------------------------------------------------------------------------------
# shapes
# ---------------------------------------------------------------------------------------------
def _inside(shape, p, r, nsides=6):
    x, y = p[:, 0], p[:, 1]
    if shape == "disk":
        return x * x + y * y <= r * r
    if shape == "ngon":
        ok = np.ones(len(p), bool)
        apothem = r * math.cos(math.pi / nsides)
        for k in range(nsides):
            a = 2 * math.pi * (k + 0.5) / nsides
            ok &= x * math.cos(a) + y * math.sin(a) <= apothem
        return ok
    if shape == "plus":
        w = r / 3.0
        return ((np.abs(x) <= r) & (np.abs(y) <= w)) | ((np.abs(x) <= w) & (np.abs(y) <= r))
    if shape == "square":
        s = r / math.sqrt(2.0)
        return (np.abs(x) <= s) & (np.abs(y) <= s)
    if shape == "sphere":
        return (p * p).sum(1) <= r * r
    raise ValueError(shape)


def grid_nodes(shape, r, h, dim=2, nsides=6, jitter=0.0, rng=None, angle=0.0):
    """Grid points (spacing h) inside the shape, optionally jittered by U(-jitter*h, jitter*h)
    and rotated by `angle` (2D). Returns local positions and edge flags."""
    k = int(math.ceil(r / h)) + 1
    ax = np.arange(-k, k + 1, dtype=np.float64) * h
    if dim == 2:
        X, Y = np.meshgrid(ax, ax, indexing="xy")
        p = np.stack([X.ravel(), Y.ravel()], 1)
    else:
        X, Y, Z = np.meshgrid(ax, ax, ax, indexing="xy")
        p = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    keep = _inside(shape, p, r, nsides)
    p = p[keep]
    # mesh-edge nodes: a grid neighbour at distance h lies outside the shape
    edge = np.zeros(len(p), bool)
    for a in range(dim):
        for s in (-1.0, 1.0):
            q = p.copy()
            q[:, a] += s * h
            edge |= ~_inside(shape, q, r, nsides)
    if jitter > 0:
        p = p + rng.uniform(-jitter * h, jitter * h, size=p.shape)
    if dim == 2 and angle != 0.0:
        c, s = math.cos(angle), math.sin(angle)
        p = p @ np.array([[c, s], [-s, c]])
    return p, edge


def bond_pairs(pos, delta):
    """Lexicographic (i < j) pairs with sqrt(sum((p_j - p_i)**2)) <= delta, the order
    itertools.combinations gives in exp_dict.py:199-222."""
    from scipy.spatial import cKDTree

    t = cKDTree(pos)
    pr = t.query_pairs(delta * (1 + 1e-9), output_type="ndarray")
    if len(pr) == 0:
        return np.zeros((0, 2), np.int64)
    i, j = np.minimum(pr[:, 0], pr[:, 1]), np.maximum(pr[:, 0], pr[:, 1])
    d = np.sqrt(np.sum(np.square(pos[j] - pos[i]), axis=1))
    ok = d <= delta
    pr = np.stack([i[ok], j[ok]], 1)
    order = np.lexsort((pr[:, 1], pr[:, 0]))
    return pr[order].astype(np.int64)


def conn_to_rows(conn, n):
    """conn2NArr (load_hdf5.h:28-38): row (i, j) appends j to NArr[i] and i to NArr[j]."""
    conn = np.asarray(conn, np.int64).reshape(-1, 2)
    src = np.stack([conn[:, 0], conn[:, 1]], 1).ravel()
    dst = np.stack([conn[:, 1], conn[:, 0]], 1).ravel()
    order = np.argsort(src, kind="stable")
    off = np.zeros(n + 1, np.uint64)
    np.add.at(off, src + 1, 1)
    off = np.cumsum(off).astype(np.uint64)
    return off, dst[order].astype(np.uint32)


def rows_to_conn(off, loc):
    """NbdArr2conn (timeloop.h:25-49): pairs (i, q), i < q, in row order."""
    n = len(off) - 1
    i = np.repeat(np.arange(n, dtype=np.int64), np.diff(off.astype(np.int64)))
    q = loc.astype(np.int64)
    keep = i < q
    return np.stack([i[keep], q[keep]], 1)


@dataclass
class Grain:
    pos: np.ndarray
    vol: np.ndarray
    conn: np.ndarray
    bdry: np.ndarray
    delta: float
    rho: float
    cnot: float
    snot: float
    vel: np.ndarray = None
    disp: np.ndarray = None
    acc: np.ndarray = None
    extforce: np.ndarray = None
    clamped: np.ndarray = None
    movable: int = 1
    breakable: int = 1
    stoppable: int = 1
    torque_axis: int = 2
    torque_val: float = 0.0


def make_grain(shape, r, h, center, dim=2, nsides=6, jitter=0.0, rng=None, angle=0.0,
               delta_factor=3.0, contact_radius=None, material="peridem"):
    p, edge = grid_nodes(shape, r, h, dim, nsides, jitter, rng, angle)
    p = p + np.asarray(center, np.float64)[None, :]
    delta = delta_factor * h
    if jitter == 0.0:
        delta = delta * (1 + 1e-12)  # keep grid pairs at exactly delta on the bonded side
    cnot, snot = (peridem_2d(delta) if dim == 2 else peridem_3d(delta))
    conn = bond_pairs(p, delta)
    rc = contact_radius if contact_radius is not None else delta / 5
    # nonlocal boundary nodes: within rc of a mesh-edge node (exp_dict.py:284-301)
    from scipy.spatial import cKDTree

    e = np.nonzero(edge)[0]
    if len(e):
        t = cKDTree(p)
        hits = t.query_ball_point(p[e], rc)
        bd = np.unique(np.concatenate([np.asarray(x, np.int64) for x in hits] + [e]))
    else:
        bd = np.zeros(0, np.int64)
    n = len(p)
    z = np.zeros((n, dim))
    return Grain(pos=p, vol=np.full(n, h ** dim), conn=conn, bdry=bd, delta=delta, rho=RHO, cnot=cnot,
                 snot=snot, vel=z.copy(), disp=z.copy(), acc=z.copy(), extforce=z.copy(),
                 clamped=np.zeros(0, np.int64))


# ---------------------------------------------------------------------------------------------
# Setup: arrays in the C-ABI layout
# ---------------------------------------------------------------------------------------------
@dataclass
class Setup:
    dim: int
    grain_instance: np.ndarray
    grain_node_offset: np.ndarray
    pos: np.ndarray
    vol: np.ndarray
    disp: np.ndarray
    vel: np.ndarray
    acc: np.ndarray
    extforce: np.ndarray
    bond_offset: np.ndarray
    bond_local: np.ndarray
    bdry_offset: np.ndarray
    bdry_nodes: np.ndarray
    clamped_offset: np.ndarray
    clamped_nodes: np.ndarray
    delta: np.ndarray
    rho: np.ndarray
    cnot: np.ndarray
    snot: np.ndarray
    movable: np.ndarray
    breakable: np.ndarray
    stoppable: np.ndarray
    break_bonds: np.ndarray
    torque_axis: np.ndarray
    torque_val: np.ndarray
    contact_radius: np.ndarray
    normal_stiffness: np.ndarray
    friction_coefficient: np.ndarray
    damping_ratio: np.ndarray
    allow_wall: np.ndarray
    wall_geom: np.ndarray
    wall_speed: np.ndarray
    name: str = ""
    _keep: list = field(default_factory=list, repr=False)

    @property
    def n_nodes(self):
        return int(self.grain_node_offset[-1])

    @property
    def n_grains(self):
        return len(self.grain_instance)

    @property
    def n_instances(self):
        return len(self.contact_radius)

    @property
    def n_bonds(self):
        return int(self.bond_offset[-1])

    def desc(self):
        """pg_setup_desc pointing at this setup's arrays (kept alive by the setup)."""
        d = N.SetupDesc()
        d.dim, d.n_instances, d.n_grains, d.n_nodes = self.dim, self.n_instances, self.n_grains, self.n_nodes
        typ = {np.float64: C.c_double, np.uint32: C.c_uint32, np.uint64: C.c_uint64, np.int32: C.c_int32,
               np.uint8: C.c_uint8}
        for name, _ in N.SetupDesc._fields_[4:]:
            a = getattr(self, name)
            a = np.ascontiguousarray(a)
            setattr(self, name, a)
            if a.size == 0:
                a = np.zeros(1, a.dtype)
                self._keep.append(a)
            setattr(d, name, a.ctypes.data_as(C.POINTER(typ[a.dtype.type])))
        return d

    def copy(self):
        kw = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in self.__dict__.items() if k != "_keep"}
        return Setup(**kw)

    def instance_nodes(self, k):
        g = np.nonzero(self.grain_instance == k)[0]
        return int(self.grain_node_offset[g[0]]), int(self.grain_node_offset[g[-1] + 1])

    def save_h5(self, path):
        """Write all.h5 (Experiment.save layout) for a single-instance setup."""
        assert self.n_instances == 1
        L = N.lib()
        h = C.c_void_p()
        d = self.desc()
        N.check(L.pg_setup_from_desc(C.byref(d), C.byref(h)))
        try:
            N.check(L.pg_setup_save(h, str(path).encode()))
        finally:
            L.pg_setup_free(h)


def build_setup(grains: List[Grain], dim, contact_radius, normal_stiffness, friction, damping,
                allow_wall=0, wall=None, wall_speed=None, instance_of=None, name=""):
    """Assemble grains into a Setup. Contact and wall parameters may be scalars (one instance)
    or per-instance sequences; instance_of[g] gives the instance of grain g."""
    G = len(grains)
    if instance_of is None:
        instance_of = np.zeros(G, np.uint32)
    instance_of = np.asarray(instance_of, np.uint32)
    I = int(instance_of.max()) + 1 if G else 1

    def per_inst(x, default=0.0):
        a = np.asarray(x if x is not None else default, np.float64)
        return np.broadcast_to(a, (I,) if a.ndim == 0 else a.shape).astype(np.float64).copy()

    nodes = np.array([len(g.pos) for g in grains], np.int64)
    goff = np.zeros(G + 1, np.uint32)
    goff[1:] = np.cumsum(nodes)
    cat = lambda attr: np.concatenate([getattr(g, attr).reshape(len(g.pos), -1) for g in grains]).reshape(-1)
    boff, bloc = [np.zeros(1, np.uint64)], []
    base = 0
    for g in grains:
        off, loc = conn_to_rows(g.conn, len(g.pos))
        boff.append(off[1:] + np.uint64(base))
        bloc.append(loc)
        base += int(off[-1])
    bd_off = np.zeros(G + 1, np.uint32)
    bd_off[1:] = np.cumsum([len(g.bdry) for g in grains])
    cl_off = np.zeros(G + 1, np.uint32)
    cl_off[1:] = np.cumsum([len(g.clamped) for g in grains])
    ns = 2 * dim
    if wall is None:
        wall = np.zeros((I, ns))
    wall = np.asarray(wall, np.float64).reshape(-1, ns)
    if len(wall) == 1 and I > 1:
        wall = np.repeat(wall, I, 0)
    if wall_speed is None:
        wall_speed = np.zeros((I, ns))
    wall_speed = np.asarray(wall_speed, np.float64).reshape(-1, ns)
    if len(wall_speed) == 1 and I > 1:
        wall_speed = np.repeat(wall_speed, I, 0)
    aw = np.asarray(allow_wall, np.int32)
    aw = np.broadcast_to(aw, (I,)).astype(np.int32).copy()
    return Setup(
        dim=dim, grain_instance=instance_of, grain_node_offset=goff,
        pos=cat("pos"), vol=np.concatenate([g.vol for g in grains]).astype(np.float64),
        disp=cat("disp"), vel=cat("vel"), acc=cat("acc"), extforce=cat("extforce"),
        bond_offset=np.concatenate(boff).astype(np.uint64), bond_local=np.concatenate(bloc).astype(np.uint32),
        bdry_offset=bd_off, bdry_nodes=np.concatenate([g.bdry for g in grains]).astype(np.uint32),
        clamped_offset=cl_off, clamped_nodes=np.concatenate([g.clamped for g in grains]).astype(np.uint32),
        delta=np.array([g.delta for g in grains]), rho=np.array([g.rho for g in grains]),
        cnot=np.array([g.cnot for g in grains]), snot=np.array([g.snot for g in grains]),
        movable=np.array([g.movable for g in grains], np.int32),
        breakable=np.array([g.breakable for g in grains], np.int32),
        stoppable=np.array([g.stoppable for g in grains], np.int32),
        break_bonds=np.ones(G, np.uint8),
        torque_axis=np.array([g.torque_axis for g in grains], np.uint32),
        torque_val=np.array([g.torque_val for g in grains], np.float64),
        contact_radius=per_inst(contact_radius), normal_stiffness=per_inst(normal_stiffness),
        friction_coefficient=per_inst(friction), damping_ratio=per_inst(damping),
        allow_wall=aw, wall_geom=wall.reshape(-1).copy(), wall_speed=wall_speed.reshape(-1).copy(), name=name)


def concat(setups: List[Setup], name=""):
    """Batch independent single-instance setups into one multi-instance setup."""
    dim = setups[0].dim
    gi, goff, boff, bl, bdo, bdn, clo, cln = [], [np.zeros(1, np.uint32)], [np.zeros(1, np.uint64)], [], \
        [np.zeros(1, np.uint32)], [], [np.zeros(1, np.uint32)], []
    nb = nn = nbd = ncl = ninst = 0
    for s in setups:
        gi.append(s.grain_instance + ninst)
        goff.append(s.grain_node_offset[1:] + np.uint32(nn))
        boff.append(s.bond_offset[1:] + np.uint64(nb))
        bl.append(s.bond_local)
        bdo.append(s.bdry_offset[1:] + np.uint32(nbd))
        bdn.append(s.bdry_nodes)
        clo.append(s.clamped_offset[1:] + np.uint32(ncl))
        cln.append(s.clamped_nodes)
        nb += s.n_bonds
        nn += s.n_nodes
        nbd += len(s.bdry_nodes)
        ncl += len(s.clamped_nodes)
        ninst += s.n_instances
    cat = lambda k: np.concatenate([getattr(s, k) for s in setups])
    return Setup(
        dim=dim, grain_instance=np.concatenate(gi).astype(np.uint32),
        grain_node_offset=np.concatenate(goff).astype(np.uint32),
        pos=cat("pos"), vol=cat("vol"), disp=cat("disp"), vel=cat("vel"), acc=cat("acc"), extforce=cat("extforce"),
        bond_offset=np.concatenate(boff).astype(np.uint64), bond_local=np.concatenate(bl).astype(np.uint32),
        bdry_offset=np.concatenate(bdo).astype(np.uint32), bdry_nodes=np.concatenate(bdn).astype(np.uint32),
        clamped_offset=np.concatenate(clo).astype(np.uint32), clamped_nodes=np.concatenate(cln).astype(np.uint32),
        delta=cat("delta"), rho=cat("rho"), cnot=cat("cnot"), snot=cat("snot"), movable=cat("movable"),
        breakable=cat("breakable"), stoppable=cat("stoppable"), break_bonds=cat("break_bonds"),
        torque_axis=cat("torque_axis"), torque_val=cat("torque_val"), contact_radius=cat("contact_radius"),
        normal_stiffness=cat("normal_stiffness"), friction_coefficient=cat("friction_coefficient"),
        damping_ratio=cat("damping_ratio"), allow_wall=cat("allow_wall"), wall_geom=cat("wall_geom"),
        wall_speed=cat("wall_speed"), name=name)


# ---------------------------------------------------------------------------------------------
# named workloads
# ---------------------------------------------------------------------------------------------
def two_disk_collision(r=1e-3, h=5e-5, gap=1e-4, speed=20.0, jitter_frac=0.05, seed=0, shape_a="disk",
                       shape_b="disk", angle_deg=0.0, nsides=6, mesh_jitter=0.0, kn_power=4):
    """Two grains approaching head-on (or at an impact angle), no wall, no gravity."""
    rng = np.random.default_rng(seed)
    xa = -(r + gap / 2)
    theta = math.radians(angle_deg)
    off = 2 * r * math.sin(theta)
    a = make_grain(shape_a, r, h, (xa, 0.0), nsides=nsides, jitter=mesh_jitter, rng=rng)
    b = make_grain(shape_b, r, h, (-xa, off), nsides=nsides, jitter=mesh_jitter, rng=rng)
    va = speed * (1 + rng.uniform(-jitter_frac, jitter_frac))
    vb = speed * (1 + rng.uniform(-jitter_frac, jitter_frac))
    a.vel[:, 0] = va
    b.vel[:, 0] = -vb
    delta = min(a.delta, b.delta)
    rc = delta / 5
    kn = contact_stiffness(delta, kn_power)
    return build_setup([a, b], 2, rc, kn, 0.8, 0.9, allow_wall=0, name="two_disk_collision")


def settling_2d(n_grains=400, rmin=0.6e-3, rmax=1.0e-3, nodes_per_grain=300, width=2e-2, seed=1,
                gravity=9.8, mesh_jitter=0.1, kn_power=4):
    """Mixed shapes (disk, n-gon n=3..8, plus) on a seeded non-overlapping lattice with random
    rotations, settling under gravity in a rectangular box with rigid walls. The box keeps the
    2e-2 width; its height is raised until the lattice holds every grain without overlap."""
    rng = np.random.default_rng(seed)
    pitch = 2 * rmax * 1.08
    ncol = max(1, int(width // pitch))
    nrow = int(math.ceil(n_grains / ncol))
    height = max(4e-2, nrow * pitch + pitch)
    grains = []
    for k in range(n_grains):
        r = rng.uniform(rmin, rmax)
        kind = rng.integers(0, 3)
        shape, ns = ("disk", 6) if kind == 0 else (("ngon", int(rng.integers(3, 9))) if kind == 1 else ("plus", 4))
        h = math.sqrt(shape_area(shape, r, ns) / nodes_per_grain)
        cx = (k % ncol + 0.5) * (width / ncol)
        cy = (k // ncol + 0.5) * pitch + 0.5 * pitch
        g = make_grain(shape, r, h, (cx, cy), nsides=ns, jitter=mesh_jitter, rng=rng,
                       angle=rng.uniform(0, 2 * math.pi))
        g.extforce[:, 1] = -gravity * g.rho
        g.acc[:, 1] = -gravity
        grains.append(g)
    delta = min(g.delta for g in grains)
    rc = delta / 5
    kn = contact_stiffness(delta, kn_power)
    wall = [0.0, width, height, 0.0]
    return build_setup(grains, 2, rc, kn, 0.8, 0.9, allow_wall=1, wall=wall, name="settling_2d")


def spheres_3d(n=64, rmin=0.8e-3, rmax=1.2e-3, nodes_per_grain=2000, box=1e-2, seed=2, gravity=9.8,
               mesh_jitter=0.1, friction=0.5, kn_power=4):
    """Spheres on a seeded jittered cubic grid, placed on a non-overlapping lattice in a cube."""
    rng = np.random.default_rng(seed)
    m = int(round(n ** (1 / 3)))
    while m ** 3 < n:
        m += 1
    pitch = box / m
    grains = []
    for k in range(n):
        r = rng.uniform(rmin, rmax)
        h = r * (4 * math.pi / 3 / nodes_per_grain) ** (1 / 3)
        ix, iy, iz = k % m, (k // m) % m, k // (m * m)
        c = ((ix + 0.5) * pitch, (iy + 0.5) * pitch, (iz + 0.5) * pitch)
        g = make_grain("sphere", r, h, c, dim=3, jitter=mesh_jitter, rng=rng)
        g.extforce[:, 2] = -gravity * g.rho
        g.acc[:, 2] = -gravity
        grains.append(g)
    delta = min(g.delta for g in grains)
    rc = delta / 5
    kn = contact_stiffness(delta, kn_power)
    wall = [0.0, 0.0, 0.0, box, box, box]
    return build_setup(grains, 3, rc, kn, friction, 0.9, allow_wall=1, wall=wall, name="spheres_3d")


def collision_ensemble(n_inst=256, rmin=0.5e-3, rmax=1.5e-3, h=6.25e-5, seed=3, smin=5.0, smax=40.0,
                       amax=60.0, kn_power=4):
    """Independent two-grain collisions (disk or n-gon) with seeded radius, impact speed and angle."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_inst):
        r = float(rng.uniform(rmin, rmax))
        sa = "disk" if rng.integers(0, 2) == 0 else "ngon"
        sb = "disk" if rng.integers(0, 2) == 0 else "ngon"
        ns = int(rng.integers(3, 9))
        sp = float(rng.uniform(smin, smax))
        ang = float(rng.uniform(0, amax))
        s = two_disk_collision(r=r, h=h, gap=1e-4, speed=sp / 2, jitter_frac=0.0, seed=seed * 100003 + k,
                               shape_a=sa, shape_b=sb, angle_deg=ang, nsides=ns, kn_power=kn_power)
        out.append(s)
    return concat(out, name="collision_ensemble")


def compaction_2d(n_grains=50, r=0.6e-3, nodes_per_grain=400, seed=4, wall_speed=-1.0, kn_power=4, gap_frac=0.5,
                  stir=2.0):
    """Disks and axis-aligned squares (half side r) on a 5-column lattice whose node extents are
    gap_frac * R_c apart, in a box whose walls sit gap_frac/2 * R_c outside the outermost nodes; the
    top wall moves at wall_speed (m/s). Seeded grain velocities U(-stir, stir) m/s per component
    keep every grain in contact with its neighbours during a 5000-step run."""
    rng = np.random.default_rng(seed)
    ncol = 5
    nrow = int(math.ceil(n_grains / ncol))
    grains = []
    for k in range(n_grains):
        shape = "disk" if rng.integers(0, 2) == 0 else "square"
        rs = r if shape == "disk" else r * math.sqrt(2.0)
        h = math.sqrt(shape_area(shape, rs) / nodes_per_grain)
        grains.append(make_grain(shape, rs, h, (0.0, 0.0), jitter=0.1, rng=rng))
    delta = min(g.delta for g in grains)
    rc = delta / 5
    gap = gap_frac * rc
    ext = max(float(np.abs(g.pos).max()) for g in grains)  # largest half extent of the node sets
    pitch = 2 * ext + gap
    for k, g in enumerate(grains):
        g.pos = g.pos + np.array([(k % ncol + 0.5) * pitch, (k // ncol + 0.5) * pitch])
        g.vel[:, 0] = rng.uniform(-stir, stir)
        g.vel[:, 1] = rng.uniform(-stir, stir)
    kn = contact_stiffness(delta, kn_power)
    wall = [0.0, ncol * pitch, nrow * pitch, 0.0]
    speed = [0.0, 0.0, wall_speed, 0.0]
    return build_setup(grains, 2, rc, kn, 0.8, 0.9, allow_wall=1, wall=wall, wall_speed=speed, name="compaction_2d")


WORKLOADS = {
    0: dict(name="two_disk_collision", dt=2e-8, steps=20000, modulo=100, build=two_disk_collision),
    1: dict(name="settling_2d", dt=1e-8, steps=50000, modulo=100, build=settling_2d),
    2: dict(name="spheres_3d", dt=1e-8, steps=20000, modulo=100, build=spheres_3d),
    3: dict(name="collision_ensemble", dt=2e-8, steps=10000, modulo=100, build=collision_ensemble),
    4: dict(name="compaction_2d", dt=2e-8, steps=5000, modulo=100, build=compaction_2d),
}


def workload(k, **kw):
    return WORKLOADS[k]["build"](**kw)


def small_pair(dim=2, r=2.5e-4, h=5e-5, speed=30.0, gap=2e-5, seed=7, wall=False, clamp=False, torque=False,
               extforce=False, shape="disk", jitter=0.1, n_grains=2, kn_power=4, wall_speed=0.5):
    """A few-hundred-node setup that exercises every branch (fracture, self-contact, friction,
    damping, walls, clamped nodes, torque, external force) -- small enough for the reference."""
    rng = np.random.default_rng(seed)
    grains = []
    shape3 = "sphere" if dim == 3 else shape
    for k in range(n_grains):
        x = (k - (n_grains - 1) / 2) * (2 * r + gap)
        c = (x, 0.3 * r * (k % 2)) if dim == 2 else (x, 0.3 * r * (k % 2), 0.0)
        g = make_grain(shape3 if k % 2 == 0 else ("ngon" if dim == 2 else "sphere"), r, h, c, dim=dim,
                       nsides=5, jitter=jitter, rng=rng, angle=0.3 * k)
        g.vel[:, 0] = speed * (1 if x < 0 else -1) * (1 + 0.1 * rng.uniform(-1, 1))
        g.vel[:, 1] = speed * 0.3 * rng.uniform(-1, 1)
        if extforce:
            g.extforce[:, 1] = -9.8e5 * g.rho
        if torque:
            g.torque_val = 1e9 * (1 if k % 2 else -1)
            g.torque_axis = 2
        if clamp and k == 0:
            g.clamped = np.array([0, 1], np.int64)
        grains.append(g)
    delta = min(g.delta for g in grains)
    rc = delta / 5
    kn = contact_stiffness(delta, kn_power)
    ns = 2 * dim
    if wall:
        lo = min(g.pos[:, 0].min() for g in grains) - 0.5 * rc
        hi = max(g.pos[:, 0].max() for g in grains) + 0.5 * rc
        blo = min(g.pos[:, 1].min() for g in grains) - 0.3 * rc
        bhi = max(g.pos[:, 1].max() for g in grains) + 2 * r
        if dim == 2:
            w = [lo, hi, bhi, blo]
        else:
            zlo = min(g.pos[:, 2].min() for g in grains) - 0.3 * rc
            zhi = max(g.pos[:, 2].max() for g in grains) + 0.3 * rc
            w = [lo, blo, zlo, hi, bhi, zhi]
        sp = np.zeros(ns)
        sp[3 if dim == 2 else 2] = wall_speed  # bottom / z_min moves
    else:
        w, sp = np.zeros(ns), np.zeros(ns)
    return build_setup(grains, dim, rc, kn, 0.8, 0.9, allow_wall=int(wall), wall=w, wall_speed=sp,
                       name="small_pair")
