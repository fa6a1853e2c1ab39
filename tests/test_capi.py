"""The C-ABI library loads without a GPU and exports every function the public headers declare."""
import ctypes as C
import os
import re

import numpy as np

from perigrain_gb300 import _native as N
from perigrain_gb300 import setups

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in ("perigrain.h", "perigrain_io.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\**(pg_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_every_declared_symbol_is_exported():
    L = N.lib()
    names = declared_functions()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    bound = {p[0] for p in N.PROTOTYPES}
    assert set(names) <= bound, set(names) - bound


def test_status_strings_and_defaults():
    L = N.lib()
    assert L.pg_version() == 1
    assert L.pg_status_string(0) == b"ok"
    assert L.pg_status_string(N.PG_ECAPACITY).startswith(b"device table")
    cfg = N.Config()
    L.pg_config_default(C.byref(cfg))
    assert cfg.dt == 0.02 / 1e5 and cfg.max_contacts == 48 and cfg.first_step == 1


def test_create_validates_before_touching_the_device():
    s = setups.small_pair()
    s.bond_local[0] = 10 ** 6  # neighbour outside the grain
    d = s.desc()
    cfg = N.Config()
    N.lib().pg_config_default(C.byref(cfg))
    h = C.c_void_p()
    rc = N.lib().pg_create(C.byref(d), C.byref(cfg), C.byref(h))
    assert rc == N.PG_EINVAL and b"outside its grain" in N.lib().pg_last_error()


def test_setup_h5_roundtrip(tmp_path):
    s = setups.small_pair(dim=2, wall=True, clamp=True)
    fn = str(tmp_path / "all.h5")
    s.save_h5(fn)
    L = N.lib()
    h = C.c_void_p()
    N.check(L.pg_setup_load(fn.encode(), 2, 0, C.byref(h)))
    d = N.SetupDesc()
    N.check(L.pg_setup_desc_get(h, C.byref(d)))
    n, nb = d.n_nodes, int(d.bond_offset[d.n_nodes])
    assert n == s.n_nodes and nb == s.n_bonds and d.n_grains == s.n_grains
    pos = np.ctypeslib.as_array(d.pos, (n * 2,))
    assert np.array_equal(pos, s.pos)
    assert np.array_equal(np.ctypeslib.as_array(d.bond_local, (nb,)), s.bond_local)
    assert np.array_equal(np.ctypeslib.as_array(d.clamped_nodes, (len(s.clamped_nodes),)), s.clamped_nodes)
    assert list(np.ctypeslib.as_array(d.wall_geom, (4,))) == list(s.wall_geom)
    assert d.contact_radius[0] == s.contact_radius[0]
    L.pg_setup_free(h)


def test_write_tc_from_host_arrays(tmp_path):
    """pg_write_tc: the tc_/wall_ layout (timeloop.h:881-1006) from host arrays, Connectivity from
    the alive bytes (i < q, rows in CSR order), datasets borrowed by the writer without a copy."""
    from perigrain_gb300 import h5

    s = setups.small_pair(dim=2, wall=True)
    L = N.lib()
    h = C.c_void_p()
    d = s.desc()
    N.check(L.pg_setup_from_desc(C.byref(d), C.byref(h)))
    rng = np.random.default_rng(5)
    f = [rng.standard_normal((s.n_nodes, 2)) for _ in range(4)]
    alive = (rng.random(s.n_bonds) > 0.2).astype(np.uint8)
    wall, re_ = rng.standard_normal(4), rng.standard_normal(8)
    out = str(tmp_path)
    N.check(L.pg_write_tc(h, out.encode(), 7, *[N.ptr(a, C.c_double) for a in f], N.ptr(alive, C.c_uint8),
                          N.ptr(wall, C.c_double), N.ptr(re_, C.c_double), 1))
    tc, wf = os.path.join(out, "tc_00007.h5"), os.path.join(out, "wall_00007.h5")
    off = np.asarray(s.grain_node_offset, np.int64)
    bo = np.asarray(s.bond_offset, np.int64)
    for g in range(s.n_grains):
        sl = slice(off[g], off[g + 1])
        for name, a in zip(("CurrPos", "vel", "acc", "force"), f):
            assert np.array_equal(h5.read(tc, "P_%05d/%s" % (g, name)), a[sl])
        conn = []
        for i in range(off[g], off[g + 1]):
            for b in range(bo[i], bo[i + 1]):
                q = int(s.bond_local[b])
                if alive[b] and i - off[g] < q:
                    conn.append([int(i - off[g]), q])
        got = h5.read(tc, "P_%05d/Connectivity" % g, np.uint32)
        assert got.tolist() == conn
    assert np.array_equal(h5.read(wf, "wall_info").ravel(), wall)
    assert np.array_equal(h5.read(wf, "reaction").ravel(), re_)
    L.pg_setup_free(h)
