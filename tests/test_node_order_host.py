"""The device node layout inside the grains (pg_node_order), computed on the host through
pg_debug_node_order, the permutation pg_create lays the arrays out by: a permutation that keeps
every grain's nodes inside the grain; the input order as the identity; the cell order keeping a
generated (already local) mesh as it is and bringing a shuffled mesh's bonded nodes close; the
degree groupings sorting by bond count over the grain or inside 256-node windows of the cell order;
the seeded shuffle deterministic. CPU only (no device is needed)."""
import ctypes as C

import numpy as np
import pytest

from perigrain_gb300 import _native as N
from perigrain_gb300 import setups

INPUT, CELL, CELL_DEGREE, SHUFFLE, CELL_BLOCK_DEGREE = range(5)
WINDOW = 256


def _perm(s, order):
    d = s.desc()
    perm = np.zeros(s.n_nodes, np.uint32)
    permuted = C.c_int32(-1)
    rc = N.lib().pg_debug_node_order(C.byref(d), order, perm.ctypes.data_as(C.c_void_p), C.byref(permuted))
    return rc, perm, permuted.value


def _ok(s, order):
    rc, perm, permuted = _perm(s, order)
    assert rc == N.PG_OK, N.lib().pg_last_error()
    return perm, permuted


def _degree(s):
    return np.diff(s.bond_offset.astype(np.int64))


def _shuffled_grain(seed=3, n=2000):
    """One jittered disk grain whose nodes (and bond rows, boundary lists) are written in a random
    order, as an unordered mesh writer would."""
    rng = np.random.default_rng(seed)
    h = 5e-5
    g = setups.make_grain("disk", h * np.sqrt(n / np.pi), h, (0.0, 0.0), dim=2, jitter=0.1, rng=rng)
    m = len(g.pos)
    p = rng.permutation(m)          # new node k is old node p[k]
    inv = np.empty(m, np.int64)
    inv[p] = np.arange(m)
    for f in ("pos", "vel", "disp", "acc", "extforce"):
        setattr(g, f, getattr(g, f)[p].copy())
    g.vol = g.vol[p].copy()
    c = inv[np.asarray(g.conn, np.int64)]
    c.sort(axis=1)
    g.conn = c[np.lexsort((c[:, 1], c[:, 0]))]
    g.bdry = np.sort(inv[np.asarray(g.bdry, np.int64)])
    return setups.build_setup([g], 2, g.delta / 5, setups.contact_stiffness(g.delta), 0.5, 0.5, name="shuffled")


def _mean_bond_span(s, perm):
    """Mean |device index of j - device index of i| over all bonds in the layout perm."""
    at = np.empty_like(perm)
    at[perm] = np.arange(len(perm), dtype=perm.dtype)
    rows = np.repeat(np.arange(s.n_nodes), _degree(s))
    g0 = np.repeat(s.grain_node_offset[:-1].astype(np.int64), np.diff(s.grain_node_offset.astype(np.int64)))
    j = g0[rows] + s.bond_local.astype(np.int64)
    return float(np.abs(at[j].astype(np.int64) - at[rows].astype(np.int64)).mean())


CASES = {
    "small_pair_2d": lambda: setups.small_pair(dim=2),
    "small_pair_3d": lambda: setups.small_pair(dim=3),
    "two_disk": lambda: setups.two_disk_collision(),
    "shuffled": lambda: _shuffled_grain(),
}


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("order", [INPUT, CELL, CELL_DEGREE, SHUFFLE, CELL_BLOCK_DEGREE])
def test_permutation_stays_inside_grains(case, order):
    s = CASES[case]()
    perm, permuted = _ok(s, order)
    assert np.array_equal(np.sort(perm), np.arange(s.n_nodes))
    off = s.grain_node_offset.astype(np.int64)
    for g in range(s.n_grains):
        seg = perm[off[g]:off[g + 1]].astype(np.int64)
        assert seg.min() >= off[g] and seg.max() < off[g + 1]
    assert permuted == int(not np.array_equal(perm, np.arange(s.n_nodes)))
    if order == INPUT:
        assert permuted == 0


def test_cell_order_keeps_generated_meshes_and_sorts_shuffled_ones():
    # the generated row-major meshes are local already: the cell order keeps them
    for case in ("two_disk", "small_pair_2d"):
        _, permuted = _ok(CASES[case](), CELL)
        assert permuted == 0, case
    s = _shuffled_grain()
    perm, permuted = _ok(s, CELL)
    assert permuted == 1
    ident = np.arange(s.n_nodes, dtype=np.uint32)
    assert _mean_bond_span(s, perm) < 0.1 * _mean_bond_span(s, ident)


@pytest.mark.parametrize("case", sorted(CASES))
def test_degree_groupings(case):
    s = CASES[case]()
    deg = _degree(s)
    off = s.grain_node_offset.astype(np.int64)
    cell, _ = _ok(s, CELL)
    whole, _ = _ok(s, CELL_DEGREE)
    block, _ = _ok(s, CELL_BLOCK_DEGREE)
    for g in range(s.n_grains):
        a, b = off[g], off[g + 1]
        # whole grain: bond counts non-increasing along the device order
        assert np.all(np.diff(deg[whole[a:b]]) <= 0)
        # windows of 256 nodes from the grain's start: sorted inside, and each window holds the
        # cell order's nodes of that window (no node moves 256 places or more)
        for w in range(a, b, WINDOW):
            e = min(b, w + WINDOW)
            assert np.all(np.diff(deg[block[w:e]]) <= 0)
            assert np.array_equal(np.sort(block[w:e]), np.sort(cell[w:e]))
            # stable: equal bond counts keep the cell order's sequence
            pos_in_cell = {int(v): k for k, v in enumerate(cell[w:e])}
            seq = [pos_in_cell[int(v)] for v in block[w:e]]
            for k in range(1, len(seq)):
                if deg[block[w + k]] == deg[block[w + k - 1]]:
                    assert seq[k] > seq[k - 1]


def test_shuffle_is_seeded():
    s = CASES["two_disk"]()
    a, pa = _ok(s, SHUFFLE)
    b, pb = _ok(s, SHUFFLE)
    assert pa == pb == 1 and np.array_equal(a, b)


def test_bad_arguments():
    s = CASES["small_pair_2d"]()
    rc, _, _ = _perm(s, 99)
    assert rc == N.PG_EINVAL
    d = s.desc()
    assert N.lib().pg_debug_node_order(C.byref(d), CELL, None, None) == N.PG_EINVAL
    # a bond pointing outside its grain is rejected before the order is computed
    bad = s.copy()
    bad.bond_local = bad.bond_local.copy()
    bad.bond_local[0] = np.uint32(10 ** 6)
    rc, _, _ = _perm(bad, CELL)
    assert rc == N.PG_EINVAL
