"""pg_build_bonds_noalloc, the bond-list builder for callers that cannot allocate device memory
(allocator hooks that must not re-enter the allocator, hosts with a fixed device-memory budget):
called through the C ABI, it must give
exactly the pairs of the allocating pg_build_bonds, on two calls in a row (the shared scratch keeps
the first call's contents, so the second call proves it clears what it needs). Kept in its own
file, collected last."""
import ctypes as C

import numpy as np
import pytest

from perigrain_gb300 import _native as N
from perigrain_gb300 import setups

pytestmark = pytest.mark.gpu


def _call(entry, d_pos, n, dim, delta, d_pairs, cap):
    L = N.lib()
    fn = getattr(L, entry)
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_double, C.c_void_p, C.c_uint64,
                   C.POINTER(C.c_uint64), C.c_void_p]
    m = C.c_uint64()
    rc = fn(C.c_void_p(d_pos.data_ptr()), n, dim, delta, C.c_void_p(d_pairs.data_ptr()), cap, C.byref(m), None)
    return rc, m.value


def test_noalloc_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(17)
    cases = [("disk", 2, 30), ("sphere", 3, 9)]
    for shape, dim, k in cases:
        h = 5e-5
        p, _ = setups.grid_nodes(shape, k * h, h, dim=dim, jitter=0.1, rng=rng)
        n = len(p)
        d_pos = torch.from_numpy(np.ascontiguousarray(p)).cuda()
        cap = n * (64 if dim == 2 else 256)
        ref = torch.zeros((cap, 2), dtype=torch.int32, device="cuda")
        rc, m_ref = _call("pg_build_bonds", d_pos, n, dim, 3 * h, ref, cap)
        assert rc == 0 and m_ref > 0
        want = ref[:m_ref].cpu().numpy()
        for _ in range(2):
            out = torch.full((cap, 2), -1, dtype=torch.int32, device="cuda")
            rc, m = _call("pg_build_bonds_noalloc", d_pos, n, dim, 3 * h, out, cap)
            assert rc == 0, N.lib().pg_noalloc_last_error()
            assert m == m_ref
            assert np.array_equal(out[:m].cpu().numpy(), want)


def test_noalloc_rejects_oversize():
    torch = pytest.importorskip("torch")
    n = 32768 + 1
    d_pos = torch.zeros((n, 2), dtype=torch.float64, device="cuda")
    out = torch.zeros((16, 2), dtype=torch.int32, device="cuda")
    rc, _ = _call("pg_build_bonds_noalloc", d_pos, n, 2, 1.0, out, 16)
    assert rc == N.PG_EINVAL
    assert b"at most 32768 nodes" in N.lib().pg_noalloc_last_error()
