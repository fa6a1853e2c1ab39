"""Handle creation on a GPU: malformed bond rows are rejected by the device-side check of the
uploaded CSR with the same status and message as the host check (tests/test_capi.py covers the
host path), and a valid setup still creates."""
import ctypes as C

import numpy as np
import pytest

from perigrain_gb300 import _native as N
from perigrain_gb300 import setups

pytestmark = pytest.mark.gpu


def _create(s):
    d = s.desc()
    cfg = N.Config()
    N.lib().pg_config_default(C.byref(cfg))
    h = C.c_void_p()
    rc = N.lib().pg_create(C.byref(d), C.byref(cfg), C.byref(h))
    if rc == N.PG_OK:
        N.lib().pg_destroy(h)
    return rc, N.lib().pg_last_error()


def test_neighbour_outside_grain_rejected_on_device():
    s = setups.small_pair()
    s.bond_local[5] = 10 ** 6
    rc, msg = _create(s)
    row = int(np.searchsorted(s.bond_offset, 5, side="right") - 1)
    assert rc == N.PG_EINVAL and msg == b"bond of node %d points outside its grain" % row


def test_decreasing_offsets_rejected_on_device():
    s = setups.small_pair()
    s.bond_offset[3], s.bond_offset[4] = s.bond_offset[4], s.bond_offset[3]
    rc, msg = _create(s)
    assert rc == N.PG_EINVAL and msg == b"bond_offset decreasing"


def test_valid_setup_creates():
    rc, _ = _create(setups.small_pair())
    assert rc == N.PG_OK
