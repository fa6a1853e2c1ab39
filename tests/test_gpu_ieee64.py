"""The integer FP64 division and square root used by the FP64 force kernel (pg_ieee64.cuh), run on
the GPU through pg_debug_ieee64, return the bits of numpy's IEEE `a / b` and `sqrt(|a|)` on random
operands of every exponent, significands at the edges of the reciprocal estimate's range, exact
squares and their neighbours, and the operands of the bond loop (squared bond lengths, stretches)."""
import ctypes as C

import numpy as np
import pytest

from perigrain_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _run(a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    q = np.empty_like(a)
    r = np.empty_like(a)
    p = lambda x: x.ctypes.data_as(C.c_void_p)
    N.check(N.lib().pg_debug_ieee64(p(a), p(b), a.size, p(q), p(r)))
    return q, r


class _Same:
    """Bitwise equality (NaNs of any payload equal) with the first mismatches in the message."""

    def __init__(self, x, y, args):
        xb, yb = x.view(np.uint64), y.view(np.uint64)
        self.ok = (xb == yb) | (np.isnan(x) & np.isnan(y))
        self.x, self.y, self.args = x, y, args

    def all(self):
        bad = np.flatnonzero(~self.ok)[:5]
        assert bad.size == 0, "%d mismatches, first: %s" % (
            (~self.ok).sum(), [(tuple(float(a[i]).hex() for a in self.args), self.x[i].hex(), self.y[i].hex())
                               for i in bad])
        return True


def _same(got, want, *args):
    return _Same(got, want, args)


def _bits(sign, exp, frac):
    return ((sign.astype(np.uint64) << np.uint64(63)) | (exp.astype(np.uint64) << np.uint64(52))
            | frac.astype(np.uint64)).view(np.float64)


def test_random_operands_every_exponent():
    rng = np.random.default_rng(3)
    n = 1 << 22
    frac = lambda: rng.integers(0, 1 << 52, n, dtype=np.uint64)
    a = _bits(rng.integers(0, 2, n), rng.integers(0, 2048, n), frac())
    b = _bits(rng.integers(0, 2, n), rng.integers(0, 2048, n), frac())
    with np.errstate(all="ignore"):
        q, r = _run(a, b)
        assert _same(q, a / b, a, b).all()
        assert _same(r, np.sqrt(np.abs(a)), a).all()


def test_random_operands_near_each_other():
    rng = np.random.default_rng(4)
    n = 1 << 22
    frac = lambda: rng.integers(0, 1 << 52, n, dtype=np.uint64)
    a = _bits(rng.integers(0, 2, n), 1023 - 40 + rng.integers(0, 80, n), frac())
    b = _bits(rng.integers(0, 2, n), 1023 - 40 + rng.integers(0, 80, n), frac())
    q, r = _run(a, b)
    assert _same(q, a / b, a, b).all()
    assert _same(r, np.sqrt(np.abs(a)), a).all()


def test_edge_significands_and_specials():
    edge = np.array([0, 1, (1 << 52) - 1, (1 << 52) - 2, (1 << 29) - 1, 1 << 29, 1 << 51, (1 << 51) - 1,
                     0x5555555555555, 0xAAAAAAAAAAAAA], dtype=np.uint64)
    fa, fb, de = np.meshgrid(edge, edge, np.arange(-3, 4), indexing="ij")
    one = np.zeros(fa.size, dtype=np.int64)
    a = _bits(one, 1023 + de.ravel(), fa.ravel())
    b = _bits(one, one + 1023, fb.ravel())
    sp = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1.0, -1.0, 5e-324, 2.2250738585072014e-308,
                   1.7976931348623157e308, 1e-310, -1e-310])
    sa, sb = np.meshgrid(sp, sp, indexing="ij")
    a = np.concatenate([a, -a, sa.ravel()])
    b = np.concatenate([b, b, sb.ravel()])
    with np.errstate(all="ignore"):
        q, r = _run(a, b)
        assert _same(q, a / b, a, b).all()
        assert _same(r, np.sqrt(np.abs(a)), a).all()


def test_squares_and_neighbours():
    rng = np.random.default_rng(5)
    s = (1 << 25) + rng.integers(0, 1 << 25, 1 << 20, dtype=np.int64)
    sq = np.ldexp((s * s).astype(np.float64), rng.integers(-40, 40, s.size))
    a = np.concatenate([sq, np.nextafter(sq, np.inf), np.nextafter(sq, 0)])
    x = rng.uniform(1.0, 2.0, 1 << 20)
    a = np.concatenate([a, x * x, np.nextafter(x * x, np.inf)])
    _, r = _run(a, np.ones_like(a))
    assert _same(r, np.sqrt(a), a).all()


def test_bond_loop_operands():
    # squared bond lengths and stretches at the scale of mm-sized grains (lengths 1e-5..1e-3 m)
    rng = np.random.default_rng(6)
    n = 1 << 21
    xin = rng.uniform(1e-5, 1e-3, n)
    en = xin * (1 + rng.normal(0, 1e-3, n))
    e = en * rng.uniform(-1, 1, n)
    q, r = _run(np.concatenate([en - xin, e, en * en]), np.concatenate([xin, en, np.ones(n)]))
    assert _same(q[:n], (en - xin) / xin).all()
    assert _same(q[n:2 * n], e / en).all()
    assert _same(r[2 * n:], np.sqrt(en * en)).all()


def test_empty_and_bad_sizes():
    assert N.lib().pg_debug_ieee64(None, None, 0, None, None) == 0
    assert N.lib().pg_debug_ieee64(None, None, -1, None, None) == N.PG_EINVAL
    assert N.lib().pg_debug_ieee64(None, None, 5, None, None) == N.PG_EINVAL
