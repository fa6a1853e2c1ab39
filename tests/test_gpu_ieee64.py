"""The integer FP64 arithmetic of the kernels (pg_ieee64.cuh: division, square root, addition,
subtraction, multiplication, FP32 -> FP64 conversion), run on the GPU through pg_debug_ieee64,
returns the bits of numpy's IEEE results on random operands of every exponent, operands with
nearby exponents, significands at the edges of the reciprocal estimate's range, near-cancelling
differences, exact squares and their neighbours, and the operands of the bond loop."""
import ctypes as C

import numpy as np
import pytest

from perigrain_gb300 import _native as N

pytestmark = pytest.mark.gpu

DIV, SQRT, ADD, SUB, MUL, WIDEN = range(6)


def _run(op, a, b=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ones_like(a) if b is None else np.ascontiguousarray(b, dtype=np.float64)
    out = np.empty_like(a)
    p = lambda x: x.ctypes.data_as(C.c_void_p)
    N.check(N.lib().pg_debug_ieee64(op, p(a), p(b), a.size, p(out)))
    return out


def _check(got, want, *args):
    """Bitwise equality (NaNs of any payload equal), the first mismatches in the message."""
    ok = (got.view(np.uint64) == want.view(np.uint64)) | (np.isnan(got) & np.isnan(want))
    bad = np.flatnonzero(~ok)[:5]
    assert bad.size == 0, "%d mismatches, first: %s" % (
        (~ok).sum(), [(tuple(float(a[i]).hex() for a in args), got[i].hex(), want[i].hex()) for i in bad])


def _all_ops(a, b):
    with np.errstate(all="ignore"):
        _check(_run(DIV, a, b), a / b, a, b)
        _check(_run(SQRT, a), np.sqrt(np.abs(a)), a)
        _check(_run(ADD, a, b), a + b, a, b)
        _check(_run(SUB, a, b), a - b, a, b)
        _check(_run(MUL, a, b), a * b, a, b)
        _check(_run(WIDEN, a), a.astype(np.float32).astype(np.float64), a)


def _bits(sign, exp, frac):
    return ((np.asarray(sign).astype(np.uint64) << np.uint64(63)) | (np.asarray(exp).astype(np.uint64) << np.uint64(52))
            | np.asarray(frac).astype(np.uint64)).view(np.float64)


def test_random_operands_every_exponent():
    rng = np.random.default_rng(3)
    n = 1 << 22
    frac = lambda: rng.integers(0, 1 << 52, n, dtype=np.uint64)
    a = _bits(rng.integers(0, 2, n), rng.integers(0, 2048, n), frac())
    b = _bits(rng.integers(0, 2, n), rng.integers(0, 2048, n), frac())
    _all_ops(a, b)


def test_random_operands_near_each_other():
    rng = np.random.default_rng(4)
    n = 1 << 22
    frac = lambda: rng.integers(0, 1 << 52, n, dtype=np.uint64)
    ea = 1023 - 40 + rng.integers(0, 80, n)
    a = _bits(rng.integers(0, 2, n), ea, frac())
    b = _bits(rng.integers(0, 2, n), np.clip(ea + rng.integers(-66, 67, n), 1, 2046), frac())
    _all_ops(a, b)


def test_near_cancellation_and_tiny_results():
    rng = np.random.default_rng(7)
    n = 1 << 21
    a = _bits(rng.integers(0, 2, n), 1023 - 30 + rng.integers(0, 60, n), rng.integers(0, 1 << 52, n, dtype=np.uint64))
    near = (a.view(np.int64) + rng.integers(-4, 5, n)).view(np.float64)
    t = _bits(rng.integers(0, 2, n), 1 + rng.integers(0, 3, n), rng.integers(0, 1 << 52, n, dtype=np.uint64))
    tnear = (t.view(np.int64) + rng.integers(-512, 513, n)).view(np.float64)
    _all_ops(np.concatenate([a, a, t]), np.concatenate([near, -near, tnear]))


def test_edge_significands_and_specials():
    edge = np.array([0, 1, (1 << 52) - 1, (1 << 52) - 2, (1 << 29) - 1, 1 << 29, 1 << 51, (1 << 51) - 1,
                     0x5555555555555, 0xAAAAAAAAAAAAA], dtype=np.uint64)
    fa, fb, de = np.meshgrid(edge, edge, np.arange(-60, 61), indexing="ij")
    a = _bits(0, 1023 + de.ravel(), fa.ravel())
    b = _bits(0, np.full(fa.size, 1023), fb.ravel())
    sp = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1.0, -1.0, 5e-324, 2.2250738585072014e-308,
                   1.7976931348623157e308, 1e-310, -1e-310, 1e-45, 3.5e38])
    sa, sb = np.meshgrid(sp, sp, indexing="ij")
    _all_ops(np.concatenate([a, -a, sa.ravel()]), np.concatenate([b, b, sb.ravel()]))


def test_squares_and_neighbours():
    rng = np.random.default_rng(5)
    s = (1 << 25) + rng.integers(0, 1 << 25, 1 << 20, dtype=np.int64)
    sq = np.ldexp((s * s).astype(np.float64), rng.integers(-40, 40, s.size))
    x = rng.uniform(1.0, 2.0, 1 << 20)
    a = np.concatenate([sq, np.nextafter(sq, np.inf), np.nextafter(sq, 0), x * x, np.nextafter(x * x, np.inf)])
    _check(_run(SQRT, a), np.sqrt(a), a)


def test_bond_loop_operands():
    # squared bond lengths and stretches at the scale of mm-sized grains (lengths 1e-5..1e-3 m)
    rng = np.random.default_rng(6)
    n = 1 << 21
    xin = rng.uniform(1e-5, 1e-3, n)
    en = xin * (1 + rng.normal(0, 1e-3, n))
    e = en * rng.uniform(-1, 1, n)
    _check(_run(DIV, en - xin, xin), (en - xin) / xin)
    _check(_run(DIV, e, en), e / en)
    _check(_run(SQRT, en * en), np.sqrt(en * en))
    _check(_run(DIV, np.zeros(n), xin), np.zeros(n) / xin)


def test_empty_and_bad_arguments():
    assert N.lib().pg_debug_ieee64(DIV, None, None, 0, None) == 0
    assert N.lib().pg_debug_ieee64(DIV, None, None, -1, None) == N.PG_EINVAL
    assert N.lib().pg_debug_ieee64(DIV, None, None, 5, None) == N.PG_EINVAL
    assert N.lib().pg_debug_ieee64(6, None, None, 0, None) == N.PG_EINVAL
