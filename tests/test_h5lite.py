"""The project's HDF5-subset reader/writer: round trips, layout of the files it writes, type
conversion on read (the reference reads h5py's int64 as NATIVE_UINT/NATIVE_INT)."""
import os

import numpy as np
import pytest

from perigrain_gb300 import h5


def test_roundtrip_types_and_shapes(tmp_path):
    fn = tmp_path / "a.h5"
    rng = np.random.default_rng(0)
    data = {
        "f64": rng.standard_normal((7, 3)),
        "f32": rng.standard_normal(5).astype(np.float32),
        "u32": rng.integers(0, 2**32 - 1, (4, 2), dtype=np.uint32),
        "i32": rng.integers(-2**31, 2**31 - 1, 9, dtype=np.int32),
        "i64": rng.integers(-2**62, 2**62, (3, 1), dtype=np.int64),
        "g1/g2/deep": np.arange(12, dtype=np.float64).reshape(3, 4),
        "empty": np.zeros((0, 2), np.uint32),
        "scalarlike": np.array([[3.5]]),
    }
    h5.write(fn, data)
    with open(fn, "rb") as f:
        assert f.read(8) == b"\x89HDF\r\n\x1a\n"
    for k, v in data.items():
        r = h5.read(fn, k)
        assert r.dtype == v.dtype and r.shape == v.shape and np.array_equal(r, v), k
    assert sorted(h5.list_group(fn)) == sorted(["f64", "f32", "u32", "i32", "i64", "g1", "empty", "scalarlike"])
    assert h5.list_group(fn, "g1") == ["g2"]


def test_many_members_multilevel_btree(tmp_path):
    """Groups with more members than one symbol-table node / B-tree node holds."""
    fn = tmp_path / "many.h5"
    data = {"P_%05d/x" % i: np.array([[float(i)]]) for i in range(1500)}
    data.update({"flat_%04d" % i: np.array([i], np.int64) for i in range(700)})
    h5.write(fn, data)
    names = h5.list_group(fn)
    assert len(names) == 2200 and names == sorted(names)
    for i in (0, 1, 7, 8, 255, 256, 257, 1023, 1499):
        assert h5.read(fn, "P_%05d/x" % i)[0, 0] == float(i)
    for i in (0, 699):
        assert h5.read(fn, "flat_%04d" % i)[0] == i


def test_conversion_on_read(tmp_path):
    fn = tmp_path / "c.h5"
    h5.write(fn, {"i64": np.array([-5, 0, 7, 2**40], np.int64), "f": np.array([1.9, -2.9, 1e20])})
    assert h5.read(fn, "i64", np.uint32).tolist() == [0, 0, 7, 2**32 - 1]  # clamped like libhdf5
    assert h5.read(fn, "i64", np.float64).tolist() == [-5.0, 0.0, 7.0, float(2**40)]
    assert h5.read(fn, "f", np.int32).tolist() == [1, -2, 2**31 - 1]


def test_missing_and_corrupt(tmp_path):
    fn = tmp_path / "m.h5"
    h5.write(fn, {"a": np.zeros(3)})
    with pytest.raises(KeyError):
        h5.read(fn, "b")
    bad = tmp_path / "bad.h5"
    bad.write_bytes(b"not an hdf5 file at all" * 10)
    with pytest.raises(KeyError):
        h5.read(bad, "a")
    trunc = tmp_path / "t.h5"
    trunc.write_bytes(open(fn, "rb").read()[:150])
    with pytest.raises(KeyError):
        h5.read(trunc, "a")
