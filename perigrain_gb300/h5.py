"""Read/write HDF5 files through the project's HDF5-subset library (no h5py needed)."""
import ctypes as C

import numpy as np

from . import _native as N

_DT = {np.dtype(np.float64): 0, np.dtype(np.float32): 1, np.dtype(np.uint32): 2, np.dtype(np.int32): 3,
       np.dtype(np.uint64): 4, np.dtype(np.int64): 5, np.dtype(np.uint8): 6}


def info(filename, path):
    L = N.lib()
    rank = C.c_uint32()
    dims = (C.c_uint64 * 8)()
    cls, size, sgn = C.c_int32(), C.c_uint32(), C.c_int32()
    rc = L.pg_h5_info(str(filename).encode(), path.encode(), C.byref(rank), dims, C.byref(cls), C.byref(size),
                      C.byref(sgn))
    if rc:
        raise KeyError("%s: %s: %s" % (filename, path, L.pg_last_error().decode(errors="replace")))
    return tuple(dims[i] for i in range(rank.value)), cls.value, size.value, bool(sgn.value)


def read(filename, path, dtype=None):
    """Read a dataset; dtype defaults to the stored type (f64 / i64 / u64 / ...)."""
    shape, cls, size, sgn = info(filename, path)
    if dtype is None:
        dtype = {(1, 8): np.float64, (1, 4): np.float32, (0, 8): np.int64 if sgn else np.uint64,
                 (0, 4): np.int32 if sgn else np.uint32}.get((cls, size), np.float64)
    dtype = np.dtype(dtype)
    out = np.empty(int(np.prod(shape)) if shape else 1, dtype)
    buf = out if out.size else np.empty(1, dtype)
    rc = N.lib().pg_h5_read(str(filename).encode(), path.encode(), _DT[dtype], buf.ctypes.data_as(C.c_void_p),
                            buf.size)
    if rc:
        raise KeyError("%s: %s" % (filename, path))
    return out.reshape(shape)


def list_group(filename, path=""):
    buf = C.create_string_buffer(1 << 20)
    rc = N.lib().pg_h5_list(str(filename).encode(), path.encode(), buf, len(buf))
    if rc:
        raise KeyError("%s: %s" % (filename, path))
    return [x for x in buf.value.decode().split("\n") if x]


def write(filename, datasets, groups=()):
    """datasets: {path: ndarray}. Writes an HDF5 file with those datasets."""
    L = N.lib()
    w = L.pg_h5w_new()
    try:
        for g in groups:
            N.check(L.pg_h5w_group(w, g.encode()))
        for path, a in datasets.items():
            a = np.ascontiguousarray(a)
            dims = (C.c_uint64 * max(1, a.ndim))(*a.shape)
            buf = a if a.size else np.empty(1, a.dtype)
            rc = L.pg_h5w_add(w, path.encode(), _DT[a.dtype], a.ndim, dims, buf.ctypes.data_as(C.c_void_p))
            if rc:
                raise ValueError("cannot add dataset %s" % path)
        N.check(L.pg_h5w_write(w, str(filename).encode()))
    finally:
        L.pg_h5w_free(w)
