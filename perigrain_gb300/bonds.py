"""GPU bond-list builder (pg_build_bonds in include/perigrain.h).

build_bonds(pos, delta) returns the lexicographic (i < j) Connectivity of one grain: every node
pair with sqrt(sum((p_j - p_i)**2)) <= delta -- the rule of the reference's setup
(exp_dict.py:171-222), evaluated with the same FP64 arithmetic. Device buffers come from torch.
"""
import ctypes as C

import numpy as np

from . import _native as N


def build_bonds(pos, delta, capacity=None, entry="pg_build_bonds"):
    import torch

    pos = np.ascontiguousarray(pos, np.float64)
    n, dim = pos.shape
    d_pos = torch.from_numpy(pos).cuda()
    if capacity is None:
        capacity = max(16, n * (64 if dim == 2 else 256))
    d_pairs = torch.empty((capacity, 2), dtype=torch.int32, device="cuda")
    npairs = C.c_uint64()
    torch.cuda.synchronize()
    fn = getattr(N.lib(), entry)
    rc = fn(C.c_void_p(d_pos.data_ptr()), n, dim, float(delta), C.c_void_p(d_pairs.data_ptr()), capacity,
            C.byref(npairs), None)
    if rc != N.PG_OK:
        raise N.PerigrainError(rc, N.lib().pg_bond_last_error().decode())
    m = npairs.value
    return d_pairs[:m].cpu().numpy().astype(np.int64)
