"""Host-side parts of the gradient path (no GPU): the torch material map, the compaction setup
of the differentiable benchmark, and the C-ABI entry points' argument checks."""
import ctypes as C

import numpy as np
import pytest

from perigrain_gb300 import _native as N
from perigrain_gb300 import grad, setups


def test_bulk_to_cnot_matches_reference_material_formulas():
    torch = pytest.importorskip("torch")
    delta = np.array([1.5e-4, 2e-4])
    K = torch.tensor([setups.BULK, 3e9], dtype=torch.float64)
    c2 = grad.bulk_to_cnot(K, torch.tensor(delta), 2).numpy()
    for i in range(2):
        ref, _ = setups.peridem_2d(delta[i], K=float(K[i]))
        assert abs(c2[i] - ref) <= 1e-12 * ref
    c3 = grad.bulk_to_cnot(K, torch.tensor(delta), 3).numpy()
    for i in range(2):
        ref, _ = setups.peridem_3d(delta[i], K=float(K[i]))
        assert abs(c3[i] - ref) <= 1e-12 * ref


def test_bulk_to_cnot_is_differentiable():
    torch = pytest.importorskip("torch")
    K = torch.tensor([2e9], dtype=torch.float64, requires_grad=True)
    c = grad.bulk_to_cnot(K, torch.tensor([1.5e-4], dtype=torch.float64), 2)
    c.sum().backward()
    h = 1e-3 * 2e9
    num = (setups.peridem_2d(1.5e-4, K=2e9 + h)[0] - setups.peridem_2d(1.5e-4, K=2e9 - h)[0]) / (2 * h)
    assert abs(float(K.grad[0]) - num) <= 1e-6 * abs(num)


def test_compaction_setup_touches_walls_and_neighbours():
    s = setups.compaction_2d(n_grains=10, nodes_per_grain=100)
    p = s.pos.reshape(-1, 2)
    rc = float(s.contact_radius[0])
    wall = np.asarray(s.wall_geom, np.float64).reshape(-1)
    # outermost nodes sit within the contact radius of the walls they face
    assert p[:, 0].min() - wall[0] <= rc and wall[1] - p[:, 0].max() <= rc
    assert wall[2] - p[:, 1].max() <= rc and p[:, 1].min() - wall[3] <= rc
    # the top wall moves down at 1 m/s
    assert np.asarray(s.wall_speed).reshape(-1)[2] == -1.0
    assert s.n_grains == 10


def test_grad_entry_points_reject_null_handles():
    L = N.lib()
    assert L.pg_grad_begin(None) == N.PG_EINVAL
    assert L.pg_grad_reset(None) == N.PG_EINVAL
    assert L.pg_grad_forward(None, 10, 5, None) == N.PG_EINVAL
    g = np.zeros(4)
    assert L.pg_grad_backward(None, None, None, None, N.ptr(g, C.c_double)) == N.PG_EINVAL
    m = C.c_void_p()
    assert L.pg_masks_record(None, 10, C.byref(m)) == N.PG_EINVAL
    assert L.pg_set_grain_params(None, None, None, None, None, None) == N.PG_EINVAL
    L.pg_masks_free(None)
