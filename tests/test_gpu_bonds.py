"""GPU bond-list builder vs the reference's rule (exp_dict.py:171-222), evaluated with numpy."""
import numpy as np
import pytest

from perigrain_gb300 import setups
from perigrain_gb300.bonds import build_bonds

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape,dim,jitter", [("disk", 2, 0.0), ("ngon", 2, 0.1), ("plus", 2, 0.1),
                                              ("sphere", 3, 0.1), ("sphere", 3, 0.0)])
def test_matches_reference_rule(shape, dim, jitter):
    rng = np.random.default_rng(5)
    h = 5e-5
    p, _ = setups.grid_nodes(shape, 25 * h if dim == 2 else 8 * h, h, dim=dim, jitter=jitter, rng=rng, angle=0.3)
    p = p + 1e-3
    delta = 3 * h  # uniform grids put many pairs at exactly delta: both sides must agree on them
    got = build_bonds(p, delta)
    ref = setups.bond_pairs(p, delta)
    assert got.shape == ref.shape and np.array_equal(got, ref), (got.shape, ref.shape)


def test_empty_and_tiny():
    assert build_bonds(np.zeros((1, 2)), 1.0).shape == (0, 2)
    got = build_bonds(np.array([[0.0, 0.0], [1.0, 0.0], [3.0, 0.0]]), 2.0)
    assert got.tolist() == [[0, 1], [1, 2]]


def test_capacity_error():
    from perigrain_gb300 import _native as N

    p, _ = setups.grid_nodes("disk", 1e-3, 5e-5, dim=2)
    with pytest.raises(N.PerigrainError):
        build_bonds(p, 1.5e-4, capacity=10)
