"""The reference's collision dynamics amplify tiny perturbations (measured with the FP64
oracle, which is bit-identical to the reference): this bounds what any implementation that does
not reproduce the reference's arithmetic bit for bit -- e.g. FP32 forces, or the reference built
with FMA contraction -- can match pointwise."""
import numpy as np

import _oracle as O
from perigrain_gb300 import setups


def test_one_ulp_scale_perturbation_grows_through_contact():
    s = setups.two_disk_collision()
    s2 = s.copy()
    v = s2.vel.reshape(-1, 2)
    v[100, 0] *= 1 + 1e-12
    s2.vel = v.reshape(-1)
    a, b = O.OracleSim(s, dt=2e-8, enable_fracture=1), O.OracleSim(s2, dt=2e-8, enable_fracture=1)
    a.step(100)
    b.step(100)
    x, y = a.field("CurrPos"), b.field("CurrPos")
    before = np.abs(x - y).max() / np.abs(x).max()
    a.step(250)
    b.step(250)
    x, y = a.field("CurrPos"), b.field("CurrPos")
    after = np.abs(x - y).max() / np.abs(x).max()
    assert before < 1e-14
    assert after > 1e-5  # amplified by > 1e9 within 250 steps of contact
