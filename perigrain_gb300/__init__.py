"""perigrain_gb300: GB300-native (sm_103a) PeriDEM time integration.

A drop-in for the time-integration hot path of debdeepbh/perigrain: peridynamic bond forces
with bond breaking, node-node and analytic-wall contact with damping and friction, and the
velocity-Verlet update, as hand-written CUDA kernels behind a C ABI (include/perigrain.h).
"""
from . import _native
from .engine import Simulation, Snapshot, device_count, pinned_empty, run_simulation
from . import setups

__all__ = ["Simulation", "Snapshot", "pinned_empty", "run_simulation", "device_count", "setups", "_native"]
