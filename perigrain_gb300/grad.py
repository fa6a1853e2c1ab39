"""Gradients of PeriDEM objectives with respect to per-grain parameters.

The reference has no gradient path. This module differentiates its time step
(``src/particle/timeloop.h:608-879``) through the engine's hand-written adjoint kernels
(``csrc/pg_adjoint.cu``), reached over the C ABI (``pg_grad_*`` in ``include/perigrain.h``):

* parameters per grain: ``cnot`` (bond stiffness, ``particle2.h:140``; it also sets the
  self-contact stiffness ``cnot/R_c'``, ``contact.h:709-730``), normal contact stiffness ``kn``,
  damping ratio ``zeta`` and friction coefficient ``mu``; two grains in contact use the mean of
  their values (with equal values this is the reference's global ``Contact``);
* objectives: the wall reactions of the last step (``RectWall::reaction``, ``contact.h:339``) and
  the kinetic energy ``sum 1/2 rho vol |v|^2`` per instance (mass convention of
  ``read_sim_output.py:311``);
* bond breaks, contact pairs, friction branches and wall contacts are frozen as the forward pass
  decided them; memory is one checkpoint every ``checkpoint_every`` steps plus one segment of tape.

``objectives(cnot, kn, zeta, mu, run)`` is a ``torch.autograd.Function``; ``bulk_to_cnot`` maps a
per-grain bulk modulus to ``cnot`` with the reference's material formulas in torch, so gradients
with respect to bulk moduli follow by autograd.
"""
import ctypes as C
import math

import numpy as np

from . import _native as N

PARAMS = ("cnot", "kn", "zeta", "mu")


class Masks:
    """Masks of a recorded run (``pg_masks``); frees the device memory on close."""

    def __init__(self, handle, n_steps):
        self.h = handle
        self.n_steps = n_steps

    def close(self):
        if getattr(self, "h", None):
            N.lib().pg_masks_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _vec(a, n):
    if a is None:
        return None
    a = np.ascontiguousarray(np.broadcast_to(np.asarray(a, np.float64), (n,)))
    return a


class GradRun:
    """A differentiable run of ``n_steps`` steps of a :class:`~perigrain_gb300.engine.Simulation`
    from its current state (the origin)."""

    def __init__(self, sim, n_steps, checkpoint_every=100):
        self.sim = sim
        self.n_steps = int(n_steps)
        self.checkpoint_every = int(checkpoint_every)
        s = sim.setup
        self.G = s.n_grains
        self.I = s.n_instances
        self.dim = s.dim
        N.check(N.lib().pg_grad_begin(sim.h))
        off = np.asarray(s.grain_node_offset, np.int64)
        counts = np.diff(off)
        self.node_grain = np.repeat(np.arange(self.G), counts)
        self.node_inst = np.asarray(s.grain_instance, np.int64)[self.node_grain]
        self.node_mass = np.asarray(s.rho, np.float64)[self.node_grain] * np.asarray(s.vol, np.float64)

    def params(self):
        out = {k: np.empty(self.G) for k in ("cnot", "snot", "kn", "zeta", "mu")}
        p = [N.ptr(out[k], C.c_double) for k in ("cnot", "snot", "kn", "zeta", "mu")]
        N.check(N.lib().pg_get_grain_params(self.sim.h, *p))
        return out

    def set_params(self, cnot=None, snot=None, kn=None, zeta=None, mu=None):
        args = []
        keep = []
        for a in (cnot, snot, kn, zeta, mu):
            v = _vec(a, self.G)
            keep.append(v)
            args.append(N.ptr(v, C.c_double) if v is not None else None)
        N.check(N.lib().pg_set_grain_params(self.sim.h, *args))

    def reset(self):
        N.check(N.lib().pg_grad_reset(self.sim.h))

    def record_masks(self, n_steps=None):
        """Run from the origin recording every step's masks (for frozen FP64 replays)."""
        n = int(n_steps or self.n_steps)
        m = C.c_void_p()
        N.check(N.lib().pg_masks_record(self.sim.h, n, C.byref(m)))
        return Masks(m, n)

    def kinetic_energy(self, vel=None):
        v = self.sim.field("vel") if vel is None else vel
        e = 0.5 * self.node_mass * (v * v).sum(1)
        return np.bincount(self.node_inst, weights=e, minlength=self.I)

    def forward(self, frozen=None):
        """Run from the origin; returns (reactions [I, 2*dim, dim] of the last step, kinetic
        energy [I] at the end)."""
        fh = frozen.h if frozen is not None else None
        N.check(N.lib().pg_grad_forward(self.sim.h, self.n_steps, self.checkpoint_every, fh))
        self._vel = self.sim.field("vel")
        return self.sim.reaction(), self.kinetic_energy(self._vel)

    def backward(self, reaction_bar=None, ke_bar=None, vel_bar=None, disp_bar=None):
        """Gradient [G, 4] (cnot, kn, zeta, mu) of
        sum(reaction_bar * reaction) + sum(ke_bar * ke) + sum(vel_bar * vel) + sum(disp_bar * disp)
        at the end of the last forward."""
        n, d = self.sim.setup.n_nodes, self.dim
        vb = np.zeros((n, d)) if vel_bar is None else np.array(vel_bar, np.float64).reshape(n, d)
        if ke_bar is not None:
            kb = np.broadcast_to(np.asarray(ke_bar, np.float64), (self.I,))
            vb = vb + (kb[self.node_inst] * self.node_mass)[:, None] * self._vel
        vb = np.ascontiguousarray(vb)
        db = None if disp_bar is None else np.ascontiguousarray(np.asarray(disp_bar, np.float64).reshape(n, d))
        rb = None
        if reaction_bar is not None:
            rb = np.ascontiguousarray(np.broadcast_to(np.asarray(reaction_bar, np.float64),
                                                      (self.I, 2 * d, d)))
        g = np.empty((self.G, 4), np.float64)
        N.check(N.lib().pg_grad_backward(self.sim.h, N.ptr(db, C.c_double) if db is not None else None,
                                         N.ptr(vb, C.c_double), N.ptr(rb, C.c_double) if rb is not None else None,
                                         N.ptr(g, C.c_double)))
        return g

    def times(self):
        f, b = C.c_double(), C.c_double()
        nf, nb = C.c_uint64(), C.c_uint64()
        N.check(N.lib().pg_grad_times(self.sim.h, C.byref(f), C.byref(b), C.byref(nf), C.byref(nb)))
        return dict(forward_ms=f.value, backward_ms=b.value, forward_launches=nf.value, backward_launches=nb.value)


# ---------------------------------------------------------------------------------------------
# torch
# ---------------------------------------------------------------------------------------------
def _torch():
    import torch

    return torch


def _make_function():
    torch = _torch()

    class PeriDEMObjectives(torch.autograd.Function):
        """(cnot, kn, zeta, mu) [G] -> (wall reactions of the last step [I, 2*dim, dim],
        kinetic energy at the end [I]); backward = the engine's adjoint."""

        @staticmethod
        def forward(ctx, cnot, kn, zeta, mu, run, frozen):
            run.set_params(cnot=cnot.detach().cpu().numpy(), kn=kn.detach().cpu().numpy(),
                           zeta=zeta.detach().cpu().numpy(), mu=mu.detach().cpu().numpy())
            r, ke = run.forward(frozen)
            ctx.run = run
            ctx.frozen = frozen
            return torch.from_numpy(r), torch.from_numpy(ke)

        @staticmethod
        def backward(ctx, g_r, g_ke):
            rb = None if g_r is None else g_r.detach().cpu().numpy()
            kb = None if g_ke is None else g_ke.detach().cpu().numpy()
            g = torch.from_numpy(ctx.run.backward(reaction_bar=rb, ke_bar=kb))
            return g[:, 0], g[:, 1], g[:, 2], g[:, 3], None, None

    return PeriDEMObjectives


_FN = None


def objectives(cnot, kn, zeta, mu, run, frozen=None):
    """Differentiable (reactions, kinetic energy) of ``run`` as functions of the per-grain
    parameter tensors (float64, shape [G])."""
    global _FN
    if _FN is None:
        _FN = _make_function()
    return _FN.apply(cnot, kn, zeta, mu, run, frozen)


def bulk_to_cnot(K, delta, dim, shear=1.33e9):
    """Bond constant from a per-grain bulk modulus (torch, differentiable): 2D ``peridem``
    (material_dict.py:61-82) with the shear modulus held, 3D ``peridem_3d``
    (material_dict.py:186-197)."""
    torch = _torch()
    delta = torch.as_tensor(delta, dtype=K.dtype)
    if dim == 3:
        return 18 * K / (math.pi * delta ** 4)
    G = shear
    nu = (3 * K - 2 * G) / (2 * (3 * K + G))
    E = 9 * K * G / (9 * K + G)
    return 24 * E / ((1 - nu) * math.pi * delta ** 3)
