"""Gradient path: frozen-mask FP64 replay, hand-written adjoint, checkpoint recomputation.

Checks, each on small seeded compaction runs (walls, contact, damping, friction, fracture on):
* the FP64 replay under the masks the FP64 engine recorded reproduces that engine bit for bit;
* the product backward (engine recompute from checkpoints) equals, bit for bit, the backward
  through the replay of the same masks, and repeats bit for bit;
* the adjoint gradient equals central finite differences of the frozen-mask FP64 map, every
  parameter of every grain: at h = 1e-4 relative to FD_TOL of the largest sensitivity
  theta*dJ/dtheta, and at h = 1e-7 (where FD has converged) to FD_TOL_FINE. The h = 1e-4 bound is
  looser because the reference's wall damping, 2 zeta sqrt(K_n rho) sqrt(Area) (contact.h:417-429),
  has a derivative that grows without bound as a node reaches the edge of the wall-contact zone
  (Area ~ (R - d)^(3/2)), so a 1e-4 difference quotient is not yet converged for such nodes;
* the gradient along the mixed-precision trajectory (FP32 bond products in the reverse step)
  agrees with the FP64 reference gradient (FP64 replay of the same masks, FP64 reverse step) to
  MIXED_TOL over 200 steps. The two gradients are taken along two trajectories that differ by the
  mixed-precision rounding, and the frozen-mask compaction map amplifies that difference (the
  velocity gap grows ~10x per 100 steps here), so the bound is stated at a horizon where the
  trajectories still agree to ~1e-5; the gap tracks the trajectory gap, not the reverse step;
* the torch.autograd.Function gives d(objective)/d(bulk modulus) by the chain rule;
* on the full differentiable compaction (50 grains, 200 parameters) the mixed gradient, the FP64
  reference gradient and central differences agree through its stated horizon (HORIZON below)."""
import numpy as np
import pytest

from perigrain_gb300 import Simulation, grad, setups

pytestmark = pytest.mark.gpu
H = 1e-4
FD_TOL = 5e-4
H_FINE = 1e-7
FD_TOL_FINE = 1e-6
MIXED_TOL = 1e-4


def _case(n_grains=6, nodes=120, r=0.3e-3, seed=11):
    return setups.compaction_2d(n_grains=n_grains, r=r, nodes_per_grain=nodes, seed=seed)


def _sim(s, precision="fp64", contact_skin=0.0):
    return Simulation(s, dt=2e-8, enable_fracture=1, allow_damping=1, allow_friction=1, self_contact=1,
                      precision=precision, contact_skin=contact_skin)


def _weights(run, frozen, rng):
    r0, ke0 = run.forward(frozen)
    wr = rng.uniform(-1, 1, r0.shape) / max(np.abs(r0).max(), 1e-30)
    wk = np.full(ke0.shape, 1.0 / max(ke0.max(), 1e-30))
    return wr, wk


def _J(run, frozen, wr, wk):
    r, ke = run.forward(frozen)
    return float((wr * r).sum() + (wk * ke).sum())


def _sens(run, frozen, wr, wk, theta, h=H):
    """theta * dJ/dtheta by central differences of the frozen map, every parameter."""
    base = {k: theta[k].copy() for k in grad.PARAMS}
    out = np.zeros((run.G, 4))
    for a, k in enumerate(grad.PARAMS):
        for g in range(run.G):
            vals = []
            for sgn in (1, -1):
                p = {kk: base[kk].copy() for kk in grad.PARAMS}
                p[k][g] *= 1 + sgn * h
                run.set_params(**p)
                vals.append(_J(run, frozen, wr, wk))
            out[g, a] = (vals[0] - vals[1]) / (2 * h)
    run.set_params(**base)
    return out


def test_replay_reproduces_fp64_engine():
    s = _case()
    sim = _sim(s)
    run = grad.GradRun(sim, 400, checkpoint_every=64)
    m = run.record_masks()
    x_e, v_e = sim.field("CurrPos"), sim.field("vel")
    assert run.kinetic_energy().sum() > 0
    r_e = sim.reaction()
    run.forward(m)
    assert np.array_equal(sim.field("CurrPos"), x_e)
    assert np.array_equal(sim.field("vel"), v_e)
    np.testing.assert_allclose(sim.reaction(), r_e, rtol=1e-12, atol=1e-12 * np.abs(r_e).max())
    m.close()


@pytest.mark.parametrize("skin", [0.0, 0.5])
def test_product_backward_equals_replay_backward_and_repeats(skin):
    s = _case(seed=12)
    sim = _sim(s, contact_skin=skin)
    run = grad.GradRun(sim, 300, checkpoint_every=40)
    m = run.record_masks()
    rng = np.random.default_rng(0)
    wr, wk = _weights(run, None, rng)
    run.forward(None)
    g1 = run.backward(reaction_bar=wr, ke_bar=wk)
    run.forward(None)
    g2 = run.backward(reaction_bar=wr, ke_bar=wk)
    assert np.array_equal(g1, g2)
    run.forward(m)
    g3 = run.backward(reaction_bar=wr, ke_bar=wk)
    assert np.array_equal(g1, g3)
    assert np.abs(g1).max() > 0
    # backward leaves the handle at the final state of the forward
    v = sim.field("vel")
    run.forward(m)
    assert np.array_equal(sim.field("vel"), v)
    m.close()


@pytest.mark.parametrize("seed", [13, 14])
def test_adjoint_matches_central_differences(seed):
    s = _case(seed=seed)
    sim = _sim(s)
    run = grad.GradRun(sim, 500, checkpoint_every=64)
    m = run.record_masks()
    rng = np.random.default_rng(seed)
    wr, wk = _weights(run, m, rng)
    theta = run.params()
    run.forward(m)
    g = run.backward(reaction_bar=wr, ke_bar=wk)
    sens_adj = g * np.stack([theta[k] for k in grad.PARAMS], 1)
    sens_fd = _sens(run, m, wr, wk, theta)
    scale = np.abs(sens_fd).max()
    assert scale > 0
    err = np.abs(sens_adj - sens_fd).max() / scale
    assert err <= FD_TOL, (err, sens_adj, sens_fd)
    fine = _sens(run, m, wr, wk, theta, h=H_FINE)
    err_fine = np.abs(sens_adj - fine).max() / scale
    assert err_fine <= FD_TOL_FINE, (err_fine, sens_adj, fine)
    # every parameter kind is exercised
    for a in range(4):
        assert np.abs(sens_fd[:, a]).max() > 1e-6 * scale
    m.close()


def test_mixed_gradient_matches_fp64_reference():
    s = _case(seed=15)
    sim = _sim(s, precision="mixed")
    run = grad.GradRun(sim, 200, checkpoint_every=64)
    m = run.record_masks()
    rng = np.random.default_rng(1)
    wr, wk = _weights(run, None, rng)
    theta = run.params()
    tv = np.stack([theta[k] for k in grad.PARAMS], 1)
    run.forward(None)
    g_mx = run.backward(reaction_bar=wr, ke_bar=wk) * tv
    run.forward(m)
    g_ref = run.backward(reaction_bar=wr, ke_bar=wk) * tv
    err = np.abs(g_mx - g_ref).max() / np.abs(g_ref).max()
    assert err <= MIXED_TOL, err
    m.close()


def test_torch_function_bulk_modulus_chain_rule():
    torch = pytest.importorskip("torch")
    s = _case(seed=16)
    sim = _sim(s)
    run = grad.GradRun(sim, 300, checkpoint_every=50)
    m = run.record_masks()
    theta = run.params()
    delta = torch.tensor(np.asarray(s.delta, np.float64))
    K = torch.full((run.G,), setups.BULK, dtype=torch.float64, requires_grad=True)
    cnot = grad.bulk_to_cnot(K, delta, 2)
    np.testing.assert_allclose(cnot.detach().numpy(), theta["cnot"], rtol=1e-12)
    kn = torch.tensor(theta["kn"], requires_grad=True)
    zeta = torch.tensor(theta["zeta"], requires_grad=True)
    mu = torch.tensor(theta["mu"], requires_grad=True)
    r, ke = grad.objectives(cnot, kn, zeta, mu, run, m)
    r0, ke0 = abs(float(r[0, 2, 1].detach())), float(ke.sum().detach())
    loss = r[0, 2, 1] / max(r0, 1e-30) + ke.sum() / ke0
    loss.backward()
    # finite difference in K of grain 0 through the same frozen map
    def J(k0):
        Kp = K.detach().clone()
        Kp[0] = k0
        c = grad.bulk_to_cnot(Kp, delta, 2).numpy()
        run.set_params(cnot=c)
        rr, kk = run.forward(m)
        return rr[0, 2, 1] / max(r0, 1e-30) + kk.sum() / ke0
    k0 = setups.BULK
    fd = (J(k0 * (1 + H)) - J(k0 * (1 - H))) / (2 * H * k0)
    assert abs(float(K.grad[0]) - fd) <= FD_TOL * max(abs(fd), float(K.grad.abs().max())), (float(K.grad[0]), fd)
    assert kn.grad is not None and zeta.grad is not None and mu.grad is not None
    m.close()


def test_grad_rejects_torque_and_unstoppable():
    s = _case(seed=17)
    s.stoppable[0] = 0
    sim = _sim(s)
    with pytest.raises(Exception):
        grad.GradRun(sim, 10)


def test_mixed_backward_with_overlapped_recording_equals_serial():
    """With candidate lists the mixed engine runs each step's finalize beside the next position
    update, also in the recording replays of the backward; without lists it runs them in order.
    Lists do not change results, so the two gradients are identical."""
    s = _case(seed=15)
    gs = []
    for skin in (0.0, 0.5):
        sim = _sim(s, precision="mixed", contact_skin=skin)
        run = grad.GradRun(sim, 240, checkpoint_every=40)
        rng = np.random.default_rng(3)
        wr, wk = _weights(run, None, rng)
        run.forward(None)
        gs.append(run.backward(reaction_bar=wr, ke_bar=wk))
        sim.close()
    assert np.abs(gs[0]).max() > 0
    assert np.array_equal(gs[0], gs[1])


# The differentiable compaction at full size (50 grains, 18,930 nodes, 200 parameters): the checks
# hold through HORIZON steps of its 5000-step run (measured by bench.py's adjoint section at 200,
# 500, 1000, 2000 and 5000 steps: gap 4.8e-5, differences 6.9e-5 / 3.6e-8 at 2000 steps; at 5000 the
# chaotic dynamics separate the mixed and FP64 trajectories and their gradients).
HORIZON = 2000
HORIZON_TOL = 1e-3


def test_full_compaction_gradient_at_its_horizon():
    spec = setups.WORKLOADS[4]
    s = setups.workload(4)
    assert s.n_grains == 50
    sim = Simulation(s, dt=spec["dt"], precision="mixed")
    run = grad.GradRun(sim, HORIZON, checkpoint_every=100)
    r0, ke0 = run.forward()
    wr = np.zeros_like(r0)
    wr[0, 2, 1] = 1.0 / abs(float(r0[0, 2, 1]))  # top-wall reaction (y), normalised
    wk = 1.0 / ke0
    g = run.backward(reaction_bar=wr, ke_bar=wk)
    theta = run.params()
    tv = np.stack([theta[k] for k in grad.PARAMS], 1)
    sens = g * tv
    m = run.record_masks()
    run.forward(m)
    ref = run.backward(reaction_bar=wr, ke_bar=wk) * tv
    scale = np.abs(ref).max()
    assert scale > 0
    # mixed-precision gradient vs the FP64 reference gradient, every parameter of every grain
    assert np.abs(sens - ref).max() <= HORIZON_TOL * scale
    # central differences of the frozen FP64 map for the four largest sensitivities
    for h in (1e-4, 1e-6):
        for fi in np.argsort(-np.abs(ref).ravel())[:4]:
            gi, a = divmod(int(fi), 4)
            vals = []
            for sg in (1, -1):
                p = {k: theta[k].copy() for k in grad.PARAMS}
                p[grad.PARAMS[a]][gi] *= 1 + sg * h
                run.set_params(**p)
                rr, kk = run.forward(m)
                vals.append(float((wr * rr).sum() + (wk * kk).sum()))
            run.set_params(**{k: theta[k] for k in grad.PARAMS})
            fd = (vals[0] - vals[1]) / (2 * h)
            assert abs(fd - ref[gi, a]) <= HORIZON_TOL * scale, (h, gi, a, fd, ref[gi, a])
    m.close()
    sim.close()
