"""Adjoint of batched BDF1 rollouts on the GPU (sdfc_sim_record / sdfc_sim_backward)
against the reference's backward pass, the oracle's restatement of it, and central
finite differences.

tests/golden/sim_trans.npz holds the reference's dL/dq0 and dL/dqdot0 for
L = sum_k w_k . q_k over 20 steps.  Bars (relative to the gradient's norm):
  * FP64 evaluations, FD-stencil derivatives (the reference's own Hessian): 1e-9;
  * FP64 evaluations, analytic derivatives: 1e-6 (the reference's FD Hessian
    diagonal carries ~1e-7 relative round-off that the analytic one does not);
  * mixed-precision evaluations: 1e-4;
  * finite differences (step 1e-6, Newton tolerance 1e-8): 1e-4."""
import numpy as np
import pytest

from _helpers import load
from conftest import submodule
from test_gpu_sim import make_sim

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sdfc():
    submodule("build").build()
    return submodule("sdfc")


def nrel(got, want):
    return np.linalg.norm(np.asarray(got) - np.asarray(want)) / np.linalg.norm(want)


@pytest.mark.parametrize("precision,deriv,bar", [(0, 1, 1e-9), (0, 0, 1e-6), (1, 0, 1e-4)])
def test_reference_backward(sdfc, precision, deriv, bar):
    fx = load("sim_trans.npz")
    T = int(fx["bw_steps"])
    ctx = sdfc.Context(0)
    try:
        ctx.set_derivative_mode(deriv)
        sim = make_sim(sdfc, ctx, fx, precision=precision)
        sim.record(T)
        assert sim.step(T).all()
        qh = sim.history()
        assert qh.shape == (1, T + 1, 3)
        np.testing.assert_allclose(qh[0], fx["q"][: T + 1], rtol=0, atol=1e-9 if precision == 0 else 1e-6)
        g0, gd0, gf = sim.backward(fx["bw_df_dq"][None])
        assert nrel(g0[0], fx["bw_df_dq0"]) <= bar
        assert nrel(gd0[0], fx["bw_df_dqdot0"]) <= bar
        assert np.all(gf[0, :3] == 0.0)
    finally:
        ctx.close()


def test_batch_against_oracle(sdfc, oracle):
    """12 differently pushed scenes: each scene's gradients against the oracle's
    backward on the oracle's own trajectory."""
    fx = load("sim_trans.npz")
    from test_oracle_sim import scene
    rng = np.random.default_rng(11)
    n, T = 12, 10
    F = np.zeros((n, 6))
    F[:, 3:] = rng.normal(size=(n, 3)) * 3.0
    q0 = np.tile(fx["q0"], (n, 1)) + rng.normal(size=(n, 3)) * [0.004, 0.004, 0.05]
    qd0 = rng.normal(size=(n, 3)) * 0.3
    w = rng.normal(size=(n, T, 3))
    ctx = sdfc.Context(0)
    try:
        sim = make_sim(sdfc, ctx, fx, n=n, f_ext=F, q0=q0, qd0=qd0)
        sim.record(T)
        sim.step(T)
        qh = sim.history()
        g0, gd0, gf = sim.backward(w)
    finally:
        ctx.close()
    mover, pairs = scene(oracle, fx)
    contact = 0
    for i in range(n):
        m = oracle.Mover(mover.mass, mover.inertia, mover.E_ji, mover.E_pj0, mover.gravity, mover.h, F[i])
        qs, _, _, its, _ = oracle.bdf1_steps(m, pairs, q0[i], qd0[i], T)
        contact += int(its.max() > 2)
        np.testing.assert_allclose(qh[i], qs, rtol=0, atol=1e-9)
        o0, od0, of = oracle.bdf1_backward(m, pairs, qs, qd0[i], w[i])
        assert nrel(g0[i], o0) <= 1e-6, i
        assert nrel(gd0[i], od0) <= 1e-6, i
        assert nrel(gf[i], of) <= 1e-6, i
    assert contact > 0


def test_gradients_against_finite_differences(sdfc):
    """One batch holds the base scene and its +-1e-6 perturbations of q0, qdot0 and
    the external force; L's central differences across the batch against the
    adjoint of the base scene."""
    fx = load("sim_trans.npz")
    T, eps = 12, 1e-6
    w = np.random.default_rng(5).normal(size=(T, 3))
    base = (np.asarray(fx["q0"], float), np.asarray(fx["qdot0"], float), np.asarray(fx["f_ext"], float))
    scenes = [base]
    for which, dim, offset in ((0, 3, 0), (1, 3, 0), (2, 3, 3)):
        for j in range(dim):
            for sgn in (1, -1):
                s = [a.copy() for a in base]
                s[which][offset + j] += sgn * eps
                scenes.append(tuple(s))
    n = len(scenes)
    ctx = sdfc.Context(0)
    try:
        sim = make_sim(sdfc, ctx, fx, n=n, f_ext=np.array([s[2] for s in scenes]),
                       q0=np.array([s[0] for s in scenes]), qd0=np.array([s[1] for s in scenes]))
        sim.record(T)
        assert sim.step(T).all()
        L = (sim.history()[:, 1:] * w).sum(axis=(1, 2))
        g0, gd0, gf = sim.backward(np.tile(w, (n, 1, 1)))
    finally:
        ctx.close()
    fd = (L[1::2] - L[2::2]) / (2 * eps)
    for got, want in ((g0[0], fd[0:3]), (gd0[0], fd[3:6]), (gf[0, 3:], fd[6:9])):
        assert np.linalg.norm(got - want) <= 1e-4 * np.linalg.norm(got), (got, want)


def test_recording_rules(sdfc):
    fx = load("sim_trans.npz")
    ctx = sdfc.Context(0)
    try:
        sim = make_sim(sdfc, ctx, fx)
        with pytest.raises(sdfc.SdfcError):
            sim.backward(np.zeros((1, 0, 3)))  # not recording
        sim.record(3)
        g0, gd0, gf = sim.backward(np.zeros((1, 0, 3)))  # nothing recorded yet
        assert not g0.any() and not gd0.any() and not gf.any()
        sim.step(2)
        with pytest.raises(sdfc.SdfcError):
            sim.step(2)  # beyond max_steps
        sim.step(1)
        assert sim.history().shape == (1, 4, 3)
        with pytest.raises(ValueError):
            sim.backward(np.zeros((1, 2, 3)))  # wrong horizon
        # a new initial state restarts the recording
        sim.set_state(fx["q0"][None], fx["qdot0"][None])
        assert sim.history().shape == (1, 1, 3)
        sim.step(1)
        g0, _, _ = sim.backward(np.ones((1, 1, 3)))
        assert np.all(np.isfinite(g0)) and np.abs(g0).sum() > 0
        sim.record(0)
        with pytest.raises(sdfc.SdfcError):
            sim.history()
    finally:
        ctx.close()


def test_torch_autograd(sdfc):
    torch = pytest.importorskip("torch")
    ag = submodule("autograd")
    fx = load("sim_trans.npz")
    T, n = 8, 3
    rng = np.random.default_rng(2)
    w = torch.tensor(rng.normal(size=(n, T, 3)))
    ctx = sdfc.Context(0)
    try:
        sim = make_sim(sdfc, ctx, fx, n=n)
        q0 = torch.tensor(np.tile(fx["q0"], (n, 1)), requires_grad=True)
        qd0 = torch.tensor(np.tile(fx["qdot0"], (n, 1)), requires_grad=True)
        fe = torch.tensor(np.tile(fx["f_ext"], (n, 1)) * np.array([[1, 1, 1, 1, 0.5, 2]]), requires_grad=True)
        q, E = ag.rollout(sim, q0, qd0, fe, T)
        assert q.shape == (n, T, 3) and not E.any()
        loss = (q * w).sum()
        loss.backward()
        g0, gd0, gf = sim.backward(w.numpy())
        np.testing.assert_array_equal(q0.grad.numpy(), g0)
        np.testing.assert_array_equal(qd0.grad.numpy(), gd0)
        np.testing.assert_array_equal(fe.grad.numpy(), gf)
        # a stepped simulation no longer holds the rollout's trajectory
        q, _ = ag.rollout(sim, q0, qd0, fe, T)
        sim.step(0)
        with pytest.raises(RuntimeError):
            (q * w).sum().backward()
    finally:
        ctx.close()
