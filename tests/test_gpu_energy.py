"""Penetration-energy losses on rollouts (sdfc_sim_record_energy / sdfc_sim_backward_energy):
the recorded per-step energies equal sdfc_batch_energy at the recorded states, and the adjoint of
L = sum_t E_t + |q_T - target|^2 (a rotating free3d-exp peg, the loss of the differentiable-rollout
workload) matches central differences (step 1e-6, Newton solved to 1e-13 so that the differences
resolve the implicit steps) to 1e-4 of the gradient's norm, for the initial pose, initial velocity
and pull force."""
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


def test_recorded_energy_matches_batch_energy(sdfc):
    fx = load("sim_free.npz")
    T = 6
    ctx = sdfc.Context(0)
    try:
        sim = make_sim(sdfc, ctx, fx, precision=0, joint=sdfc.JOINT_FREE3D_EXP)
        sim.record_energy(True)
        sim.record(T)
        sim.step(T)
        per, tot = sim.energy()
        qh = sim.history()
        assert per.shape == (1, T) and np.allclose(tot, per.sum(1)) and per.max() > 0
        # the same energies through sdfc_batch_energy at the recorded end states
        g = ctx.upload_grid(fx["grid"], fx["min_box"], fx["max_box"], fx["dx"], float(fx["col_th"]), 1)
        p = ctx.upload_points(fx["points"], 1)
        b = ctx.batch([p] * T, [g] * T)
        b.set_precision(0)
        W = submodule("workloads")
        h = float(fx["h"])
        EA = []
        for t in range(1, T + 1):
            # pose of the free joint: [R(r) p] composed with E_ji (q = (p, r))
            R = W.rotvec_to_matrix(qh[0, t, 3:])
            EA.append(W.pose(R, qh[0, t, :3]) @ fx["E_ji"])
        prm = [sdfc.Params(*[float(x) for x in fx["params"]])] * T
        e, _ = b.energy(np.array(EA), np.tile(fx["E_fixed"], (T, 1, 1)), prm)
        np.testing.assert_allclose(per[0], e, rtol=1e-10, atol=0)
        b.close()
    finally:
        ctx.close()


def test_energy_loss_adjoint_against_central_differences(sdfc):
    fx = load("sim_free.npz")
    T, eps, tol = 8, 1e-6, 1e-13
    target = np.asarray(fx["q"][T], float) + np.array([0.01, -0.02, 0.005, 0.01, 0.0, -0.02])
    base = [np.asarray(fx["q0"], float), np.asarray(fx["qdot0"], float), np.asarray(fx["f_ext"], float)]
    scenes = [base]
    for which, dim, off in ((0, 6, 0), (1, 6, 0), (2, 6, 0)):
        for j in range(dim):
            for sgn in (1, -1):
                s_ = [a.copy() for a in base]
                s_[which][off + j] += sgn * eps
                scenes.append(s_)
    n = len(scenes)
    ctx = sdfc.Context(0)
    try:
        sim = make_sim(sdfc, ctx, fx, n=n, precision=0, joint=sdfc.JOINT_FREE3D_EXP,
                       q0=np.array([s_[0] for s_ in scenes]), qd0=np.array([s_[1] for s_ in scenes]),
                       f_ext=np.array([s_[2] for s_ in scenes]))
        sim.set_tolerance(tol)
        sim.record_energy(True)
        sim.record(T)
        sim.step(T)
        qh = sim.history()
        _, E = sim.energy()
        assert E[0] > 0
        L = E + ((qh[:, T] - target) ** 2).sum(1)
        df_dq = np.zeros((n, T, 6))
        df_dq[:, T - 1] = 2.0 * (qh[:, T] - target)
        g0, gd0, gf = sim.backward(df_dq, np.ones(n))
    finally:
        ctx.close()
    fd = (L[1::2] - L[2::2]) / (2 * eps)
    for got, want in ((g0[0], fd[0:6]), (gd0[0], fd[6:12]), (gf[0], fd[12:18])):
        assert np.linalg.norm(got - want) <= 1e-4 * np.linalg.norm(got), (got, want)


def test_torch_rollout_with_energy(sdfc):
    """autograd.rollout's energy output backpropagates through sdfc_sim_backward_energy."""
    torch = pytest.importorskip("torch")
    ag = submodule("autograd")
    fx = load("sim_free.npz")
    T, n = 5, 2
    ctx = sdfc.Context(0)
    try:
        sim = make_sim(sdfc, ctx, fx, n=n, joint=sdfc.JOINT_FREE3D_EXP)
        q0 = torch.tensor(np.tile(fx["q0"], (n, 1)), requires_grad=True)
        qd0 = torch.tensor(np.tile(fx["qdot0"], (n, 1)), requires_grad=True)
        fe = torch.tensor(np.tile(fx["f_ext"], (n, 1)), requires_grad=True)
        q, E = ag.rollout(sim, q0, qd0, fe, T, energy=True)
        assert (E > 0).all()
        (E.sum() + (q[:, -1] ** 2).sum()).backward()
        df_dq = np.zeros((n, T, 6))
        df_dq[:, -1] = 2.0 * q[:, -1].detach().numpy()
        g0, gd0, gf = sim.backward(df_dq, np.ones(n))
        np.testing.assert_array_equal(q0.grad.numpy(), g0)
        np.testing.assert_array_equal(fe.grad.numpy(), gf)
    finally:
        ctx.close()
