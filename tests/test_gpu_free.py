"""Free3d-exp movers (6 dof: translation and exponential rotation coordinates) on the GPU:
batched BDF1 steps and their adjoint against the reference's free-joint trajectory and backward
(tests/golden/sim_free.npz) and against the oracle's restatement for a batch of differently
pushed, rotating scenes.

Bars: FP64 evaluations 1e-9 in q (Newton stops at |g| < 1e-8), mixed precision 1e-6; adjoint
against the reference backward 1e-7 (stencil mode: the reference's own Hessians), 1e-6 (analytic),
1e-4 (mixed), and 1e-6 against the oracle's adjoint on the oracle's trajectory."""
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


@pytest.mark.parametrize("precision,atol", [(0, 1e-9), (1, 1e-6)])
def test_reference_trajectory(sdfc, precision, atol):
    fx = load("sim_free.npz")
    ctx = sdfc.Context(0)
    try:
        sim = make_sim(sdfc, ctx, fx, precision=precision, joint=sdfc.JOINT_FREE3D_EXP)
        for t in range(1, len(fx["q"])):
            conv = sim.step(1)
            q, qd = sim.get_state()
            assert q.shape == (1, 6)
            np.testing.assert_allclose(q[0], fx["q"][t], rtol=0, atol=atol, err_msg=f"step {t}")
            np.testing.assert_allclose(qd[0], fx["qdot"][t], rtol=0, atol=atol / fx["h"] * 2, err_msg=f"step {t}")
            if precision == 0:
                assert bool(conv[0]) == bool(fx["converged"][t - 1])
    finally:
        ctx.close()


@pytest.mark.parametrize("precision,deriv,bar", [(0, 1, 1e-7), (0, 0, 1e-6), (1, 0, 1e-4)])
def test_reference_backward(sdfc, precision, deriv, bar):
    fx = load("sim_free.npz")
    T = int(fx["bw_steps"])
    ctx = sdfc.Context(0)
    try:
        ctx.set_derivative_mode(deriv)
        sim = make_sim(sdfc, ctx, fx, precision=precision, joint=sdfc.JOINT_FREE3D_EXP)
        sim.record(T)
        sim.step(T)
        g0, gd0, gf = sim.backward(fx["bw_df_dq"][None])
        assert nrel(g0[0], fx["bw_df_dq0"]) <= bar
        assert nrel(gd0[0], fx["bw_df_dqdot0"]) <= bar
        assert np.abs(gf[0, :3]).max() > 0  # torques reach the rotation
    finally:
        ctx.close()


def test_batch_against_oracle(sdfc, oracle):
    fx = load("sim_free.npz")
    from test_oracle_free import scene
    rng = np.random.default_rng(17)
    n, T = 8, 10
    F = np.zeros((n, 6))
    F[:, :3] = rng.normal(size=(n, 3)) * 0.1
    F[:, 3:] = rng.normal(size=(n, 3)) * 3.0
    q0 = np.tile(fx["q0"], (n, 1)) + rng.normal(size=(n, 6)) * [0.004, 0.004, 0.05, 0.01, 0.01, 0.3]
    qd0 = rng.normal(size=(n, 6)) * [0.3, 0.3, 0.3, 0.5, 0.5, 0.5]
    w = rng.normal(size=(n, T, 6))
    ctx = sdfc.Context(0)
    try:
        sim = make_sim(sdfc, ctx, fx, n=n, f_ext=F, q0=q0, qd0=qd0, joint=sdfc.JOINT_FREE3D_EXP)
        sim.record(T)
        sim.step(T)
        qh = sim.history()
        g0, gd0, gf = sim.backward(w)
    finally:
        ctx.close()
    contact = 0
    for i in range(n):
        mover, pairs = scene(oracle, fx, F[i])
        qs, _, _, its, _ = oracle.bdf1_steps(mover, pairs, q0[i], qd0[i], T)
        contact += int(its.max() > 2)
        np.testing.assert_allclose(qh[i], qs, rtol=0, atol=1e-9, err_msg=f"scene {i}")
        o0, od0, of = oracle.bdf1_backward(mover, pairs, qs, qd0[i], w[i])
        assert nrel(g0[i], o0) <= 1e-6, i
        assert nrel(gd0[i], od0) <= 1e-6, i
        assert nrel(gf[i], of) <= 1e-6, i
    assert contact > 0


def test_mixed_joint_types_rejected(sdfc):
    fx = load("sim_free.npz")
    ctx = sdfc.Context(0)
    try:
        g = ctx.upload_grid(fx["grid"], fx["min_box"], fx["max_box"], fx["dx"], float(fx["col_th"]), 1)
        p = ctx.upload_points(fx["points"], 1)
        a = sdfc.Mover.make(1.0, np.ones(6), np.eye(4), 1e-3, joint=sdfc.JOINT_FREE3D_EXP)
        b = sdfc.Mover.make(1.0, np.ones(6), np.eye(4), 1e-3, joint=sdfc.JOINT_TRANSLATIONAL)
        prm = sdfc.Params(1e5)
        pairs = [sdfc.ScenePair.make(i, p, g, True, np.eye(4), prm) for i in range(2)]
        with pytest.raises(sdfc.SdfcError):
            ctx.sim([a, b], pairs)
        with pytest.raises(sdfc.SdfcError):
            ctx.sim([sdfc.Mover.make(1.0, np.ones(6), np.eye(4), 1e-3, joint=4)], pairs[:1])
    finally:
        ctx.close()
