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


def test_warp_newton_matches_thread_newton(sdfc, monkeypatch):
    """The free-joint Newton update runs on one warp per scene (sdfc_joint_warp.cuh); the one-
    thread version (selected by SDFC_FREE_NEWTON_THREAD at creation) computes the same entries
    in the same order.  Both drive the same rollout: trajectories agree to round-off and the
    Newton counts are identical."""
    fx = load("sim_free.npz")
    rng = np.random.default_rng(23)
    n, T = 16, 12
    F = np.zeros((n, 6))
    F[:, :3] = rng.normal(size=(n, 3)) * 0.1
    F[:, 3:] = rng.normal(size=(n, 3)) * 3.0
    q0 = np.tile(fx["q0"], (n, 1)) + rng.normal(size=(n, 6)) * [0.004, 0.004, 0.05, 0.01, 0.01, 0.3]
    q0[0, 3:] = 0.0  # the small-rotation branch of the exponential map
    qd0 = rng.normal(size=(n, 6)) * [0.3, 0.3, 0.3, 0.5, 0.5, 0.5]
    out = []
    for thread in (False, True):
        if thread:
            monkeypatch.setenv("SDFC_FREE_NEWTON_THREAD", "1")
        else:
            monkeypatch.delenv("SDFC_FREE_NEWTON_THREAD", raising=False)
        ctx = sdfc.Context(0)
        try:
            sim = make_sim(sdfc, ctx, fx, n=n, f_ext=F, q0=q0, qd0=qd0, joint=sdfc.JOINT_FREE3D_EXP)
            sim.record(T)
            conv = sim.step(T)
            out.append((sim.history(), conv, sim.stats()))
        finally:
            ctx.close()
    (qa, ca, sa), (qb, cb, sb) = out
    np.testing.assert_allclose(qa, qb, rtol=0, atol=1e-12)
    assert np.array_equal(ca, cb)
    assert sa == sb


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("joint", ["free", "trans"])
def test_compacted_rounds_match_full_rounds(sdfc, monkeypatch, joint, precision):
    """Late Newton rounds evaluate only the scenes still iterating (compacted rounds, sized by
    capacity buckets).  Every pair's evaluation is independent of the others, and both kinds of
    round pose the movers with one compiled function, so a rollout with compaction is
    bit-identical to one with full rounds only (SDFC_SIM_NO_COMPACT), with FP64 evaluations too
    (where a pose differing in its last bit would show)."""
    fx = load("sim_free.npz" if joint == "free" else "sim_trans.npz")
    nd = 6 if joint == "free" else 3
    rng = np.random.default_rng(29)
    n, T = 64, 8
    F = np.zeros((n, 6))
    F[:, 3:] = rng.normal(size=(n, 3)) * 3.0
    q0 = np.tile(fx["q0"], (n, 1)) + rng.normal(size=(n, nd)) * 0.004
    qd0 = rng.normal(size=(n, nd)) * 0.3
    out = []
    for compact in (True, False):
        if compact:
            monkeypatch.delenv("SDFC_SIM_NO_COMPACT", raising=False)
        else:
            monkeypatch.setenv("SDFC_SIM_NO_COMPACT", "1")
        ctx = sdfc.Context(0)
        try:
            sim = make_sim(sdfc, ctx, fx, n=n, f_ext=F, q0=q0, qd0=qd0,
                           joint=sdfc.JOINT_FREE3D_EXP if joint == "free" else sdfc.JOINT_TRANSLATIONAL)
            sim.set_precision(precision)
            sim.record(T)
            conv = sim.step(T)
            out.append((sim.history(), conv, sim.stats()))
        finally:
            ctx.close()
    (qa, ca, sa), (qb, cb, sb) = out
    assert np.array_equal(qa, qb)
    assert np.array_equal(ca, cb)
    assert sa == sb


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("joint", ["free", "trans"])
def test_free_running_steps_match_lockstep(sdfc, monkeypatch, joint, precision):
    """Within one sdfc_sim_step call every scene takes its steps one after another without
    waiting for the other scenes (a scene that has converged starts its next step in the next
    round).  Scenes are independent and each evaluation depends on its own inputs alone, so the
    trajectories, convergence flags, recorded energies, adjoint gradients and per-scene evaluation
    counts are bit-identical to rounds in which every step waits for all scenes
    (SDFC_SIM_LOCKSTEP), in fewer rounds.  The call is split (5 + 7 steps) to cover a call
    starting from the state and recording row the previous call left."""
    fx = load("sim_free.npz" if joint == "free" else "sim_trans.npz")
    nd = 6 if joint == "free" else 3
    rng = np.random.default_rng(31)
    n, T = 48, 12
    F = np.zeros((n, 6))
    F[:, 3:] = rng.normal(size=(n, 3)) * 3.0
    q0 = np.tile(fx["q0"], (n, 1)) + rng.normal(size=(n, nd)) * 0.004
    qd0 = rng.normal(size=(n, nd)) * 0.3
    df_dq = rng.normal(size=(n, T, nd))
    out = []
    for lockstep in (False, True):
        if lockstep:
            monkeypatch.setenv("SDFC_SIM_LOCKSTEP", "1")
        else:
            monkeypatch.delenv("SDFC_SIM_LOCKSTEP", raising=False)
        ctx = sdfc.Context(0)
        try:
            sim = make_sim(sdfc, ctx, fx, n=n, f_ext=F, q0=q0, qd0=qd0, precision=precision,
                           joint=sdfc.JOINT_FREE3D_EXP if joint == "free" else sdfc.JOINT_TRANSLATIONAL)
            sim.record_energy(True)
            sim.record(T)
            c1 = sim.step(5)
            c2 = sim.step(T - 5)
            E, Etot = sim.energy()
            grads = sim.backward(df_dq, np.ones(n))
            out.append((sim.history(), c1, c2, E, Etot, grads, sim.scene_evaluations(), sim.stats(), sim.get_state()))
        finally:
            ctx.close()
    free, lock = out
    for a, b in zip(free[:5], lock[:5]):
        assert np.array_equal(a, b)
    assert all(np.array_equal(a, b) for a, b in zip(free[5], lock[5]))
    assert np.array_equal(free[6], lock[6])
    assert free[7][1] == lock[7][1]  # evaluations
    assert free[7][0] < lock[7][0]  # rounds
    assert all(np.array_equal(a, b) for a, b in zip(free[8], lock[8]))
    assert (free[4] > 0).any()  # the scenes touch the bore
