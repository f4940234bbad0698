"""The oracle's adjoint of the BDF1 rollout (Simulation::backward_BDF1) against the
reference's own backward pass and against central finite differences.

tests/golden/sim_trans.npz holds, besides the reference trajectory, the reference's
dL/dq0 and dL/dqdot0 for L = sum_k w_k . q_k over 20 steps (bw_df_dq = w).  The
external-force gradient has no reference counterpart (the reference does not treat
the external force as a parameter), so it is checked against central differences
only.  FD bar: |fd - adjoint| <= 1e-4 |adjoint| with step 1e-6 (Newton stops at
|g| < 1e-8, which bounds how well the rollout's derivatives can be resolved)."""
import numpy as np

from _helpers import load
from test_oracle_sim import scene

FD_EPS = 1e-6
FD_REL = 1e-4


def rollout_loss(oracle, mover, pairs, q0, qd0, f_ext, w):
    m = oracle.Mover(mover.mass, mover.inertia, mover.E_ji, mover.E_pj0, mover.gravity, mover.h, np.asarray(f_ext))
    qs, _, _, _, _ = oracle.bdf1_steps(m, pairs, q0, qd0, len(w))
    return float((qs[1:] * w).sum())


def test_adjoint_matches_reference_backward(oracle):
    fx = load("sim_trans.npz")
    mover, pairs = scene(oracle, fx)
    T = int(fx["bw_steps"])
    qs, _, conv, _, _ = oracle.bdf1_steps(mover, pairs, fx["q0"], fx["qdot0"], T)
    assert conv.all()
    g0, gd0, gf = oracle.bdf1_backward(mover, pairs, qs, fx["qdot0"], fx["bw_df_dq"])
    np.testing.assert_allclose(g0, fx["bw_df_dq0"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(gd0, fx["bw_df_dqdot0"], rtol=1e-12, atol=0)
    assert np.all(gf[:3] == 0.0)  # the translational joint does not see torques


def test_adjoint_against_central_differences(oracle):
    fx = load("sim_trans.npz")
    mover, pairs = scene(oracle, fx)
    T = 12
    w = np.random.default_rng(5).normal(size=(T, 3))
    q0, qd0, fe = fx["q0"], fx["qdot0"], fx["f_ext"]
    qs, _, conv, its, _ = oracle.bdf1_steps(mover, pairs, q0, qd0, T)
    assert conv.all() and its.max() > 2
    g0, gd0, gf = oracle.bdf1_backward(mover, pairs, qs, qd0, w)

    def fd(which, n):
        out = np.zeros(n)
        for j in range(n):
            e = np.zeros(n)
            e[j] = FD_EPS
            args = {"q0": q0, "qd0": qd0, "f_ext": fe}
            args[which] = args[which] + e
            lp = rollout_loss(oracle, mover, pairs, args["q0"], args["qd0"], args["f_ext"], w)
            args[which] = args[which] - 2 * e
            lm = rollout_loss(oracle, mover, pairs, args["q0"], args["qd0"], args["f_ext"], w)
            out[j] = (lp - lm) / (2 * FD_EPS)
        return out

    for got, want in ((g0, fd("q0", 3)), (gd0, fd("qd0", 3)), (gf, fd("f_ext", 6))):
        assert np.linalg.norm(got - want) <= FD_REL * np.linalg.norm(got), (got, want)


def test_adjoint_short_horizons(oracle):
    """T = 1 and T = 2 exercise the recursion's boundary terms (Simulation.cpp:1577-1584,
    1596-1614)."""
    fx = load("sim_trans.npz")
    mover, pairs = scene(oracle, fx)
    for T in (1, 2):
        w = np.random.default_rng(T).normal(size=(T, 3))
        qs, _, _, _, _ = oracle.bdf1_steps(mover, pairs, fx["q0"], fx["qdot0"], T)
        g0, gd0, _ = oracle.bdf1_backward(mover, pairs, qs, fx["qdot0"], w)
        # dense check: every q_k is linear in q0 to first order; compare with FD
        fd0 = np.zeros(3)
        for j in range(3):
            e = np.zeros(3)
            e[j] = FD_EPS
            fd0[j] = (rollout_loss(oracle, mover, pairs, fx["q0"] + e, fx["qdot0"], fx["f_ext"], w) -
                      rollout_loss(oracle, mover, pairs, fx["q0"] - e, fx["qdot0"], fx["f_ext"], w)) / (2 * FD_EPS)
        assert np.linalg.norm(g0 - fd0) <= FD_REL * np.linalg.norm(g0), (T, g0, fd0)
        assert np.all(np.isfinite(gd0))
