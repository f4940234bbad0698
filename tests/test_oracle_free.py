"""The oracle's free3d-exp mover (6 dof: translation and exponential rotation coordinates)
against the reference: tests/golden/sim_free.npz holds a peg on a free3d-exp joint stepped by
the reference simulator (40 steps, rotating, in contact with a socket, pushed by an external
torque and force) and the reference's backward() for a 20-step loss.

Bars: trajectory to 1e-11 (the restatement follows the reference's operations up to summation
order), backward to 1e-7 relative (its FD-stencil Hessians amplify the trajectories' 1e-13
differences), central differences (step 1e-6) to 1e-4 of the gradient's norm."""
import numpy as np

from _helpers import load


def scene(oracle, fx, f_ext=None, newton_tol=0.0):
    grid = oracle.Grid(fx["grid"], fx["min_box"], fx["max_box"], fx["dx"], float(fx["col_th"]))
    mover = oracle.Mover(float(fx["mass"]), fx["inertia"], fx["E_ji"], np.eye(4), tuple(fx["gravity"]),
                         float(fx["h"]), fx["f_ext"] if f_ext is None else f_ext, ndof=6, newton_tol=newton_tol)
    pair = oracle.ScenePair(grid, fx["points"], True, fx["E_fixed"], oracle.Params(*fx["params"]))
    return mover, [pair]


def test_free_trajectory_matches_reference(oracle):
    fx = load("sim_free.npz")
    mover, pairs = scene(oracle, fx)
    steps = len(fx["q"]) - 1
    qs, qds, conv, its, _ = oracle.bdf1_steps(mover, pairs, fx["q0"], fx["qdot0"], steps)
    np.testing.assert_allclose(qs, fx["q"], rtol=0, atol=1e-11)
    np.testing.assert_allclose(qds, fx["qdot"], rtol=0, atol=1e-9)
    assert np.array_equal(conv, fx["converged"])
    assert its.max() > 4 and np.abs(qs[-1, 3:] - qs[0, 3:]).max() > 1e-3  # contact and rotation


def test_free_adjoint_matches_reference(oracle):
    fx = load("sim_free.npz")
    mover, pairs = scene(oracle, fx)
    T = int(fx["bw_steps"])
    qs, _, _, _, _ = oracle.bdf1_steps(mover, pairs, fx["q0"], fx["qdot0"], T)
    g0, gd0, _ = oracle.bdf1_backward(mover, pairs, qs, fx["qdot0"], fx["bw_df_dq"])
    np.testing.assert_allclose(g0, fx["bw_df_dq0"], rtol=1e-7, atol=0)
    np.testing.assert_allclose(gd0, fx["bw_df_dqdot0"], rtol=1e-7, atol=0)


def test_free_adjoint_against_central_differences(oracle):
    """The adjoint differentiates the solution of g = 0 at every step.  With the reference's
    stopping rule (|g| < 1e-8) a +-1e-6 perturbation can stop Newton at a different iterate
    (here one step ends at |g| = 9e-9), which puts ~1e-2 relative noise into central
    differences; so both rollouts here solve g = 0 to 1e-13."""
    fx = load("sim_free.npz")
    T, eps, tol = 10, 1e-6, 1e-13
    w = np.random.default_rng(4).normal(size=(T, 6))
    mover, pairs = scene(oracle, fx, newton_tol=tol)
    qs, _, conv, _, _ = oracle.bdf1_steps(mover, pairs, fx["q0"], fx["qdot0"], T)
    assert conv.all()
    g0, gd0, gf = oracle.bdf1_backward(mover, pairs, qs, fx["qdot0"], w)

    def loss(q0, qd0, fe):
        m, p = scene(oracle, fx, fe, newton_tol=tol)
        q, _, _, _, _ = oracle.bdf1_steps(m, p, q0, qd0, T)
        return float((q[1:] * w).sum())

    base = [np.asarray(fx["q0"], float), np.asarray(fx["qdot0"], float), np.asarray(fx["f_ext"], float)]
    for which, got in ((0, g0), (1, gd0), (2, gf)):
        fd = np.zeros(len(base[which]))
        for j in range(len(fd)):
            a, b = [x.copy() for x in base], [x.copy() for x in base]
            a[which][j] += eps
            b[which][j] -= eps
            fd[j] = (loss(*a) - loss(*b)) / (2 * eps)
        assert np.linalg.norm(got - fd) <= 1e-4 * np.linalg.norm(got), (which, got, fd)
