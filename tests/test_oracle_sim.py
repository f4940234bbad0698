"""The oracle's BDF1 Newton restatement against the reference's own trajectory.

tests/golden/sim_trans.npz holds a scene and the joint trajectory the reference
simulator produced for it (tests/golden/make_golden.py); where the reference
build is present the restatement is also run against it live."""
import numpy as np

from _helpers import load


def scene(oracle, fx):
    grid = oracle.Grid(fx["grid"], fx["min_box"], fx["max_box"], fx["dx"], float(fx["col_th"]))
    mover = oracle.Mover(float(fx["mass"]), fx["inertia"], fx["E_ji"], np.eye(4), tuple(fx["gravity"]),
                         float(fx["h"]), fx["f_ext"])
    pair = oracle.ScenePair(grid, fx["points"], True, fx["E_fixed"], oracle.Params(*fx["params"]))
    return mover, [pair]


def test_bdf1_trajectory_matches_reference(oracle):
    fx = load("sim_trans.npz")
    mover, pairs = scene(oracle, fx)
    steps = len(fx["q"]) - 1
    qs, qds, conv, its, evs = oracle.bdf1_steps(mover, pairs, fx["q0"], fx["qdot0"], steps)
    # the restatement follows the reference's arithmetic: the trajectory agrees to round-off
    np.testing.assert_allclose(qs, fx["q"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(qds, fx["qdot"], rtol=0, atol=1e-9)
    assert np.array_equal(conv, fx["converged"])
    assert its.max() > 2  # the scene exercises Newton with contact
