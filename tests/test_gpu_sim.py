"""Batched BDF1 Newton steps on the GPU (sdfc_sim_*) against the reference's
trajectory (tests/golden/sim_trans.npz, made by the reference simulator) and
against the oracle's restatement for a batch of differently pushed scenes.

Bars: FP64 force evaluations reproduce the reference trajectory to 1e-9 in q
(Newton stops at |g| < 1e-8, so converged iterates agree to that order) with
the same convergence flags; the mixed-precision evaluations to 1e-6."""
import numpy as np
import pytest

from _helpers import load
from conftest import submodule

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sdfc():
    submodule("build").build()
    return submodule("sdfc")


def make_sim(sdfc, ctx, fx, n=1, f_ext=None, q0=None, qd0=None, precision=0, joint=3):
    g = ctx.upload_grid(fx["grid"], fx["min_box"], fx["max_box"], fx["dx"], float(fx["col_th"]), 1)
    p = ctx.upload_points(fx["points"], 1)
    mover = sdfc.Mover.make(float(fx["mass"]), fx["inertia"], fx["E_ji"], float(fx["h"]), tuple(fx["gravity"]),
                            joint=joint)
    prm = sdfc.Params(*[float(x) for x in fx["params"]])
    pairs = [sdfc.ScenePair.make(i, p, g, True, fx["E_fixed"], prm) for i in range(n)]
    sim = ctx.sim([mover] * n, pairs)
    sim.set_precision(precision)
    sim.set_state(np.tile(fx["q0"], (n, 1)) if q0 is None else q0, np.tile(fx["qdot0"], (n, 1)) if qd0 is None else qd0)
    sim.set_external_force(np.tile(fx["f_ext"], (n, 1)) if f_ext is None else f_ext)
    return sim


@pytest.mark.parametrize("precision,atol", [(0, 1e-9), (1, 1e-6)])
def test_reference_trajectory(sdfc, precision, atol):
    fx = load("sim_trans.npz")
    ctx = sdfc.Context(0)
    try:
        sim = make_sim(sdfc, ctx, fx, precision=precision)
        for t in range(1, len(fx["q"])):
            conv = sim.step(1)
            q, qd = sim.get_state()
            np.testing.assert_allclose(q[0], fx["q"][t], rtol=0, atol=atol, err_msg=f"step {t}")
            assert bool(conv[0]) == bool(fx["converged"][t - 1])
        rounds, evals = sim.stats()
        assert rounds >= 2 * (len(fx["q"]) - 1)
    finally:
        ctx.close()


def test_batch_against_oracle(sdfc, oracle):
    fx = load("sim_trans.npz")
    rng = np.random.default_rng(3)
    n, steps = 12, 12
    F = np.zeros((n, 6))
    F[:, 3:] = rng.normal(size=(n, 3)) * 3.0
    q0 = np.tile(fx["q0"], (n, 1)) + rng.normal(size=(n, 3)) * [0.004, 0.004, 0.05]
    qd0 = rng.normal(size=(n, 3)) * 0.3
    ctx = sdfc.Context(0)
    try:
        sim = make_sim(sdfc, ctx, fx, n=n, f_ext=F, q0=q0, qd0=qd0)
        conv = sim.step(steps)
        q, qd = sim.get_state()
    finally:
        ctx.close()
    grid = oracle.Grid(fx["grid"], fx["min_box"], fx["max_box"], fx["dx"], float(fx["col_th"]))
    pair = oracle.ScenePair(grid, fx["points"], True, fx["E_fixed"], oracle.Params(*fx["params"]))
    for i in range(n):
        mover = oracle.Mover(float(fx["mass"]), fx["inertia"], fx["E_ji"], np.eye(4), tuple(fx["gravity"]),
                             float(fx["h"]), F[i])
        qs, qds, cv, _, _ = oracle.bdf1_steps(mover, [pair], q0[i], qd0[i], steps)
        np.testing.assert_allclose(q[i], qs[-1], rtol=0, atol=1e-9, err_msg=f"scene {i}")
        np.testing.assert_allclose(qd[i], qds[-1], rtol=0, atol=1e-7, err_msg=f"scene {i}")
        assert bool(conv[i]) == bool(cv[-1])
