"""Failure detection, with every fault made on the host (no GPU fault, trap or hang).

  * A non-finite pose or coefficient in one instance of a batch sets that instance's status
    (bit 1), finds no contact for it (the reference's distance query puts non-finite points
    outside the grid), and leaves every other instance bit-identical to a clean evaluation.
  * A scene whose state is not finite never converges (Simulation::is_converged false, as the
    reference's Newton stops on its line-search strikes, rm/Simulation.cpp:1040-1076) while the
    other scenes of the sim step exactly as without it.
  * A Newton tolerance that cannot be met (1e-300) runs each step to the reference's stopping
    rule and reports converged = false, as the oracle's restatement of that rule does, on the
    same trajectory.
  * The level-set sweep's bounded waits, made to run out (the test hook
    SDFC_TEST_EXPIRE_SWEEP_WAITS makes every wait await progress that no plane reaches), end the
    call with an error status; the context stays usable and the next call is exact."""
import os
import subprocess
import sys

import numpy as np
import pytest

from _helpers import load
from conftest import ROOT, submodule
from test_gpu_sim import make_sim

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sdfc():
    submodule("build").build()
    return submodule("sdfc")


def test_nonfinite_inputs_flag_only_their_instance(sdfc, workloads):
    rng = np.random.default_rng(12)
    g = workloads.socket_grid(48, dtype=np.float32)
    ctx = sdfc.Context(0)
    try:
        gh = ctx.upload_grid(g.values, g.min_box, g.max_box, g.dx, 0.01, 1)
        ph = ctx.upload_points(workloads.peg_points(6000, seed=4), 1)
        n = 6
        ang = rng.uniform(0, 2 * np.pi, n)
        EA = np.stack([workloads.pose(workloads.rotvec_to_matrix(rng.normal(size=3) * 0.004),
                                      [0.026 * np.cos(a), 0.026 * np.sin(a), 0.3 * rng.normal()]) for a in ang])
        EB = np.tile(np.eye(4), (n, 1, 1))
        phiA = rng.normal(size=(n, 6)) * 0.2
        phiB = np.zeros((n, 6))
        prm = [sdfc.Params(1e5, 1e3, 0.3, 1e3)] * n
        for precision in (0, 1):
            b = ctx.batch([ph] * n, [gh] * n)
            b.set_precision(precision)
            clean = b.evaluate(EA, phiA, EB, phiB, prm, want_deriv=True)
            assert (clean[3] > 0).all() and not clean[4].any()
            EA2 = EA.copy()
            EA2[2, 0, 3] = np.nan  # a pose
            prm2 = list(prm)
            prm2[4] = sdfc.Params(np.inf, 1e3, 0.3, 1e3)  # a coefficient
            bad = b.evaluate(EA2, phiA, EB, phiB, prm2, want_deriv=True)
            fm, Km, Dm, nact, st = bad
            assert st[2] & 2 and st[4] & 2
            assert nact[2] == 0 and not fm[2].any()
            for k in (0, 1, 3, 5):
                assert st[k] == 0
                assert np.array_equal(fm[k], clean[0][k]) and np.array_equal(Km[k], clean[1][k])
                assert np.array_equal(Dm[k], clean[2][k]) and nact[k] == clean[3][k]
            # the value pass too
            fv, _, _, nv, sv = b.evaluate(EA2, phiA, EB, phiB, prm2, want_deriv=False)
            assert sv[2] & 2 and sv[4] & 2 and not sv[[0, 1, 3, 5]].any() and nv[2] == 0
            b.close()
    finally:
        ctx.close()


def test_nonfinite_scene_does_not_converge(sdfc):
    fx = load("sim_trans.npz")
    n, T = 6, 8
    rng = np.random.default_rng(3)
    f_ext = np.tile(fx["f_ext"], (n, 1)) * (1.0 + 0.2 * rng.normal(size=(n, 1)))
    runs = []
    ctx = sdfc.Context(0)
    try:
        for poison in (False, True):
            q0 = np.tile(fx["q0"], (n, 1))
            if poison:
                q0[3, 1] = np.nan
            sim = make_sim(sdfc, ctx, fx, n=n, q0=q0, f_ext=f_ext)
            qs, convs = [], []
            for _ in range(T):
                convs.append(sim.step(1))
                qs.append(sim.get_state()[0])
            runs.append((np.array(qs), np.array(convs)))
            sim.close()
    finally:
        ctx.close()
    (q_ok, c_ok), (q_bad, c_bad) = runs
    assert c_ok.all()
    assert not c_bad[:, 3].any()
    keep = [0, 1, 2, 4, 5]
    assert c_bad[:, keep].all()
    assert np.array_equal(q_bad[:, keep], q_ok[:, keep])


def test_unreachable_tolerance_reports_not_converged(sdfc, oracle):
    fx = load("sim_trans.npz")
    T, tol = 4, 1e-300
    ctx = sdfc.Context(0)
    try:
        sim = make_sim(sdfc, ctx, fx)
        sim.set_tolerance(tol)
        qs, convs = [], []
        for _ in range(T):
            convs.append(bool(sim.step(1)[0]))
            qs.append(sim.get_state()[0][0])
        rounds, _ = sim.stats()
    finally:
        ctx.close()
    og = oracle.Grid(fx["grid"], fx["min_box"], fx["max_box"], fx["dx"], float(fx["col_th"]))
    prm = oracle.Params(*[float(x) for x in fx["params"]])
    mover = oracle.Mover(float(fx["mass"]), fx["inertia"], fx["E_ji"], np.eye(4),
                         tuple(fx["gravity"]), float(fx["h"]), fx["f_ext"], newton_tol=tol)
    pair = oracle.ScenePair(og, fx["points"], True, fx["E_fixed"], prm)
    rq, _, rconv, rits, _ = oracle.bdf1_steps(mover, [pair], fx["q0"], fx["qdot0"], T)
    assert not any(convs) and not rconv.any()
    assert rounds > 20 * T  # each step ran to the stopping rule, not to convergence
    np.testing.assert_allclose(np.array(qs), rq[1:], rtol=0, atol=1e-9)


def test_expired_sweep_waits_are_reported():
    """In a child process (the hook is read per call from the environment): a level set with
    every sweep wait made to run out fails with the library's error, then the same call without
    the hook succeeds in the same context."""
    code = r"""
import sys, importlib, os, numpy as np
sys.path.insert(0, sys.argv[1])
sdfc = importlib.import_module("assemble-them-all_gb300.sdfc")
W = importlib.import_module("assemble-them-all_gb300.workloads")
V, F = W.torus_mesh(0.6, 0.25, 24, 12)
ctx = sdfc.Context(0)
shape, origin, dx = (40, 40, 24), np.array([-1.0, -1.0, -0.4]), 0.05
os.environ["SDFC_TEST_EXPIRE_SWEEP_WAITS"] = "1"
try:
    ctx.make_level_set3(V, F, origin, dx, shape)
    print("NO_ERROR")
except sdfc.SdfcError as e:
    print("ERROR", "timed out" in str(e))
del os.environ["SDFC_TEST_EXPIRE_SWEEP_WAITS"]
phi = ctx.make_level_set3(V, F, origin, dx, shape)
print("AFTER", bool(np.isfinite(phi).all()), float(phi.min()) < 0.0)
np.save(sys.argv[2], phi)
ctx.close()
"""
    out_path = os.path.join(os.environ.get("TMPDIR", "/tmp"), f"ls_after_{os.getpid()}.npy")
    r = subprocess.run([sys.executable, "-c", code, ROOT, out_path], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = r.stdout.split("\n")
    assert "ERROR True" in lines, r.stdout
    assert "AFTER True True" in lines, r.stdout
    from oracle import oracle as O
    W = submodule("workloads")
    V, F = W.torus_mesh(0.6, 0.25, 24, 12)
    want = O.make_level_set3(V, F, np.array([-1.0, -1.0, -0.4]), 0.05, (40, 40, 24))
    assert np.array_equal(np.load(out_path), want)
    os.remove(out_path)
