"""Pins the oracle restatement against the reference itself, run here.

Skipped where the reference build (oracle/_ref/libredmax_ref.so, made by
oracle/ref/Makefile from the reference sources) is absent."""
import numpy as np
import pytest

from _helpers import assert_close
from oracle import refsim

pytestmark = pytest.mark.skipif(not refsim.available(), reason="reference build not present")


@pytest.fixture(scope="module")
def scene(workloads):
    grid = workloads.socket_grid(32, dtype=np.float64)
    pts = workloads.peg_points(4000, seed=3)
    sim, _ = refsim.make_pair_sim()
    sim.set_sdf("B", grid.values, grid.min_box, grid.max_box, grid.dx, 0.01)
    sim.set_contact_points("A", pts)
    return sim, grid, pts


def test_pair_eval_random(oracle, workloads, scene):
    sim, grid, pts = scene
    g = oracle.Grid(grid.values, grid.min_box, grid.max_box, grid.dx, 0.01)
    rng = np.random.default_rng(11)
    seen_dynamic = seen_static = False
    for k in range(24):
        EA = workloads.pose(workloads.rotvec_to_matrix(rng.normal(size=3) * 0.02),
                            [0.03 * rng.normal(), 0.03 * rng.normal(), 0.3 * rng.normal()])
        EB = workloads.pose(workloads.rotvec_to_matrix(rng.normal(size=3) * 0.05), rng.normal(size=3) * 0.01)
        phiA, phiB = rng.normal(size=6) * 0.5, rng.normal(size=6) * 0.1
        kt = [1e3, 1e1, 1e5][k % 3]
        prm = oracle.Params(1e5, kt, 0.3, 1e3, 1.0, 1.0)
        sim.set_pose("A", EA, phiA)
        sim.set_pose("B", EB, phiB)
        for deriv in (False, True):
            fa, Ka, Da, ia = sim.pair_eval("A", "B", prm.kn, prm.kt, prm.mu, prm.damping, 1.0, deriv)
            fb, Kb, Db, ib = oracle.pair_eval(g, pts, EA, phiA, EB, phiB, prm, deriv)
            assert np.array_equal(ia, ib)
            assert_close("fm", fb, fa, rel=1e-12)
            if deriv:
                assert_close("Km", Kb, Ka, rel=1e-12)
                assert_close("Dm", Db, Da, rel=1e-12)
        seen_dynamic |= kt == 1e1
        seen_static |= kt == 1e5
    assert seen_dynamic and seen_static


def test_collision_random(oracle, workloads, scene):
    sim, grid, _ = scene
    g = oracle.Grid(grid.values, grid.min_box, grid.max_box, grid.dx, 0.01)
    rng = np.random.default_rng(5)
    for k in range(200):
        xw, xwd = rng.uniform(-1.15, 1.15, 3), rng.normal(size=3)
        EB = workloads.pose(workloads.rotvec_to_matrix(rng.normal(size=3) * 0.3), rng.normal(size=3) * 0.02)
        phiB = rng.normal(size=6)
        sim.set_pose("B", EB, phiB)
        a = sim.collision("B", xw, xwd)
        b = oracle.collision(g, EB, phiB, xw, xwd)
        assert_close("value", b[:11], a[:11], rel=1e-11)
        assert_close("derivatives", b[11:], a[11:], rel=1e-9, abs_=1e-9)


def test_distance_outside_box(oracle, workloads, scene):
    """Outside the grid box distance() is FLT_MAX + col_th (BodySDFObj.cpp:169-170)."""
    sim, grid, _ = scene
    g = oracle.Grid(grid.values, grid.min_box, grid.max_box, grid.dx, 0.01)
    sim.set_pose("B", np.eye(4), np.zeros(6))
    pts = np.array([[5.0, 0, 0], [0, -3.0, 0], [0.2, 0.1, 0.0], [1.1, 1.1, 1.1]])
    ref = sim.distance("B", pts)
    ours = np.array([oracle.distance(g, np.eye(4), p) for p in pts])
    assert np.array_equal(ref, ours)
