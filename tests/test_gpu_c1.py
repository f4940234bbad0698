"""The plain peg-in-hole rollout at full length: socket = cube [-1, 1]^3 minus a z bore of radius
0.5 on a 64^3 FP64 grid (bbox padded 10%), peg = cylinder r 0.49, length 2, fully inserted, 10k
seeded surface points, pulled with 1.0 along +z (scaled by the mass) against gravity 9.8,
2000 BDF1 steps at dt = 5e-3 (FP32-rounded like the reference's XML), kn 1e5, kd 1e3, mu 0.3,
kt 1e3.  The peg starts 0.021 off-axis (0.001 past the bore wall plus col_th 0.01) so it rubs the wall before it drops out.

GPU (FP64 storage, FP64 evaluations) against the oracle's BDF1 restatement, every 50 steps:
1e-8 in q; the mixed-precision path to 1e-5."""
import numpy as np
import pytest

from conftest import submodule

pytestmark = pytest.mark.gpu

STEPS = 2000
H = float(np.float32(5e-3))
PRM = (1e5, 1e3, 0.3, 1e3, 1.0, 1.0)


@pytest.fixture(scope="module")
def scene():
    W = submodule("workloads")
    g = W.socket_grid(64, dtype=np.float64)
    pts = W.peg_points(10000, seed=1)
    m, inertia = W.cylinder_mass_props()
    return g, pts, m, inertia


@pytest.fixture(scope="module")
def reference(oracle, scene):
    g, pts, m, inertia = scene
    grid = oracle.Grid(g.values, g.min_box, g.max_box, g.dx, 0.01)
    F = np.array([0, 0, 0, 0, 0, 1.0])
    mover = oracle.Mover(m, inertia, np.eye(4), np.eye(4), (0.0, 0.0, -9.8), H, F)
    pair = oracle.ScenePair(grid, pts, True, np.eye(4), oracle.Params(*PRM))
    return oracle.bdf1_steps(mover, [pair], np.array([0.021, 0.0, 0.0]), np.zeros(3), STEPS)


@pytest.mark.parametrize("precision,atol", [(0, 1e-8), (1, 1e-5)])
def test_c1_rollout(scene, reference, precision, atol):
    sdfc = submodule("sdfc")
    submodule("build").build()
    g, pts, m, inertia = scene
    rq, _, rconv, rits, _ = reference
    assert rits[:40].max() > 2  # the wall contact is exercised
    ctx = sdfc.Context(0)
    try:
        gh = ctx.upload_grid(g.values, g.min_box, g.max_box, g.dx, 0.01, sdfc.STORAGE_F64)
        ph = ctx.upload_points(pts, sdfc.STORAGE_F32)
        mv = sdfc.Mover.make(m, inertia, np.eye(4), H, (0.0, 0.0, -9.8))
        sim = ctx.sim([mv], [sdfc.ScenePair.make(0, ph, gh, True, np.eye(4), sdfc.Params(*PRM))])
        sim.set_precision(precision)
        sim.set_state(np.array([[0.021, 0.0, 0.0]]), np.zeros((1, 3)))
        sim.set_external_force(np.array([[0, 0, 0, 0, 0, 1.0]]))
        for t in range(50, STEPS + 1, 50):
            conv = sim.step(50)
            q, _ = sim.get_state()
            np.testing.assert_allclose(q[0], rq[t], rtol=0, atol=atol * max(1.0, np.abs(rq[t]).max()),
                                       err_msg=f"step {t}")
        if precision == 0:
            assert bool(conv[0]) == bool(rconv[-1])
    finally:
        ctx.close()
