"""Uneven multi-part batches: procedural interlocked assemblies (2-12 parts, uneven point
counts and grid sizes per part, one pulled part per assembly), all scenes stepped by one
sdfc_sim, against the oracle's BDF1 restatement of each scene.

Each scene holds the pulled part against every still part in both directions, as the
reference's planner declares it.  Bars: FP64 evaluations 1e-9 in q after every step (Newton
stops at |g| < 1e-8), mixed precision 1e-6, with identical convergence flags (FP64)."""
import numpy as np
import pytest

from conftest import submodule

pytestmark = pytest.mark.gpu

H = float(np.float32(1e-3))
GRAVITY = (0.0, 0.0, 1e-12)
PULL = 100.0
PRM = (1e6, 1e3, 0.3, 1e2, 1.0, 1.0)
STEPS = 25


@pytest.fixture(scope="module")
def sdfc():
    submodule("build").build()
    return submodule("sdfc")


@pytest.fixture(scope="module")
def scenes():
    W = submodule("workloads")
    S = submodule("scenes")
    out = []
    for seed in range(4):
        asm = W.procedural_assembly(seed, points=(2000, 12000), grids=(48, 64, 96))
        out.append(S.AssemblyScene.make(asm, seed))
    return out


@pytest.fixture(scope="module")
def reference(oracle, scenes):
    return [oracle_trajectory(oracle, sc, STEPS) for sc in scenes]


def oracle_trajectory(oracle, sc, steps):
    grids = [oracle.Grid(g.values, g.min_box, g.max_box, g.dx, 0.0) for g in sc.grids]
    m = sc.asm.mover
    prm = oracle.Params(*PRM)
    pairs = []
    for a, b in sc.contact_pairs():
        still = b if a == m else a
        pairs.append(oracle.ScenePair(grids[b], sc.points[a], a == m, sc.placement(still), prm))
    F = np.zeros(6)
    F[3:] = PULL * sc.asm.direction
    mover = oracle.Mover(sc.mass, sc.inertia, np.eye(4), sc.placement(m), GRAVITY, H, F)
    return oracle.bdf1_steps(mover, pairs, np.zeros(3), np.zeros(3), steps)


@pytest.mark.parametrize("precision,atol", [(0, 1e-9), (1, 1e-6)])
def test_assemblies_against_oracle(sdfc, scenes, reference, precision, atol):
    S = submodule("scenes")
    ctx = sdfc.Context(0)
    try:
        sim = S.build_sim(ctx, scenes, H, GRAVITY, sdfc.Params(*PRM))
        sim.set_precision(precision)
        n = len(scenes)
        sim.set_state(np.zeros((n, 3)), np.zeros((n, 3)))
        sim.set_external_force(S.pull_forces(scenes, PULL))
        qs, convs = [], []
        for _ in range(STEPS):
            convs.append(sim.step(1))
            qs.append(sim.get_state()[0])
    finally:
        ctx.close()
    qs = np.stack(qs, 1)  # (n, steps, 3)
    blocked = 0
    for i, sc in enumerate(scenes):
        rq, _, rconv, rits, _ = reference[i]
        np.testing.assert_allclose(qs[i], rq[1:], rtol=0, atol=atol, err_msg=f"scene {i}")
        if precision == 0:
            assert np.array_equal(np.array([c[i] for c in convs]), rconv), i
        blocked += int(rits.max() > 2)
    assert blocked > 0  # some pulled parts run into their neighbours within the steps
