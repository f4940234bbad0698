"""Uneven multi-part batches at the configuration's full size: eight seeded procedural
assemblies (2-12 parts each, every part with its own point count and grid), each scene stepped
for 300 BDF1 steps in one sdfc_sim, against the oracle's BDF1 restatement of every scene.

The assemblies are workloads.procedural_assembly(seed) for seeds 0-7, generated as the
configuration's batch generates them (grids sampled on the GPU, FP32 node storage, points drawn
on the GPU); in the first one the pulled part is set to the configuration's largest part, 200k
contact points on a 256^3 grid.  Scene parameters are the planner's (examples/run_joint_plan.py:
147-153, 192-216): h = 1e-3, kn = 1e6, kt = 1e3, mu = 0, damping = 0, gravity 1e-12 along +z,
pull 100 along a random axis, col_th = 0.01 (the parts sit 0.005 apart).  The pulled part is in
contact with every other part both ways (its points against their grids and theirs against its
grid), as the planner declares it.  Bars: q after every step to 1e-9 with FP64 evaluations
(identical convergence flags) and 1e-6 with mixed precision."""
import multiprocessing as mp
import os

import numpy as np
import pytest

from conftest import submodule

pytestmark = pytest.mark.gpu

SEEDS = tuple(range(8))
STEPS = 300
H = float(np.float32(1e-3))
GRAVITY = (0.0, 0.0, 1e-12)
PULL = 100.0
PRM = (1e6, 1e3, 0.0, 0.0, 1.0, 1.0)
COL_TH = 0.01


def assemblies():
    W = submodule("workloads")
    out = []
    for s in SEEDS:
        a = W.procedural_assembly(s)
        if s == SEEDS[0]:  # the configuration's largest part, pulled
            a.n_points[a.mover] = 200000
            a.grid_n[a.mover] = 256
        out.append(a)
    return out


def _oracle_scene(args):
    """One scene stepped by the oracle (runs in a spawned worker)."""
    from oracle import oracle as O
    mover, pairs, steps = args
    grids = {}
    opairs = []
    for (gkey, gv, mn, mx, dx), pts, is_contact, E_fixed in pairs:
        if gkey not in grids:
            grids[gkey] = O.Grid(gv, mn, mx, dx, COL_TH)
        opairs.append(O.ScenePair(grids[gkey], pts, is_contact, E_fixed, O.Params(*PRM)))
    m = O.Mover(*mover)
    qs, _, conv, its, evs = O.bdf1_steps(m, opairs, np.zeros(3), np.zeros(3), steps)
    return qs, conv, its, evs


@pytest.fixture(scope="module")
def c3():
    torch = pytest.importorskip("torch")
    from oracle import oracle as O
    O.build()
    submodule("build").build()
    sdfc = submodule("sdfc")
    S = submodule("scenes")
    asms = assemblies()
    ctx = sdfc.Context(0)
    scenes = [S.AssemblyScene.make_device(ctx, a, seed, col_th=COL_TH) for seed, a in zip(SEEDS, asms)]
    torch.cuda.synchronize()
    big = scenes[0]
    assert big.asm.grid_n[big.asm.mover] == 256 and len(big.points[big.asm.mover]) == 200000
    # the oracle's inputs: the grids exactly as the GPU holds them, the same points
    jobs = []
    for sc in scenes:
        m = sc.asm.mover
        F = np.zeros(6)
        F[3:] = PULL * sc.asm.direction
        mover = (sc.mass, sc.inertia, np.eye(4), sc.placement(m), GRAVITY, H, F)
        pairs = []
        for a, b in sc.contact_pairs():
            h = sc.grid_handles[b]
            gd = ctx._grid_shapes[h]
            still = b if a == m else a
            gkey = b
            gv = ctx.grid_values(h)
            lo, hi, dx = sc.grid_boxes[b]
            assert gv.shape == gd
            pairs.append(((gkey, gv, lo, hi, dx), sc.points[a], a == m, sc.placement(still)))
        jobs.append((mover, pairs, STEPS))
    procs = min(len(jobs), max(1, os.cpu_count() or 1))
    with mp.get_context("spawn").Pool(procs) as pool:
        ref = pool.map(_oracle_scene, jobs, chunksize=1)
    yield sdfc, ctx, scenes, ref
    ctx.close()


@pytest.mark.parametrize("precision,atol", [(0, 1e-9), (1, 1e-6)])
def test_uneven_assemblies_300_steps(c3, precision, atol):
    sdfc, ctx, scenes, ref = c3
    S = submodule("scenes")
    sim = S.build_sim(ctx, scenes, H, GRAVITY, sdfc.Params(*PRM), col_th=COL_TH, storage=sdfc.STORAGE_F32_NODES)
    try:
        sim.set_precision(precision)
        n = len(scenes)
        sim.set_state(np.zeros((n, 3)), np.zeros((n, 3)))
        sim.set_external_force(S.pull_forces(scenes, PULL))
        qs, convs = [], []
        for _ in range(STEPS):
            convs.append(sim.step(1))
            qs.append(sim.get_state()[0])
    finally:
        sim.close()
    qs = np.stack(qs, 1)  # (n, steps, 3)
    blocked = 0
    for i in range(len(scenes)):
        rq, rconv, rits, _ = ref[i]
        err = np.abs(qs[i] - rq[1:]).max()
        assert err <= atol, f"scene {i}: max |q - q_oracle| = {err:.3e} over {STEPS} steps"
        if precision == 0:
            assert np.array_equal(np.array([c[i] for c in convs]), rconv), i
        blocked += int(rits.max() > 2)
    assert blocked >= 2  # pulled parts run into their neighbours within the steps
