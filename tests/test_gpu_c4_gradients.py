"""Adjoint gradients of the differentiable-rollout workload at its full length, against central
differences.

The workload: 4096 pegs on free3d-exp joints in the socket (128^3 FP32 grid, 10k points), initial
pose perturbed (sigma 0.01 translation, sigma 1 degree rotation), pulled along directions in a
30 degree cone about +z, 200 BDF1 steps at h = 5e-3; loss per instance L = sum_t E_t (penetration
energy) + |q_T - target|^2.  Eight instances spread over the 4096 (the bench's seeds) are checked:
dL/dq0 (6) and dL/d(direction) on the tangent plane of the unit sphere at the direction (2),
from sdfc_sim_backward_energy, against central differences of rollouts with FP64 evaluations
and Newton solved to |g| < 1e-13, at steps 1e-6, 1e-8 and 3e-9.

This loss is piecewise smooth: over 200 steps thousands of contact points enter and leave the
active set, and each entry is a kink of the rollout (the contact force is continuous in the
depth, its derivative is not).  At the workload's stated step 1e-6 the +- rollouts straddle such
kinks, so those differences are not the derivative; they converge to the adjoint as the step
shrinks (at 1e-8 they agree with it to about 1e-7, the tolerance-limited noise of the
differences).  Even at 1e-8 a component's +- rollouts can straddle a kink; such a component's
differences at 1e-8 and 3e-9 disagree, which the test uses to recognise it.  A kink at the base
point itself makes both central differences the mean of the two one-sided slopes, so they agree
while the adjoint takes one side: the one-sided slopes then differ by the slope jump at both
1e-8 and 3e-9 (curvature makes that gap shrink with the step), which the test uses too.  An instance with a step whose Newton iteration stops without converging (the reference's three line-search
strikes) has a non-differentiable loss and is not checked; nor is one whose rotation vector is
reparameterised between steps (the adjoint, like the reference's, does not differentiate that
map).

Bars, over the sampled instances whose base and fine-step rollouts converged at every step (at
least five of the eight): every component whose differences at 1e-8 and 3e-9 agree to 1e-5 of the
gradient's norm and that shows no kink at the base point (at least 85% of them) has the FP64
adjoint within 1e-4 of the gradient's norm of its 1e-8 difference; the mixed-precision adjoint (FP32 per-contact algebra, the reference's Newton
tolerance 1e-8) is within 1e-2 of the FP64 adjoint, relative to its norm."""
import numpy as np
import pytest

from conftest import submodule

pytestmark = pytest.mark.gpu

N_ALL, T, TOL = 4096, 200, 1e-13
STEPS = (1e-6, 1e-8, 3e-9)  # the workload's stated difference step, and two in the differentiable regime
SAMPLE = tuple(range(0, N_ALL, N_ALL // 8))
H = float(np.float32(5e-3))
GRAVITY = (0.0, 0.0, -9.8)
PARAMS = (1e5, 1e3, 0.3, 1e3, 1.0, 1.0)
PULL = 1.0
TARGET = np.array([0.0, 0.0, 0.25, 0.0, 0.0, 0.0])


def workload(W):
    """The rollout's initial poses and pull directions (bench.py's run_c4 seeds)."""
    rng = np.random.default_rng(4)
    q0 = np.zeros((N_ALL, 6))
    q0[:, :3] = rng.normal(size=(N_ALL, 3)) * 0.01
    q0[:, 3:] = rng.normal(size=(N_ALL, 3)) * np.deg2rad(1.0)
    return q0, W.cone_directions(N_ALL, 30.0, seed=4)


def tangent_basis(d):
    a = np.array([1.0, 0.0, 0.0]) if abs(d[0]) < 0.9 else np.array([0.0, 1.0, 0.0])
    t1 = np.cross(d, a)
    t1 /= np.linalg.norm(t1)
    return t1, np.cross(d, t1)


def rollout(sdfc, ctx, g, ph, q0, F, precision, tol=None):
    """Loss, adjoint gradients (dL/dq0, dL/dF) and whether every step converged, for every scene
    of one sim."""
    W = submodule("workloads")
    n = len(q0)
    m, inertia = W.cylinder_mass_props()
    mv = sdfc.Mover.make(m, inertia, np.eye(4), H, GRAVITY, joint=sdfc.JOINT_FREE3D_EXP)
    sim = ctx.sim([mv] * n, [sdfc.ScenePair.make(i, ph, g, True, np.eye(4), sdfc.Params(*PARAMS)) for i in range(n)])
    try:
        sim.set_precision(precision)
        if tol is not None:
            sim.set_tolerance(tol)
        sim.record_energy(True)
        sim.set_state(q0, np.zeros((n, 6)))
        sim.set_external_force(F)
        sim.record(T)
        conv = np.ones(n, bool)
        for _ in range(T):
            conv &= sim.step(1)
        qh = sim.history()
        _, E = sim.energy()
        L = E + ((qh[:, T] - TARGET) ** 2).sum(1)
        # a rotation vector reparameterised between steps (a jump of about 2 pi): the adjoint,
        # like the reference's, does not differentiate that map
        conv &= ~(np.linalg.norm(np.diff(qh[:, :, 3:6], axis=1), axis=2) > np.pi).any(axis=1)
        df_dq = np.zeros((n, T, 6))
        df_dq[:, T - 1] = 2.0 * (qh[:, T] - TARGET)
        g0, _, gf = sim.backward(df_dq, np.ones(n))
    finally:
        sim.close()
    return L, g0, gf, conv


@pytest.fixture(scope="module")
def c4():
    submodule("build").build()
    sdfc = submodule("sdfc")
    W = submodule("workloads")
    q0_all, d_all = workload(W)
    grid = W.socket_grid(128, dtype=np.float32)
    pts = W.peg_points(10000, seed=9)
    ctx = sdfc.Context(0)
    g = ctx.upload_grid(grid.values, grid.min_box, grid.max_box, grid.dx, 0.01, sdfc.STORAGE_F32)
    ph = ctx.upload_points(pts, sdfc.STORAGE_F32)
    # per sampled instance: the base scene, then per difference step q0 +- h e_j (j < 6) and
    # d +- h t_k (k < 2)
    q0s, Fs, bases = [], [], []
    for i in SAMPLE:
        t1, t2 = tangent_basis(d_all[i])
        bases.append((t1, t2))
        variants = [(q0_all[i], d_all[i])]
        for h in STEPS:
            for j in range(6):
                for sgn in (1.0, -1.0):
                    q = q0_all[i].copy()
                    q[j] += sgn * h
                    variants.append((q, d_all[i]))
            for t in (t1, t2):
                for sgn in (1.0, -1.0):
                    variants.append((q0_all[i], d_all[i] + sgn * h * t))
        for q, d in variants:
            F = np.zeros(6)
            F[3:] = PULL * d
            q0s.append(q)
            Fs.append(F)
    L, g0, gf, conv = rollout(sdfc, ctx, g, ph, np.array(q0s), np.array(Fs), 0, TOL)
    k = 1 + 16 * len(STEPS)
    res = []
    for s_, i in enumerate(SAMPLE):
        o = s_ * k
        t1, t2 = bases[s_]
        gdir = PULL * gf[o, 3:]
        adj = np.concatenate([g0[o], [gdir @ t1, gdir @ t2]])
        fds, ok = {}, {}
        for m, h in enumerate(STEPS):
            r = L[o + 1 + 16 * m:o + 1 + 16 * (m + 1)]
            fds[h] = (r[0::2] - r[1::2]) / (2 * h)
            ok[h] = bool(conv[o] and conv[o + 1 + 16 * m:o + 1 + 16 * (m + 1)].all())
        # the gap between the one-sided slopes at 1e-8 and at 3e-9: curvature makes it shrink with
        # the step, a kink at the base point keeps it (the slope jump)
        gap = {}
        for m in (1, 2):
            r = L[o + 1 + 16 * m:o + 1 + 16 * (m + 1)]
            gap[m] = np.abs((r[0::2] - L[o]) - (L[o] - r[1::2])) / STEPS[m]
        res.append({"instance": i, "adj": adj, "fd": fds, "converged": ok, "gap8": gap[1], "gap3": gap[2]})
    # the mixed-precision adjoint of the same base scenes at the reference's tolerance
    base_q = np.array([q0_all[i] for i in SAMPLE])
    base_F = np.zeros((len(SAMPLE), 6))
    base_F[:, 3:] = PULL * d_all[list(SAMPLE)]
    _, g0m, gfm, _ = rollout(sdfc, ctx, g, ph, base_q, base_F, 1)
    for s_, r in enumerate(res):
        t1, t2 = bases[s_]
        gm = PULL * gfm[s_, 3:]
        r["mixed"] = np.concatenate([g0m[s_], [gm @ t1, gm @ t2]])
    yield res
    ctx.close()


def _checked(c4):
    """Instances whose base and fine-step rollouts converged at every step."""
    return [r for r in c4 if r["converged"][STEPS[1]] and r["converged"][STEPS[2]]]


def test_fp64_adjoint_matches_central_differences(c4):
    checked = _checked(c4)
    assert len(checked) >= 5, [r["instance"] for r in c4 if r not in checked]
    smooth_total = 0
    for r in checked:
        scale = np.linalg.norm(r["fd"][STEPS[1]])
        kink_at_base = (r["gap8"] > 1e-5 * scale) & (r["gap3"] > 0.6 * r["gap8"])
        smooth = (np.abs(r["fd"][STEPS[1]] - r["fd"][STEPS[2]]) <= 1e-5 * scale) & ~kink_at_base
        smooth_total += int(smooth.sum())
        err = np.abs(r["adj"] - r["fd"][STEPS[1]])[smooth] / scale
        assert (err <= 1e-4).all(), (r["instance"], err, r["adj"], r["fd"][STEPS[1]])
    assert smooth_total >= 0.85 * 8 * len(checked), smooth_total


def test_mixed_adjoint_against_fp64_adjoint(c4):
    for r in _checked(c4):
        rel = np.linalg.norm(r["mixed"] - r["adj"]) / np.linalg.norm(r["adj"])
        assert rel <= 1e-2, (r["instance"], rel)
