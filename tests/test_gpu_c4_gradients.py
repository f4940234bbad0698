"""Adjoint gradients of the differentiable-rollout workload at its full length, against central
differences.

The workload: 4096 pegs on free3d-exp joints in the socket (128^3 FP32 grid, 10k points), initial
pose perturbed (sigma 0.01 translation, sigma 1 degree rotation), pulled along directions in a
30 degree cone about +z, 200 BDF1 steps at h = 5e-3; loss per instance L = sum_t E_t (penetration
energy) + |q_T - target|^2.  Eight instances spread over the 4096 (the bench's seeds) are checked:
dL/dq0 (6) and dL/d(direction) on the tangent plane of the unit sphere at the direction (2),
from sdfc_sim_backward_energy, against central differences with step 1e-6 of rollouts with FP64
evaluations and Newton solved to |g| < 1e-13 (so that the differences resolve the implicit
steps).  Bar: the FP64 adjoint within 1e-4 of the differences (relative to the gradient's norm)
for every sampled instance.  The mixed-precision adjoint (FP32 per-contact algebra, the
reference's Newton tolerance 1e-8) is compared with the same differences and its error is bounded
by 5e-2 (see the design notes for why it is not 1e-4)."""
import numpy as np
import pytest

from conftest import submodule

pytestmark = pytest.mark.gpu

N_ALL, T, EPS, TOL = 4096, 200, 1e-6, 1e-13
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
    """Loss and adjoint gradients (dL/dq0, dL/dF) of every scene of one sim."""
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
        conv = sim.step(T)
        qh = sim.history()
        _, E = sim.energy()
        L = E + ((qh[:, T] - TARGET) ** 2).sum(1)
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
    # per sampled instance: the base scene, then q0 +- eps e_j (j < 6), then d +- eps t_k (k < 2)
    q0s, Fs, bases = [], [], []
    for i in SAMPLE:
        t1, t2 = tangent_basis(d_all[i])
        bases.append((t1, t2))
        variants = [(q0_all[i], d_all[i])]
        for j in range(6):
            for sgn in (1.0, -1.0):
                q = q0_all[i].copy()
                q[j] += sgn * EPS
                variants.append((q, d_all[i]))
        for t in (t1, t2):
            for sgn in (1.0, -1.0):
                variants.append((q0_all[i], d_all[i] + sgn * EPS * t))
        for q, d in variants:
            F = np.zeros(6)
            F[3:] = PULL * d
            q0s.append(q)
            Fs.append(F)
    L, g0, gf, conv = rollout(sdfc, ctx, g, ph, np.array(q0s), np.array(Fs), 0, TOL)
    k = 17
    fd, adj = [], []
    for s, i in enumerate(SAMPLE):
        r = L[s * k:(s + 1) * k]
        t1, t2 = bases[s]
        fd_q = (r[1:13:2] - r[2:13:2]) / (2 * EPS)
        fd_d = (r[13::2] - r[14::2]) / (2 * EPS)  # along t1, t2
        gdir = PULL * gf[s * k, 3:]
        adj.append(np.concatenate([g0[s * k], [gdir @ t1, gdir @ t2]]))
        fd.append(np.concatenate([fd_q, fd_d]))
    # the mixed-precision adjoint of the same base scenes at the reference's tolerance
    base_q = np.array([q0_all[i] for i in SAMPLE])
    base_F = np.zeros((len(SAMPLE), 6))
    base_F[:, 3:] = PULL * d_all[list(SAMPLE)]
    _, g0m, gfm, _ = rollout(sdfc, ctx, g, ph, base_q, base_F, 1)
    mixed = [np.concatenate([g0m[s], [PULL * gfm[s, 3:] @ bases[s][0], PULL * gfm[s, 3:] @ bases[s][1]]])
             for s in range(len(SAMPLE))]
    yield np.array(adj), np.array(fd), np.array(mixed), conv[::k]
    ctx.close()


def test_fp64_adjoint_matches_central_differences(c4):
    adj, fd, _, conv = c4
    assert conv.all()
    rel = np.linalg.norm(adj - fd, axis=1) / np.linalg.norm(adj, axis=1)
    assert np.linalg.norm(adj, axis=1).min() > 0
    assert rel.max() <= 1e-4, f"relative errors per sampled instance: {rel}"


def test_mixed_adjoint_error_bound(c4):
    _, fd, mixed, _ = c4
    rel = np.linalg.norm(mixed - fd, axis=1) / np.linalg.norm(fd, axis=1)
    assert rel.max() <= 5e-2, f"relative errors per sampled instance: {rel}"
