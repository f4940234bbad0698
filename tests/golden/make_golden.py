"""Generates the golden fixtures of this directory from the reference itself.

Runs the reference redmax simulator, compiled from its sources by
oracle/ref/Makefile (oracle/_ref/libredmax_ref.so), on seeded synthetic inputs
and stores inputs and outputs as compressed .npz files:

  pair_eval.npz   ForceGeneralSDFContact::computeForce / computeForceWithDerivative
                  (simulation/redmax/Force/ForceGeneralSDFContact.cpp:46-105) for a set
                  of poses, velocities and coefficient variants: fm, Km, Dm, active ids
  collision.npz   BodySDFObj::collision with derivatives (simulation/redmax/Body/BodySDFObj.cpp:278-377)
                  at random points
  sim_trans.npz / sim_free.npz
                  Simulation::forward with BDF1 (simulation/redmax/Simulation.cpp:914-1079, 1248-1270)
                  of a peg on a translational joint against a fixed socket: the scene and the
                  reference's joint trajectory and Newton convergence flags

Usage (where the reference sources are present):
    make -C oracle/ref REF=<reference root> -j8 && python tests/golden/make_golden.py
"""
import importlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import refsim  # noqa: E402

W = importlib.import_module("assemble-them-all_gb300.workloads")

GRID_N = 24
N_POINTS = 1500
COL_TH = 0.01


def cases(rng):
    """(E_A, phi_A, E_B, phi_B, kn, kt, mu, damping, scale, contact_scale) variants."""
    out = []
    variants = [
        (1e5, 1e3, 0.0, 1e3, 1.0, 1.0),   # no friction
        (1e5, 1e3, 0.3, 1e3, 1.0, 1.0),   # planner-like, mostly static friction
        (1e5, 1e1, 0.3, 1e3, 1.0, 1.0),   # weak kt -> dynamic friction
        (1e6, 1e3, 0.0, 0.0, 1.0, 1.0),   # planner default (run_joint_plan.py:153)
        (1e5, 1e3, 0.5, 1e3, 0.5, 2.0),   # scaled stiffness
    ]
    for k in range(15):
        kn, kt, mu, kd, sc, cs = variants[k % len(variants)]
        R = W.rotvec_to_matrix(rng.normal(size=3) * 0.02)
        p = np.array([0.03 * rng.normal(), 0.03 * rng.normal(), 0.3 * rng.normal()])
        EA = W.pose(R, p)
        if k % 3 == 2:
            EB = W.pose(W.rotvec_to_matrix(rng.normal(size=3) * 0.05), rng.normal(size=3) * 0.01)
        else:
            EB = np.eye(4)
        phiA = rng.normal(size=6) * 0.5
        phiB = np.zeros(6) if k % 2 == 0 else rng.normal(size=6) * 0.1
        out.append((EA, phiA, EB, phiB, kn, kt, mu, kd, sc, cs))
    return out


def main():
    if not refsim.available():
        raise SystemExit("oracle/_ref/libredmax_ref.so missing: build it with make -C oracle/ref REF=<reference root>")
    rng = np.random.default_rng(20261203)
    grid = W.socket_grid(GRID_N, dtype=np.float32)
    pts = W.peg_points(N_POINTS, seed=7)
    sim, _ = refsim.make_pair_sim()
    sim.set_sdf("B", grid.values, grid.min_box, grid.max_box, grid.dx, COL_TH)
    sim.set_contact_points("A", pts)

    rows = {k: [] for k in ("EA", "phiA", "EB", "phiB", "params", "fm_v", "fm", "Km", "Dm", "ids", "n_active")}
    for (EA, phiA, EB, phiB, kn, kt, mu, kd, sc, cs) in cases(rng):
        sim.set_pose("A", EA, phiA)
        sim.set_pose("B", EB, phiB)
        sim.set_contact_scale("A", cs)
        fm_v, _, _, ids_v = sim.pair_eval("A", "B", kn, kt, mu, kd, sc, want_deriv=False)
        fm, Km, Dm, ids = sim.pair_eval("A", "B", kn, kt, mu, kd, sc, want_deriv=True)
        assert np.array_equal(ids, ids_v)
        rows["EA"].append(EA)
        rows["phiA"].append(phiA)
        rows["EB"].append(EB)
        rows["phiB"].append(phiB)
        rows["params"].append([kn, kt, mu, kd, sc, cs])
        rows["fm_v"].append(fm_v)
        rows["fm"].append(fm)
        rows["Km"].append(Km)
        rows["Dm"].append(Dm)
        rows["ids"].append(np.pad(ids, (0, N_POINTS - len(ids)), constant_values=-1))
        rows["n_active"].append(len(ids))
    np.savez_compressed(os.path.join(HERE, "pair_eval.npz"), grid=grid.values, min_box=grid.min_box,
                        max_box=grid.max_box, dx=grid.dx, col_th=COL_TH, points=pts,
                        **{k: np.array(v) for k, v in rows.items()})

    # collision() at random points near the socket surfaces, random body-B pose/velocity
    q = []
    for k in range(200):
        xw = rng.uniform(-1.05, 1.05, 3)
        xwd = rng.normal(size=3)
        EB = W.pose(W.rotvec_to_matrix(rng.normal(size=3) * 0.3), rng.normal(size=3) * 0.02)
        phiB = rng.normal(size=6)
        sim.set_pose("B", EB, phiB)
        out = sim.collision("B", xw, xwd, want_deriv=True)
        q.append((xw, xwd, EB, phiB, out))
    np.savez_compressed(os.path.join(HERE, "collision.npz"), grid=grid.values, min_box=grid.min_box,
                        max_box=grid.max_box, dx=grid.dx, col_th=COL_TH,
                        xw=np.array([a[0] for a in q]), xw_dot=np.array([a[1] for a in q]),
                        EB=np.array([a[2] for a in q]), phiB=np.array([a[3] for a in q]),
                        out=np.array([a[4] for a in q]))
    print("active counts:", rows["n_active"])


def f32(x):
    return float(np.float32(x))


SIM_CASES = {
    # name: joint, q0, qdot0, external force (torque then force), steps
    "sim_trans": ("translational", [0.012, 0.0, 0.0], [0.5, 0.0, -0.2], [0.0, 0.0, 0.0, 2.0, 0.5, 1.0], 40),
    "sim_free": ("free3d-exp", [0.012, 0.0, 0.0, 0.002, -0.003, 0.01], [0.5, 0.0, -0.2, 0.3, -0.1, 0.5],
                 [0.05, -0.1, 0.02, 2.0, 0.5, 1.0], 40),
}


def make_sim_fixture(name="sim_trans"):
    """A peg (box mesh for its mass properties, peg points as its contact points) on a
    translational or free3d-exp joint, pushed into a fixed socket; both scene files use the
    planner's layout."""
    joint, q0, qd0, F, steps = SIM_CASES[name]
    import tempfile
    wd = tempfile.mkdtemp(prefix="golden_sim_")
    Va, Fa = refsim.box_mesh((0.3, 0.25, 0.9))
    Vb, Fb = refsim.box_mesh((1.0, 1.0, 1.0))
    refsim.write_obj(os.path.join(wd, "a.obj"), Va, Fa)
    refsim.write_obj(os.path.join(wd, "b.obj"), Vb, Fb)
    kn, kt, mu, kd, h, gravity = 1e5, 1e3, 0.3, 1e3, 5e-3, (0.0, 0.0, -9.8)
    xml = refsim.two_body_xml("a.obj", "b.obj", joint_a=joint, kn=kn, kt=kt, mu=mu, damping=kd,
                              timestep=h, gravity=gravity, col_th=COL_TH)
    sim = refsim.RefSim(xml, wd)
    mA, IA, EjiA, E0iA = sim.mass_props("A")
    _, _, _, E0iB = sim.mass_props("B")
    grid = W.socket_grid(48, dtype=np.float32)
    mn, mx, dx = grid.min_box, grid.max_box, grid.dx
    n = grid.values.shape[0]
    ax = [mn[a] + dx[a] * np.arange(n) for a in range(3)]
    Z, Y, X = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    world = np.stack([X, Y, Z], -1) @ E0iB[:3, :3].T + E0iB[:3, 3]  # grid nodes are in B's body frame
    vals = W.socket_sdf(world).astype(np.float32).astype(np.float64)
    sim.set_sdf("B", vals, mn, mx, dx, COL_TH)
    pw = W.peg_points(3000, seed=2)
    pts = (pw - E0iA[:3, 3]) @ E0iA[:3, :3]  # into A's body frame at q = 0
    sim.set_contact_points("A", pts)
    q0, qd0, F = np.array(q0), np.array(qd0), np.array(F)
    n = len(q0)
    sim.set_state_init(q0, qd0)
    sim.reset(False)
    sim.set_external_force("A", F)
    qs, qds, conv = [q0], [qd0], []
    for _ in range(steps):
        sim.forward(1)
        q, qd = sim.state()
        qs.append(q)
        qds.append(qd)
        conv.append(sim.is_converged())
    # the reference's adjoint (Simulation::backward_BDF1, Simulation.cpp:1559-1634) of a loss whose
    # gradient with respect to every q_k is a seeded random vector
    T_bw = 20
    df_dq = np.random.default_rng(99).normal(size=(T_bw, n))
    sim.set_state_init(q0, qd0)
    sim.reset(True)
    sim.set_external_force("A", F)
    sim.forward(T_bw)
    df_dq0, df_dqdot0 = sim.backward(df_dq.ravel(), T_bw)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), grid=vals, min_box=mn, max_box=mx, dx=dx,
                        col_th=COL_TH, points=pts, mass=mA, inertia=IA, E_ji=EjiA, E_fixed=E0iB,
                        params=np.array([f32(kn), f32(kt), f32(mu), f32(kd), 1.0, 1.0]), h=f32(h),
                        gravity=np.array(gravity), f_ext=F, q0=q0, qdot0=qd0, q=np.array(qs), qdot=np.array(qds),
                        converged=np.array(conv), bw_steps=T_bw, bw_df_dq=df_dq, bw_df_dq0=df_dq0,
                        bw_df_dqdot0=df_dqdot0)
    print("reference adjoint: df_dq0", df_dq0, "df_dqdot0", df_dqdot0)
    print("sim trajectory: final q", qs[-1], "all converged", all(conv))


if __name__ == "__main__":
    main()
    for name in SIM_CASES:
        make_sim_fixture(name)
