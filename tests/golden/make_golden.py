"""Generates the golden fixtures of this directory from the reference itself.

Runs the reference redmax simulator, compiled from its sources by
oracle/ref/Makefile (oracle/_ref/libredmax_ref.so), on seeded synthetic inputs
and stores inputs and outputs as compressed .npz files:

  pair_eval.npz   ForceGeneralSDFContact::computeForce / computeForceWithDerivative
                  (simulation/redmax/Force/ForceGeneralSDFContact.cpp:46-105) for a set
                  of poses, velocities and coefficient variants: fm, Km, Dm, active ids
  collision.npz   BodySDFObj::collision with derivatives (simulation/redmax/Body/BodySDFObj.cpp:278-377)
                  at random points

Usage (where the reference sources are present):
    make -C oracle/ref -j8 && python tests/golden/make_golden.py
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
        raise SystemExit("oracle/_ref/libredmax_ref.so missing: build it with make -C oracle/ref")
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


if __name__ == "__main__":
    main()
