"""ORACLE — test infrastructure, not the product.

The planner's disassembly check, PhysicsPlanner.is_disassembled
(examples/run_joint_plan.py:291-302), restated with exact convex geometry so that the GPU
version can be checked where the reference's own path cannot run: it needs trimesh 3.10.8 and
python-fcl 0.6.1 (FCL 0.6.1), which this environment does not have.

The reference collides the two convex hulls' triangle surfaces with FCL (touching counts) and,
when they do not meet, calls the part disassembled unless one hull's axis-aligned box contains
the other's.  For convex hulls the surfaces meet exactly when the solids share a point and
neither solid lies inside the other.  Here:

  * solids share a point: the linear program "convex combinations of both vertex sets coincide"
    is feasible (scipy.optimize.linprog, HiGHS);
  * containment: every vertex of one hull satisfies every facet inequality of the other
    (qhull's planes n . x + offset <= 0, tolerance 1e-12);
  * boxes: the vertex bounds, as the reference compares them.

Only tests/ use this module, as the checker, and only on poses whose hulls are kept clear of
touching (the reference's own answer there depends on FCL's tolerances).
"""
from __future__ import annotations

import numpy as np
from scipy.optimize import linprog
from scipy.spatial import ConvexHull


def hull_of(points):
    pts = np.asarray(points, dtype=np.float64).reshape(-1, 3)
    h = ConvexHull(pts)
    return pts[h.vertices], h.equations


def pose_points(E, V):
    E = np.asarray(E, dtype=np.float64)
    return V @ E[:3, :3].T + E[:3, 3]


def solids_meet(VA, VB) -> bool:
    na, nb = len(VA), len(VB)
    A_eq = np.zeros((5, na + nb))
    A_eq[:3, :na] = VA.T
    A_eq[:3, na:] = -VB.T
    A_eq[3, :na] = 1.0
    A_eq[4, na:] = 1.0
    b_eq = np.array([0.0, 0.0, 0.0, 1.0, 1.0])
    r = linprog(np.zeros(na + nb), A_eq=A_eq, b_eq=b_eq, bounds=(0, None), method="highs")
    return r.status == 0


def inside(V, planes, tol=1e-12) -> bool:
    return bool(np.all(V @ planes[:, :3].T + planes[:, 3] <= tol))


class Checker:
    """The reference's predicate for a moving part (vertices in its body frame) against the still
    parts' vertices (world), hulls built once as the planner builds them (:225-228)."""

    def __init__(self, vertices_move, vertices_still):
        self.VA0, self.PA = hull_of(vertices_move)
        self.VB, self.PB = hull_of(vertices_still)
        self.blo, self.bhi = self.VB.min(0), self.VB.max(0)

    def __call__(self, E) -> bool:
        E = np.asarray(E, dtype=np.float64)
        VA = pose_points(E, self.VA0)
        # the moving hull's planes in world: n' = R n, o' = o - n' . p
        nA = self.PA[:, :3] @ E[:3, :3].T
        PAw = np.c_[nA, self.PA[:, 3] - nA @ E[:3, 3]]
        surfaces = solids_meet(VA, self.VB) and not inside(VA, self.PB) and not inside(self.VB, PAw)
        lo, hi = VA.min(0), VA.max(0)
        move_contains = bool(np.all(lo <= self.blo) and np.all(hi >= self.bhi))
        still_contains = bool(np.all(self.blo <= lo) and np.all(self.bhi >= hi))
        return (not surfaces) and not (move_contains or still_contains)


def is_disassembled(vertices_move, vertices_still, E) -> bool:
    """One pose E of the moving part (vertices in its body frame) against the still parts'
    vertices (world)."""
    return Checker(vertices_move, vertices_still)(E)
