"""Mesh distance queries of the planner side, on the GPU.

``SDFMesh`` mirrors redmax's ``SDFMesh`` (simulation/redmax/Mesh.h:29-47, Mesh.cpp:41-198,
bound to Python in simulation/redmax/python_interface.cpp:283-292): same constructor
arguments, ``vertices`` / ``faces`` (3 x n, as the reference stores them), ``distance(X)`` and
``min_distance(X)`` for X (3 x n) in the mesh's frame, ``clear_saved_sdf()``.  The grid is built
on the GPU (``sdfc_make_level_set3``, bit-identical to the reference's), loaded from or saved to
the reference's .sdf text cache, and every distance is the reference's FP64 value.

``body_distance`` / ``body_in_contact`` restate Simulation::get_body_distance and
body_in_contact (simulation/redmax/Simulation.cpp:276-303) for many poses at once:
one batched launch set per call.
"""
from __future__ import annotations

import os

import numpy as np

from . import sdfc

_SDFMESH_RES = 20  # SDFMesh::precompute_SDF's min_size (rm/Mesh.cpp:75)
_default_ctx = None


def default_context() -> "sdfc.Context":
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = sdfc.Context(0)
    return _default_ctx


class SDFMesh:
    def __init__(self, V, F, dx, load_path: str = "", save_path: str = "", ctx=None):
        self.ctx = ctx or default_context()
        self.vertices = np.array(V, dtype=np.float64).reshape(3, -1)
        self.faces = np.array(F, dtype=np.int32).reshape(3, -1)
        self._sdf_path = ""
        grid = None
        if load_path:
            self._sdf_path = load_path
            grid = sdfc.load_sdf_text(load_path)
        if grid is None:
            vals, mn, mx, sp = self.ctx.precompute_sdf(self.vertices.T, self.faces.T, float(dx), _SDFMESH_RES)
            grid = (vals, mn, mx, sp)
            if save_path:
                self._sdf_path = save_path
                sdfc.save_sdf_text(save_path, *grid)
        self.values, self.min_box, self.max_box, self.spacing = grid
        # col_th 0: SDFMesh's distance is the bare interpolated value
        self.grid = self.ctx.upload_grid(self.values, self.min_box, self.max_box, self.spacing, 0.0,
                                         sdfc.STORAGE_F64)

    def distance(self, X) -> np.ndarray:
        """SDFMesh::distance: X (3, n) in the mesh's frame -> (n,) (FLT_MAX outside the grid)."""
        d, _ = self.ctx.grid_distance(self.grid, np.asarray(X, dtype=np.float64).reshape(3, -1).T)
        return d

    def min_distance(self, X) -> float:
        """SDFMesh::min_distance (rm/Mesh.cpp:18-20)."""
        _, m = self.ctx.grid_distance(self.grid, np.asarray(X, dtype=np.float64).reshape(3, -1).T,
                                      want_values=False)
        return m

    def clear_saved_sdf(self):
        """SDFMesh::clear_saved_SDF: removes the cache file this mesh was loaded from or saved to."""
        if self._sdf_path and os.path.exists(self._sdf_path):
            os.remove(self._sdf_path)


class BodyDistance:
    """Simulation::get_body_distance(from, to) for many pose pairs at once.

    ``vertices_from``: body-frame mesh vertices of the `from` body (nv, 3); ``grid_to``: a grid
    handle of the `to` body uploaded with its col_th (BodySDFObj::distance adds it).  One batch of
    `n` instances; ``__call__(E_from, E_to)`` takes n poses each ((n, 4, 4), Body::_E_0i) and
    returns the n minima."""

    def __init__(self, ctx, vertices_from, grid_to, n):
        self.ctx = ctx
        self.points = ctx.upload_points(np.asarray(vertices_from, dtype=np.float64).reshape(-1, 3),
                                        sdfc.STORAGE_F64)
        self.batch = ctx.batch([self.points] * n, [grid_to] * n)
        self.n = n

    def __call__(self, E_from, E_to) -> np.ndarray:
        return self.batch.distance(E_from, E_to)


def body_in_contact(d_ab, d_ba, eps) -> np.ndarray:
    """Simulation::body_in_contact (rm/Simulation.cpp:298-303) from the two directions' distances."""
    return np.minimum(d_ab, d_ba) < eps


class DisassemblyCheck:
    """PhysicsPlanner.is_disassembled (examples/run_joint_plan.py:291-302) for many poses at once.

    ``vertices_move``: the moving part's mesh vertices in its body frame (get_body_vertices,
    (n, 3)); ``vertices_still``: every still part's vertices in world (stacked, (m, 3)).  Both
    hulls are built once, as the planner builds them in its constructor (:225-228);
    ``__call__(E0i)`` takes poses (k, 4, 4) of the moving part and returns k booleans."""

    def __init__(self, ctx, vertices_move, vertices_still):
        self.ctx = ctx
        self.hull_move = ctx.upload_hull(vertices_move)
        self.hull_still = ctx.upload_hull(vertices_still)

    def __call__(self, E0i, with_flags=False):
        return self.ctx.disassembled(self.hull_move, self.hull_still, E0i, with_flags)
