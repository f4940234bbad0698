"""Planner scenes on sdfc_sim.

The reference's planner builds, for one pulled part and the still parts of an assembly, a scene
whose moving part is on a joint and in contact with every still part in both directions
(general_SDF_contact with the mover as contact body and as SDF body,
examples/run_joint_plan.py:140-178).  `AssemblyScene` prepares that data for a procedural
assembly (workloads.procedural_assembly) and `build_sim` puts many such scenes, each with its own
parts, point counts and grid sizes, into one sdfc_sim.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import sdfc, workloads as W


@dataclass
class AssemblyScene:
    asm: W.Assembly
    grids: list      # GridSpec per part (part frame)
    points: list     # contact points per part (part frame, FP32-representable)
    mass: float      # the mover's mass and inertia diagonal
    inertia: np.ndarray

    @classmethod
    def make(cls, asm: W.Assembly, seed: int = 0, dtype=np.float32):
        grids = [p.grid(n, dtype=dtype) for p, n in zip(asm.parts, asm.grid_n)]
        pts = [p.surface_points(n, seed * 1000 + k).astype(np.float32).astype(np.float64)
               for k, (p, n) in enumerate(zip(asm.parts, asm.n_points))]
        m, inertia = asm.parts[asm.mover].mass_props()
        return cls(asm, grids, pts, m, inertia)

    @classmethod
    def make_device(cls, ctx: "sdfc.Context", asm: W.Assembly, seed: int = 0, storage=sdfc.STORAGE_F32_NODES,
                    col_th=0.0):
        """The scene of a large assembly generated on the device: each part's FP32 grid is sampled
        on the GPU and uploaded at once (kept only in the context, as grid handles), and its
        contact points are drawn on the GPU (kept on the host for the point upload)."""
        import torch
        handles, boxes = [], []
        for p, n in zip(asm.parts, asm.grid_n):
            vals, mn, mx, dx = p.grid_device(n)
            torch.cuda.current_stream().synchronize()  # the library reads the values on its own stream
            handles.append(ctx.upload_grid_device(vals.data_ptr(), tuple(vals.shape), mn, mx, dx, col_th, storage))
            boxes.append((mn, mx, dx))
            del vals
        pts = [p.surface_points_device(n, seed * 1000 + k) for k, (p, n) in enumerate(zip(asm.parts, asm.n_points))]
        m, inertia = asm.parts[asm.mover].mass_props()
        sc = cls(asm, None, pts, m, inertia)
        sc.grid_handles = handles
        sc.grid_boxes = boxes  # (min_box, max_box, dx) per part
        return sc

    def placement(self, k):
        return W.pose(None, self.asm.parts[k].position)

    def contact_pairs(self):
        """(contact part, SDF part) of every contact: the mover against each still part, both ways."""
        m = self.asm.mover
        out = []
        for k in range(len(self.asm.parts)):
            if k != m:
                out += [(m, k), (k, m)]
        return out


def build_sim(ctx: "sdfc.Context", scenes, h, gravity, params: "sdfc.Params", col_th=0.0,
              storage=sdfc.STORAGE_F32):
    """One sdfc_sim over `scenes` (AssemblyScene list).  Returns the sim; every mover starts at
    q = qdot = 0 with no external force."""
    movers, pairs = [], []
    for i, sc in enumerate(scenes):
        gh = getattr(sc, "grid_handles", None)  # grids generated and uploaded on the device
        if gh is None:
            gh = [ctx.upload_grid(g.values, g.min_box, g.max_box, g.dx, col_th, storage) for g in sc.grids]
        ph = [ctx.upload_points(p, sdfc.STORAGE_F32 if storage == sdfc.STORAGE_F32_NODES else storage)
              for p in sc.points]
        m = sc.asm.mover
        movers.append(sdfc.Mover.make(sc.mass, sc.inertia, np.eye(4), h, gravity, E_pj0=sc.placement(m)))
        for a, b in sc.contact_pairs():
            still = b if a == m else a
            pairs.append(sdfc.ScenePair.make(i, ph[a], gh[b], a == m, sc.placement(still), params))
    return ctx.sim(movers, pairs)


def pull_forces(scenes, magnitude):
    """External force rows (torque then force, world frame) pulling each mover along its direction."""
    F = np.zeros((len(scenes), 6))
    for i, sc in enumerate(scenes):
        F[i, 3:] = magnitude * sc.asm.direction
    return F
