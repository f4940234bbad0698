"""The oracle's restatement of the planner's disassembly check on configurations whose answer is
known by construction (the reference's own path needs trimesh and python-fcl, absent here)."""
import numpy as np

from conftest import submodule
from oracle import disassembly as D


def pose(p, R=None):
    E = np.eye(4)
    if R is not None:
        E[:3, :3] = R
    E[:3, 3] = p
    return E


def test_known_configurations():
    W = submodule("workloads")
    peg = W.peg_points(1500, radius=0.48)               # cylinder r 0.48, z in [-1, 1]
    socket, _ = W.socket_mesh(1.0, 0.5, 1.0)             # hull: the box [-1, 1]^3
    assert not D.is_disassembled(peg, socket, pose([0, 0, 0]))        # inside the box's hull
    assert not D.is_disassembled(peg, socket, pose([0, 0, 1.5]))      # surfaces cross
    assert D.is_disassembled(peg, socket, pose([0, 0, 2.1]))          # clear above
    assert D.is_disassembled(peg, socket, pose([1.6, 0, 0]))          # clear beside
    # apart but the still hull's box contains the moving hull's box: not disassembled
    big, _ = W.box_mesh((3, 3, 3))
    tilted = W.rotvec_to_matrix([0, 0, np.pi / 4]) @ np.diag([1, 0.05, 1])
    slab = socket @ tilted.T
    small, _ = W.box_mesh((0.1, 0.1, 0.1))
    assert not D.is_disassembled(small, slab, pose([0.4, -0.4, 0]))
    assert D.is_disassembled(small, slab, pose([2.0, -2.0, 0]))
    # the moving hull contains the still hull
    assert not D.is_disassembled(big, socket, pose([0, 0, 0]))
    # helpers agree with the definition
    VA, PA = D.hull_of(peg)
    assert D.inside(VA, D.hull_of(socket)[1])
    assert D.solids_meet(VA, D.hull_of(socket)[0])
    assert not D.solids_meet(VA + [0, 0, 2.5], D.hull_of(socket)[0])
