"""The planner's disassembly check on the GPU (sdfc_disassembled) against the oracle's exact
restatement (LP feasibility, facet inequalities, boxes) on seeded poses.  The two may differ
only where the answer changes within 1e-7 of the pose (hulls touching to within round-off);
every disagreement is checked to be such a pose."""
import numpy as np
import pytest

from conftest import submodule
from oracle import disassembly as D

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sdfc():
    submodule("build").build()
    return submodule("sdfc")


@pytest.fixture(scope="module")
def ctx(sdfc):
    c = sdfc.Context(0)
    yield c
    c.close()


def random_poses(rng, n, span, rot):
    W = submodule("workloads")
    E = np.zeros((n, 4, 4))
    for k in range(n):
        E[k] = W.pose(W.rotvec_to_matrix(rng.normal(size=3) * rot), rng.uniform(-span, span, 3))
    return E


def near_boundary(oracle_check, E, h=1e-7):
    """Whether the oracle's answer changes within h of pose E (translations along the axes)."""
    base = oracle_check(E)
    for a in range(3):
        for s in (-h, h):
            E2 = E.copy()
            E2[a, 3] += s
            if oracle_check(E2) != base:
                return True
    return False


def check(ctx, move, still, E):
    mesh = submodule("mesh")
    chk = mesh.DisassemblyCheck(ctx, move, still)
    got, flags = chk(E, with_flags=True)
    oc = D.Checker(move, still)
    want = np.array([oc(e) for e in E])
    bad = np.nonzero(got != want)[0]
    for q in bad:
        assert near_boundary(oc, E[q]), (q, got[q], want[q], flags[q])
    assert (flags >> 8).max() < 64  # GJK settled everywhere
    return want


def test_peg_socket(ctx):
    W = submodule("workloads")
    rng = np.random.default_rng(7)
    peg = W.peg_points(3000, radius=0.48)
    socket, _ = W.socket_mesh(1.0, 0.5, 1.0)
    E = random_poses(rng, 500, 2.5, 0.5)
    want = check(ctx, peg, socket, E)
    assert 0.1 < want.mean() < 0.9


def test_random_blobs(ctx):
    rng = np.random.default_rng(8)
    for trial in range(3):
        move = rng.normal(size=(400, 3)) * [0.3, 0.5, 0.2]
        still = np.concatenate([rng.normal(size=(300, 3)) * 0.6, rng.normal(size=(300, 3)) * 0.4 + [1.0, 0, 0]])
        E = random_poses(rng, 300, 1.8, 2.0)
        want = check(ctx, move, still, E)
        assert want.any() and not want.all()


def test_assembly_parts(ctx):
    W = submodule("workloads")
    asm = W.procedural_assembly(3, n_parts=5, points=(2000, 4000), grids=(48,))
    mover = asm.parts[0]
    move = mover.surface_points(2000, 3)
    still = np.concatenate([p.surface_points(1500, 4 + k) for k, p in enumerate(asm.parts[1:])])
    rng = np.random.default_rng(9)
    E = np.zeros((300, 4, 4))
    for k in range(300):
        E[k] = W.pose(W.rotvec_to_matrix(rng.normal(size=3) * 0.05), rng.normal(size=3) * 1.5)
    check(ctx, move, still, E)


def test_empty_and_errors(ctx, sdfc):
    W = submodule("workloads")
    peg = W.peg_points(500)
    h = ctx.upload_hull(peg)
    assert len(ctx.disassembled(h, h, np.zeros((0, 4, 4)))) == 0
    with pytest.raises(sdfc.SdfcError):
        ctx.disassembled(h, 99, np.eye(4)[None])
