"""Planner-side distances on the GPU: SDFMesh (grid, distance, min_distance, .sdf cache),
batched get_body_distance / body_in_contact, and FP16-brick cache files, against the
reference's outputs (tests/golden/mesh_distance.npz) and the oracle.  Bit-exact."""
import numpy as np
import pytest

from _helpers import load
from conftest import submodule

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


@pytest.fixture(scope="module")
def fx():
    return load("mesh_distance.npz")


def test_sdfmesh(ctx, fx):
    mesh = submodule("mesh")
    m = mesh.SDFMesh(fx["sdfmesh_V"].T, fx["sdfmesh_F"].T, float(fx["sdfmesh_dx"]), ctx=ctx)
    assert np.array_equal(m.values, fx["sdfmesh_values"])
    assert np.array_equal(m.min_box, fx["sdfmesh_min_box"]) and np.array_equal(m.spacing, fx["sdfmesh_spacing"])
    d = m.distance(fx["sdfmesh_X"].T)
    assert np.array_equal(d, fx["sdfmesh_d"])
    assert m.min_distance(fx["sdfmesh_X"].T) == fx["sdfmesh_min"]
    assert m.min_distance(np.zeros((3, 0))) == np.inf


def test_sdfmesh_cache_files(ctx, fx, tmp_path):
    """save_path writes the reference's text; load_path reads what the reference's load_SDF reads."""
    mesh = submodule("mesh")
    W = submodule("workloads")
    V, F = W.box_mesh((0.5, 0.3, 0.2))
    path = tmp_path / "box.sdf"
    m = mesh.SDFMesh(V.T, F.T, 0.06, save_path=str(path), ctx=ctx)
    assert path.read_bytes() == fx["text_bytes"].tobytes()
    back = mesh.SDFMesh(V.T, F.T, 0.06, load_path=str(path), ctx=ctx)
    assert np.array_equal(back.values, fx["text_read_values"])
    X = np.random.default_rng(1).uniform(-0.6, 0.6, (3, 500))
    assert np.isfinite(back.distance(X)).all()
    back.clear_saved_sdf()
    assert not path.exists()
    assert np.array_equal(m.values, fx["text_values"])


def test_body_distance(ctx, sdfc, fx):
    mesh = submodule("mesh")
    n = len(fx["body_EA"])
    gA = ctx.upload_grid(fx["body_gridA"], fx["body_minA"], fx["body_maxA"], fx["body_dxA"], float(fx["body_colA"]),
                         sdfc.STORAGE_F64)
    gB = ctx.upload_grid(fx["body_gridB"], fx["body_minB"], fx["body_maxB"], fx["body_dxB"], float(fx["body_colB"]),
                         sdfc.STORAGE_F64)
    ab = mesh.BodyDistance(ctx, fx["body_VA"], gB, n)
    ba = mesh.BodyDistance(ctx, fx["body_VB"], gA, n)
    dab = ab(fx["body_EA"], fx["body_EB"])
    dba = ba(fx["body_EB"], fx["body_EA"])
    assert np.array_equal(dab, fx["body_dab"]) and np.array_equal(dba, fx["body_dba"])
    inc = mesh.body_in_contact(dab, dba, float(fx["body_eps"]))
    assert np.array_equal(inc, fx["body_in_contact"])


def test_per_point_distances(ctx, sdfc, fx, oracle):
    """Every vertex's distance, in the caller's order, against the oracle; uneven instances."""
    gB = ctx.upload_grid(fx["body_gridB"], fx["body_minB"], fx["body_maxB"], fx["body_dxB"], float(fx["body_colB"]),
                         sdfc.STORAGE_F64)
    rng = np.random.default_rng(4)
    sets = [fx["body_VA"], fx["body_VA"][::-1].copy(), rng.uniform(-1.2, 1.2, (5000, 3)), np.zeros((0, 3))]
    handles = [ctx.upload_points(s, sdfc.STORAGE_F64) for s in sets]
    b = ctx.batch(handles, [gB] * len(sets))
    EA = fx["body_EA"][:4]
    EB = fx["body_EB"][:4]
    mn, per = b.distance(EA, EB, per_point=True)
    from oracle import oracle as O
    g = O.Grid(fx["body_gridB"], fx["body_minB"], fx["body_maxB"], fx["body_dxB"], float(fx["body_colB"]))
    for k, s in enumerate(sets):
        if len(s) == 0:
            assert mn[k] == np.inf and len(per[k]) == 0
            continue
        m, d = O.body_distance(g, EA[k], EB[k], s, per_point=True)
        assert np.array_equal(per[k], d), k
        assert mn[k] == m
    b.close()


def test_brick_cache_upload(ctx, sdfc, fx, tmp_path):
    """A brick cache file uploads without re-encoding: the same grid, the same evaluations, as
    uploading the FP64 values with SDFC_STORAGE_F16_BRICKS."""
    vals, mn, mx, dx = fx["sdfmesh_values"], fx["sdfmesh_min_box"], fx["sdfmesh_max_box"], fx["sdfmesh_spacing"]
    path = tmp_path / "g.sdfb"
    sdfc.save_sdf_bricks(path, vals, mn, mx, dx)
    codes, so, shape, mn2, mx2, dx2 = sdfc.load_sdf_bricks(path)
    g1 = ctx.upload_grid_bricks(codes, so, shape, mn2, mx2, dx2, 0.01)
    g2 = ctx.upload_grid(vals, mn, mx, dx, 0.01, sdfc.STORAGE_F16_BRICKS)
    assert np.array_equal(ctx.grid_values(g1), ctx.grid_values(g2))
    W = submodule("workloads")
    p = ctx.upload_points(W.peg_points(3000, radius=0.48), sdfc.STORAGE_F32)
    E = np.eye(4)
    E[0, 3] = 0.05
    r1 = ctx.evaluate(p, g1, E, np.zeros(6), np.eye(4), np.zeros(6), sdfc.Params(1e5, 1e3, 0.3, 1e3))
    r2 = ctx.evaluate(p, g2, E, np.zeros(6), np.eye(4), np.zeros(6), sdfc.Params(1e5, 1e3, 0.3, 1e3))
    assert r1[3] == r2[3] > 0
    for a, b in zip(r1[:3], r2[:3]):
        assert np.array_equal(a, b)
