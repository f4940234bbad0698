"""Planner-side distances and SDF cache files on the CPU: the oracle and the library's host
code against the reference's own outputs (tests/golden/mesh_distance.npz)."""
import os

import numpy as np
import pytest

from _helpers import load
from conftest import submodule


@pytest.fixture(scope="module")
def fx():
    return load("mesh_distance.npz")


@pytest.fixture(scope="module")
def sdfc():
    return submodule("sdfc")


def test_text_cache_bytes(fx, sdfc, tmp_path):
    """save_sdf_text writes the reference's SDFMesh::save_SDF file byte for byte."""
    path = tmp_path / "g.sdf"
    sdfc.save_sdf_text(path, fx["text_values"], fx["text_min_box"], fx["text_max_box"], fx["text_spacing"])
    assert path.read_bytes() == fx["text_bytes"].tobytes()


def test_text_cache_read(fx, sdfc, tmp_path):
    """load_sdf_text reads the reference's file into the values the reference's load_SDF reads."""
    path = tmp_path / "g.sdf"
    path.write_bytes(fx["text_bytes"].tobytes())
    v, mn, mx, dx = sdfc.load_sdf_text(path)
    assert np.array_equal(v, fx["text_read_values"])
    assert np.array_equal(mn, fx["text_read_min_box"]) and np.array_equal(mx, fx["text_read_max_box"])
    assert np.array_equal(dx, fx["text_read_spacing"])
    # the cache is lossy (6 significant digits), as the reference's
    assert not np.array_equal(v, fx["text_values"])
    assert sdfc.load_sdf_text(tmp_path / "missing.sdf") is None
    (tmp_path / "bad.sdf").write_text("3 3 3\n0 0 0\n1 1 1\n0.5 0.5\n")
    with pytest.raises(sdfc.SdfcError):
        sdfc.load_sdf_text(tmp_path / "bad.sdf")
    (tmp_path / "short.sdf").write_text("2 2 2\n0 0 0\n1 1 1\n1 1 1\n0.5\n0.25\n")
    with pytest.raises(sdfc.SdfcError):
        sdfc.load_sdf_text(tmp_path / "short.sdf")


def test_brick_cache(fx, sdfc, tmp_path):
    vals = fx["sdfmesh_values"]
    path = tmp_path / "g.sdfb"
    sdfc.save_sdf_bricks(path, vals, fx["sdfmesh_min_box"], fx["sdfmesh_max_box"], fx["sdfmesh_spacing"])
    codes, so, shape, mn, mx, dx = sdfc.load_sdf_bricks(path)
    c0, s0 = sdfc.f16_brick_encode(vals)
    assert shape == vals.shape
    assert np.array_equal(codes, c0) and np.array_equal(so.view(np.uint32), s0.view(np.uint32))
    assert np.array_equal(mn, fx["sdfmesh_min_box"]) and np.array_equal(dx, fx["sdfmesh_spacing"])
    assert sdfc.load_sdf_bricks(tmp_path / "missing.sdfb") is None
    (tmp_path / "bad.sdfb").write_bytes(b"SDFCBRK0" + bytes(100))
    with pytest.raises(sdfc.SdfcError):
        sdfc.load_sdf_bricks(tmp_path / "bad.sdfb")


def test_sdfmesh_grid_and_distance_oracle(fx, sdfc, oracle):
    """SDFMesh's grid (layout with res 20, level set) and distance() through the oracle."""
    V, F = fx["sdfmesh_V"], fx["sdfmesh_F"]
    shape, mn, mx, sp, origin = sdfc.sdf_grid_layout(V, float(fx["sdfmesh_dx"]), 20)
    assert np.array_equal(mn, fx["sdfmesh_min_box"]) and np.array_equal(sp, fx["sdfmesh_spacing"])
    phi = oracle.make_level_set3(V.astype(np.float32), F, origin, sp.astype(np.float32), shape)
    assert np.array_equal(phi.astype(np.float64), fx["sdfmesh_values"])
    g = oracle.Grid(fx["sdfmesh_values"], mn, mx, sp, 0.0)
    d = np.array([oracle.query_sdf(g, x) for x in fx["sdfmesh_X"]])
    assert np.array_equal(d, fx["sdfmesh_d"])
    assert d.min() == fx["sdfmesh_min"]


def test_body_distance_oracle(fx, oracle):
    """get_body_distance both ways and body_in_contact through the oracle, bit for bit."""
    gA = oracle.Grid(fx["body_gridA"], fx["body_minA"], fx["body_maxA"], fx["body_dxA"], float(fx["body_colA"]))
    gB = oracle.Grid(fx["body_gridB"], fx["body_minB"], fx["body_maxB"], fx["body_dxB"], float(fx["body_colB"]))
    for k in range(len(fx["body_EA"])):
        EA, EB = fx["body_EA"][k], fx["body_EB"][k]
        dab = oracle.body_distance(gB, EA, EB, fx["body_VA"])
        dba = oracle.body_distance(gA, EB, EA, fx["body_VB"])
        assert dab == fx["body_dab"][k] and dba == fx["body_dba"][k], k
        assert (min(dab, dba) < float(fx["body_eps"])) == bool(fx["body_in_contact"][k])
