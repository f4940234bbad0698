"""Mesh -> SDF grid on the CPU: the oracle's restatement of sdfgen::make_level_set3 and the
library's BodySDFObj::precompute_SDF grid layout against the reference's own outputs
(tests/golden/levelset.npz).  Bit-exact: FP32 phi compared as bit patterns."""
import numpy as np
import pytest

from _helpers import load
from conftest import submodule


@pytest.fixture(scope="module")
def fx():
    return load("levelset.npz")


def case(fx, name):
    g = lambda k: fx[f"case_{name}_{k}"]
    return g("verts"), g("tris"), g("origin"), g("dx"), tuple(int(s) for s in g("shape")), int(g("band")), g("phi")


def test_oracle_cases(fx, oracle):
    for name in fx["cases"]:
        V, T, o, d, shape, band, phi = case(fx, str(name))
        got = oracle.make_level_set3(V, T, o, d, shape, band)
        assert got.shape == phi.shape
        assert np.array_equal(got.view(np.uint32), phi.view(np.uint32)), name


def test_layout_and_body_grid(fx, oracle):
    """precompute_SDF: the grid layout (library, host arithmetic) and the values (oracle)
    of a body the reference loaded from an OBJ file."""
    sdfc = submodule("sdfc")
    shape, mn, mx, sp, origin = sdfc.sdf_grid_layout(fx["body_V"], float(fx["body_dx"]), int(fx["body_res"]))
    assert shape == tuple(int(s) for s in fx["body_shape"])
    assert np.array_equal(mn, fx["body_min_box"]) and np.array_equal(mx, fx["body_max_box"])
    assert np.array_equal(sp, fx["body_spacing"])
    assert np.array_equal(origin.astype(np.float64), mn)
    phi = oracle.make_level_set3(fx["body_V"].astype(np.float32), fx["body_F"], origin, sp.astype(np.float32),
                                 shape)
    assert np.array_equal(phi.view(np.uint32), fx["body_values"].view(np.uint32))


def test_layout_rules():
    sdfc = submodule("sdfc")
    V, _ = submodule("workloads").box_mesh((0.5, 0.25, 0.1))
    shape, mn, mx, sp, _ = sdfc.sdf_grid_layout(V, 0.05, 10)
    # spacing = min(dx, bbox / res) per axis; one cell of padding
    np.testing.assert_array_equal(sp, [0.05, 0.05, 0.02])
    np.testing.assert_allclose(mn, [-0.55, -0.3, -0.12], rtol=1e-6)
    assert shape == (23, 13, 13)
    with pytest.raises(sdfc.SdfcError):
        sdfc.sdf_grid_layout(V, 0.05, 0)


def test_float_quotient_identity():
    """The GPU level set divides in FP32 where the reference divides float operands in FP64
    and rounds to float (point_segment_distance); the two agree bit for bit.  Checked on
    random, tiny, huge and tie-prone operands."""
    r = np.random.default_rng(3)
    a = np.concatenate([r.standard_normal(200000), r.uniform(-1, 1, 50000) * 1e-38, r.uniform(1, 2, 50000) * 1e38,
                        np.arange(1, 50001), [0.0, -0.0, 1.0, 3.0]]).astype(np.float32)
    b = np.concatenate([r.standard_normal(200000), r.uniform(0.5, 2, 50000) * 1e5, r.uniform(1e-3, 1e-2, 50000),
                        np.full(50000, 3.0), [0.0, 1.0, 0.0, 7.0]]).astype(np.float32)
    with np.errstate(all="ignore"):
        via_double = (a.astype(np.float64) / b.astype(np.float64)).astype(np.float32)
        direct = a / b
    assert np.array_equal(via_double.view(np.uint32), direct.view(np.uint32))
