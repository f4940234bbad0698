"""Mesh -> SDF grid on the GPU (sdfc_make_level_set3 / sdfc_sdf_grid_layout) against the
reference's own outputs (tests/golden/levelset.npz) and the oracle.  Bit-exact: FP32 phi
compared as bit patterns."""
import numpy as np
import pytest

from _helpers import load
from conftest import submodule
from test_levelset import case

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


def same_bits(a, b):
    return a.shape == b.shape and np.array_equal(np.asarray(a, np.float32).view(np.uint32),
                                                 np.asarray(b, np.float32).view(np.uint32))


def test_golden_cases(ctx):
    fx = load("levelset.npz")
    for name in fx["cases"]:
        V, T, o, d, shape, band, phi = case(fx, str(name))
        assert same_bits(ctx.make_level_set3(V, T, o, d, shape, band), phi), name


def test_body_precompute(ctx):
    """BodySDFObj::precompute_SDF as a whole: layout + GPU level set = the reference body's grid."""
    fx = load("levelset.npz")
    vals, mn, mx, sp = ctx.precompute_sdf(fx["body_V"], fx["body_F"], float(fx["body_dx"]), int(fx["body_res"]))
    assert np.array_equal(vals, fx["body_values"].astype(np.float64))
    assert np.array_equal(mn, fx["body_min_box"]) and np.array_equal(mx, fx["body_max_box"])
    assert np.array_equal(sp, fx["body_spacing"])


def bumpy_torus(workloads, n, m, seed):
    V, F = workloads.torus_mesh(0.6, 0.25, n, m)
    r = np.random.default_rng(seed)
    return V * (1 + 0.03 * r.standard_normal((len(V), 1))), F


@pytest.mark.parametrize("n,m,dx,band", [(96, 48, 0.015, 1), (256, 128, 0.05, 1), (40, 20, 0.02, 3)])
def test_against_oracle(ctx, oracle, workloads, n, m, dx, band):
    """Seeded bumpy tori: fine grids (many sweep diagonals), and many triangles per cell (ties
    of the band's packed-key minimum)."""
    V, F = bumpy_torus(workloads, n, m, n + m)
    origin, shape = workloads.level_set_grid(V, dx)
    want = oracle.make_level_set3(V, F, origin, dx, shape, band)
    got = ctx.make_level_set3(V, F, origin, dx, shape, band)
    assert same_bits(got, want)
    assert (got < 0).any() and (got > 0).any()


def test_device_arrays(ctx, workloads):
    torch = pytest.importorskip("torch")
    V, F = workloads.socket_mesh(1.0, 0.5, 1.0)
    origin, shape = workloads.level_set_grid(V, 0.05)
    want = ctx.make_level_set3(V, F, origin, 0.05, shape)
    Vd = torch.tensor(np.asarray(V, np.float32), device="cuda")
    Fd = torch.tensor(np.asarray(F, np.int32), device="cuda")
    got = ctx.make_level_set3_device(Vd, Fd, origin, 0.05, shape)
    torch.cuda.synchronize()
    assert same_bits(got.cpu().numpy(), want)


def test_small_and_empty(ctx, oracle, workloads):
    V, F = workloads.box_mesh((0.3, 0.3, 0.3))
    # no triangles: every node keeps the upper bound (ni+nj+nk)*(dx+dy+dz)
    phi = ctx.make_level_set3(V, F[:0], [-0.5] * 3, 0.1, (11, 11, 11))
    assert same_bits(phi, oracle.make_level_set3(V, F[:0], [-0.5] * 3, 0.1, (11, 11, 11)))
    assert np.all(phi == phi.flat[0]) and phi.flat[0] > 9.8
    # grids one node thick in some direction (no sweeps there)
    for shape in ((1, 7, 7), (7, 1, 1), (2, 2, 9)):
        want = oracle.make_level_set3(V, F, [-0.4] * 3, 0.1, shape, 1)
        assert same_bits(ctx.make_level_set3(V, F, [-0.4] * 3, 0.1, shape, 1), want), shape


def test_errors(ctx, sdfc, workloads):
    V, F = workloads.box_mesh()
    with pytest.raises(sdfc.SdfcError):
        ctx.make_level_set3(V, F + 100, [0, 0, 0], 0.1, (4, 4, 4))
    with pytest.raises(sdfc.SdfcError):
        ctx.make_level_set3(V, F, [0, 0, 0], 0.1, (0, 4, 4))
    with pytest.raises(sdfc.SdfcError):
        ctx.make_level_set3(V, F, [0, 0, 0], 0.1, (4, 4, 4), exact_band=-1)


def test_grid_feeds_contact(ctx, sdfc, workloads):
    """A grid built here is an ordinary contact grid: upload it and evaluate a pair."""
    V, F = workloads.socket_mesh(1.0, 0.5, 1.0)
    vals, mn, mx, sp = ctx.precompute_sdf(V, F, 0.05, 20)
    g = ctx.upload_grid(vals, mn, mx, sp, 0.01, sdfc.STORAGE_F64)
    pts = workloads.peg_points(2000, radius=0.48)
    p = ctx.upload_points(pts, sdfc.STORAGE_F64)
    E = np.eye(4)
    E[0, 3] = 0.05  # pushes the peg 0.03 into the bore wall (col_th 0.01)
    fm, Km, Dm, n_act = ctx.evaluate(p, g, E, np.zeros(6), np.eye(4), np.zeros(6), sdfc.Params(1e5, 1e3, 0.3, 1e3))
    assert n_act > 0 and np.isfinite(fm).all() and np.abs(fm).sum() > 0
