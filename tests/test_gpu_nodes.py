"""FP32 node-value grids (SDFC_STORAGE_F32_NODES), device-side grid uploads and the detection
broad phase (tiles whose bounding sphere is away from the grid box), through the C ABI.

The node storage keeps 4 bytes per node where SDFC_STORAGE_F32 keeps 40; every evaluation sees
the same values, so results must equal SDFC_STORAGE_F32's bit for bit wherever the per-contact
algebra is FP64 (the FP64 path, the stencil mode, values and energies).  The FP32-algebra path
runs a separate compilation of the same algebra for grids with the cell-corner array, whose
multiply-add contraction may differ in the last bits: there the results agree to 1e-8 relative
(measured 7e-10 in Dm, fm and Km identical), far below that path's own error against FP64 (1e-7).
The broad phase may only skip tiles whose points would all fail the box test, so active sets stay
the reference's."""
import numpy as np
import pytest

from _helpers import assert_close, load
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


def sweep_states(workloads, n, seed):
    rng = np.random.default_rng(seed)
    ang = rng.uniform(0, 2 * np.pi, n)
    EA = np.stack([workloads.pose(workloads.rotvec_to_matrix(rng.normal(size=3) * 0.004),
                                  [0.026 * np.cos(a), 0.026 * np.sin(a), 0.3 * rng.normal()]) for a in ang])
    EB = np.tile(np.eye(4), (n, 1, 1))
    return EA, rng.normal(size=(n, 6)) * 0.2, EB, np.zeros((n, 6))


def test_golden_single_pair_nodes(sdfc, ctx):
    """The reference's golden pair evaluations on an FP32-node grid."""
    fx = load("pair_eval.npz")
    grid = ctx.upload_grid(fx["grid"], fx["min_box"], fx["max_box"], fx["dx"], float(fx["col_th"]),
                           sdfc.STORAGE_F32_NODES)
    pts = ctx.upload_points(fx["points"], 0)
    g64 = ctx.upload_grid(fx["grid"], fx["min_box"], fx["max_box"], fx["dx"], float(fx["col_th"]), 0)
    for k in range(len(fx["fm"])):
        prm = sdfc.Params(*[float(x) for x in fx["params"][k]])
        args = (fx["EA"][k], fx["phiA"][k], fx["EB"][k], fx["phiB"][k], prm)
        fm, Km, Dm, n = ctx.evaluate(pts, grid, *args, want_deriv=True)
        ids = ctx.active_ids()
        ref_ids = fx["ids"][k][: fx["n_active"][k]]
        assert n == len(ref_ids) and np.array_equal(ids, ref_ids), f"case {k}"
        # the golden grid is FP32-representable (sdfgen computes in FP32), so FP32 node values
        # are the reference's grid exactly
        f0, K0, D0, _ = ctx.evaluate(pts, g64, *args, want_deriv=True)
        assert np.array_equal(fm, f0) and np.array_equal(Km, K0) and np.array_equal(Dm, D0), f"case {k}"
        assert_close(f"case {k} fm", fm, fx["fm"][k], rel=1e-10)
        assert_close(f"case {k} Km", Km, fx["Km"][k], rel=1e-6)


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("stencil", [0, 1])
def test_nodes_equal_cell_corners(sdfc, ctx, workloads, precision, stencil):
    """A batch over FP32-node grids equals the same batch over SDFC_STORAGE_F32 bit for bit, and
    a batch mixing the two storages equals both (the cell-corner kernels and the general ones
    split its instances)."""
    g = workloads.socket_grid(48, dtype=np.float32)
    h1 = ctx.upload_grid(g.values, g.min_box, g.max_box, g.dx, 0.01, sdfc.STORAGE_F32)
    h3 = ctx.upload_grid(g.values, g.min_box, g.max_box, g.dx, 0.01, sdfc.STORAGE_F32_NODES)
    assert np.array_equal(ctx.grid_values(h3), ctx.grid_values(h1))
    ph = ctx.upload_points(workloads.peg_points(6000, seed=21), 1)
    n = 8
    EA, phiA, EB, phiB = sweep_states(workloads, n, 5)
    prm = [sdfc.Params(1e5, 1e3, 0.3, 1e3, 1.0, 1.0)] * n

    def run(grids, deriv=True):
        b = ctx.batch([ph] * n, grids)
        b.set_precision(precision)
        b.set_derivative_mode(stencil)
        out = b.evaluate(EA, phiA, EB, phiB, prm, want_deriv=deriv)
        e = b.energy(EA, EB, prm)
        b.close()
        return out, e

    (fa, Ka, Da, na, sa), ea = run([h1] * n)
    assert (na > 0).all() and not sa.any()
    fp32_algebra = precision == 1 and stencil == 0
    for grids in ([h3] * n, [h1, h3] * (n // 2)):
        (fb, Kb, Db, nb, sb), eb = run(grids)
        assert np.array_equal(na, nb) and not sb.any()
        if fp32_algebra:
            for name, x, y in (("fm", fa, fb), ("Km", Ka, Kb), ("Dm", Da, Db)):
                assert_close(name, y, x, rel=1e-8)
        else:
            assert np.array_equal(fa, fb) and np.array_equal(Ka, Kb) and np.array_equal(Da, Db)
        assert all(np.array_equal(x, y) for x, y in zip(ea, eb))
    (fv, _, _, nv, _), _ = run([h3] * n, deriv=False)
    (fw, _, _, nw, _), _ = run([h1] * n, deriv=False)
    assert np.array_equal(fv, fw) and np.array_equal(nv, nw)


def test_device_upload_equals_host_upload(sdfc, ctx, workloads):
    """sdfc_upload_grid_device (FP32 values on the device) gives the grids sdfc_upload_grid gives
    from the same values on the host, for both FP32 storages; non-finite values are refused."""
    torch = pytest.importorskip("torch")
    g = workloads.socket_grid(40, dtype=np.float32)
    d = torch.from_numpy(g.values.astype(np.float32)).cuda()
    torch.cuda.synchronize()  # the library reads the values on its own stream
    hosts = [ctx.upload_grid(g.values, g.min_box, g.max_box, g.dx, 0.01, st)
             for st in (sdfc.STORAGE_F32, sdfc.STORAGE_F32_NODES)]
    devs = [ctx.upload_grid_device(d.data_ptr(), g.shape, g.min_box, g.max_box, g.dx, 0.01, st)
            for st in (sdfc.STORAGE_F32, sdfc.STORAGE_F32_NODES)]
    for h in hosts + devs:
        assert np.array_equal(ctx.grid_values(h), g.values)
    ph = ctx.upload_points(workloads.peg_points(5000, seed=3), 1)
    n = 6
    EA, phiA, EB, phiB = sweep_states(workloads, n, 8)
    prm = [sdfc.Params(1e5, 1e3, 0.3, 1e3, 1.0, 1.0)] * n
    outs = []
    for h in hosts + devs:
        b = ctx.batch([ph] * n, [h] * n)
        b.set_precision(sdfc.PRECISION_MIXED)
        outs.append(b.evaluate(EA, phiA, EB, phiB, prm, want_deriv=True))
        b.close()
    assert (outs[0][3] > 0).all()
    # the same storage from either upload: bit for bit; across storages (the mixed path's FP32
    # algebra compiled for each): 1e-8 relative, identical active counts and statuses
    for a, b in ((0, 2), (1, 3)):
        assert all(np.array_equal(x, y) for x, y in zip(outs[a], outs[b]))
    assert np.array_equal(outs[0][3], outs[1][3]) and np.array_equal(outs[0][4], outs[1][4])
    for name, k in (("fm", 0), ("Km", 1), ("Dm", 2)):
        assert_close(name, outs[1][k], outs[0][k], rel=1e-8)
    bad = d.clone()
    bad[3, 4, 5] = float("nan")
    torch.cuda.synchronize()
    with pytest.raises(sdfc.SdfcError, match="non-finite"):
        ctx.upload_grid_device(bad.data_ptr(), g.shape, g.min_box, g.max_box, g.dx, 0.01, sdfc.STORAGE_F32_NODES)
    torch.cuda.synchronize()


def test_broad_phase_keeps_active_sets(sdfc, ctx, oracle, workloads):
    """A point cloud much larger than the grid box (most of its tiles far from the box, some
    straddling a face, some inside), posed so that parts of it cross the box: active sets equal
    the oracle's (the reference's detection) for every instance and storage, and instances whose
    cloud lies wholly outside report none."""
    rng = np.random.default_rng(77)
    g = workloads.socket_grid(32, dtype=np.float32)
    pts = rng.uniform(-3.0, 3.0, size=(60000, 3)).astype(np.float32).astype(np.float64)
    ph = ctx.upload_points(pts, 1)
    hs = [ctx.upload_grid(g.values, g.min_box, g.max_box, g.dx, 0.01, st)
          for st in (sdfc.STORAGE_F32, sdfc.STORAGE_F32_NODES)]
    n = 6
    offs = [[0, 0, 0], [2.2, 0, 0], [0, -2.9, 1.1], [4.5, 0.3, 0.0], [9.0, 9.0, 9.0], [-3.1, 3.0, -2.0]]
    EA = np.stack([workloads.pose(workloads.rotvec_to_matrix(rng.normal(size=3) * 0.3), o) for o in offs])
    EB = np.tile(np.eye(4), (n, 1, 1))
    phiA = np.zeros((n, 6))
    phiB = np.zeros((n, 6))
    og = oracle.Grid(g.values, g.min_box, g.max_box, g.dx, 0.01)
    op = oracle.Params(1e5, 0.0, 0.0, 0.0)
    prm = sdfc.Params(1e5, 0.0, 0.0, 0.0)
    for h in hs:
        for k in range(n):
            _, _, _, nact = ctx.evaluate(ph, h, EA[k], phiA[k], EB[k], phiB[k], prm, want_deriv=False)
            _, _, _, rids = oracle.pair_eval(og, pts, EA[k], phiA[k], EB[k], phiB[k], op, False)
            assert nact == len(rids), (k, nact, len(rids))
            assert np.array_equal(ctx.active_ids(), rids), k
        assert len(oracle.pair_eval(og, pts, EA[4], phiA[4], EB[4], phiB[4], op, False)[3]) == 0
