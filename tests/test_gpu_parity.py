"""GPU parity: libsdfcontact (through its C ABI) against the reference's golden
vectors and the oracle restatement on the same seeded inputs.

Bars, in the reference's relative-error convention (simulation/redmax/Utils.h:362-381):
  * the active contact set is identical (the reference's ids, ascending);
  * stencil mode (the reference's own 26-query SDF difference stencil,
    evaluated bit-identically): fm to 1e-12, Km and Dm to 1e-10;
  * analytic mode (default; analytic cell derivatives of the interpolant where
    the stencil stays in one cell): fm to 1e-10, Km and Dm to 1e-6.  The
    reference's Hessian is a second difference with step 1e-5, so its own
    round-off is about ulp(SDF) / 1e-10, which reaches Km through the
    d * dn/dq terms; 1e-6 covers penetrations of a few tenths;
  * mixed precision (FP64 depth and sums, FP32 per-contact algebra): fm, Km
    and Dm to 1e-5, the bar the batched throughput path is held to.
"""
import numpy as np
import pytest

from _helpers import assert_close, load, rel_err
from conftest import submodule

pytestmark = pytest.mark.gpu

FM_REL = 1e-10
JAC_REL = 1e-6
FM_REL_STENCIL = 1e-12
JAC_REL_STENCIL = 1e-10
MIXED_REL = 1e-5


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
    return load("pair_eval.npz")


def params_of(sdfc, row):
    return sdfc.Params(*[float(x) for x in row])


@pytest.mark.parametrize("storage", [0, 1])
def test_golden_single_pair(sdfc, ctx, fx, storage):
    grid = ctx.upload_grid(fx["grid"], fx["min_box"], fx["max_box"], fx["dx"], float(fx["col_th"]), storage)
    pts = ctx.upload_points(fx["points"], storage)
    for k in range(len(fx["fm"])):
        prm = params_of(sdfc, fx["params"][k])
        args = (pts, grid, fx["EA"][k], fx["phiA"][k], fx["EB"][k], fx["phiB"][k], prm)
        fm_v, _, _, n_v = ctx.evaluate(*args, want_deriv=False)
        ids_v = ctx.active_ids()
        fm, Km, Dm, n = ctx.evaluate(*args, want_deriv=True)
        ids = ctx.active_ids()
        ref_ids = fx["ids"][k][: fx["n_active"][k]]
        assert n == n_v == len(ref_ids)
        assert np.array_equal(ids, ref_ids) and np.array_equal(ids_v, ref_ids), f"case {k}"
        assert_close(f"case {k} fm value", fm_v, fx["fm_v"][k], rel=FM_REL)
        assert_close(f"case {k} fm", fm, fx["fm"][k], rel=FM_REL)
        assert_close(f"case {k} Km", Km, fx["Km"][k], rel=JAC_REL)
        assert_close(f"case {k} Dm", Dm, fx["Dm"][k], rel=JAC_REL)


def test_golden_stencil_mode(sdfc, ctx, fx):
    grid = ctx.upload_grid(fx["grid"], fx["min_box"], fx["max_box"], fx["dx"], float(fx["col_th"]), 1)
    pts = ctx.upload_points(fx["points"], 1)
    ctx.set_derivative_mode(sdfc.DERIV_STENCIL)
    try:
        for k in range(len(fx["fm"])):
            prm = params_of(sdfc, fx["params"][k])
            args = (pts, grid, fx["EA"][k], fx["phiA"][k], fx["EB"][k], fx["phiB"][k], prm)
            fm_v, _, _, _ = ctx.evaluate(*args, want_deriv=False)
            fm, Km, Dm, n = ctx.evaluate(*args, want_deriv=True)
            assert n == fx["n_active"][k]
            assert_close(f"case {k} fm value", fm_v, fx["fm_v"][k], rel=FM_REL_STENCIL)
            assert_close(f"case {k} fm", fm, fx["fm"][k], rel=FM_REL_STENCIL)
            assert_close(f"case {k} Km", Km, fx["Km"][k], rel=JAC_REL_STENCIL)
            assert_close(f"case {k} Dm", Dm, fx["Dm"][k], rel=JAC_REL_STENCIL)
    finally:
        ctx.set_derivative_mode(sdfc.DERIV_ANALYTIC)


def test_golden_batch_equals_single(sdfc, ctx, fx):
    grid = ctx.upload_grid(fx["grid"], fx["min_box"], fx["max_box"], fx["dx"], float(fx["col_th"]), 1)
    pts = ctx.upload_points(fx["points"], 1)
    n = len(fx["fm"])
    b = ctx.batch([pts] * n, [grid] * n)
    prms = [params_of(sdfc, fx["params"][k]) for k in range(n)]
    fm, Km, Dm, nact, st = b.evaluate(fx["EA"], fx["phiA"], fx["EB"], fx["phiB"], prms, want_deriv=True)
    assert not st.any()
    for k in range(n):
        assert nact[k] == fx["n_active"][k]
        assert_close(f"batch {k} fm", fm[k], fx["fm"][k], rel=FM_REL)
        assert_close(f"batch {k} Km", Km[k], fx["Km"][k], rel=JAC_REL)
        assert_close(f"batch {k} Dm", Dm[k], fx["Dm"][k], rel=JAC_REL)
    # deterministic: a second evaluation is bit-identical
    fm2, Km2, Dm2, _, _ = b.evaluate(fx["EA"], fx["phiA"], fx["EB"], fx["phiB"], prms, want_deriv=True)
    assert np.array_equal(fm, fm2) and np.array_equal(Km, Km2) and np.array_equal(Dm, Dm2)
    b.close()


def test_oracle_larger_uneven_batch(sdfc, ctx, oracle, workloads):
    """Uneven instances (different point sets and grids) in one batch, against the oracle."""
    rng = np.random.default_rng(42)
    g64 = workloads.socket_grid(64, dtype=np.float64)
    g40 = workloads.socket_grid(40, dtype=np.float32)
    grids = [(ctx.upload_grid(g.values, g.min_box, g.max_box, g.dx, 0.01, st), g)
             for g, st in ((g64, 0), (g40, 1))]
    psets = [workloads.peg_points(n, seed=s) for n, s in ((20000, 1), (3000, 2), (9000, 3))]
    phs = [ctx.upload_points(p, 1) for p in psets]
    inst = [(0, 0), (1, 1), (2, 0), (0, 1), (1, 0), (2, 1)]
    b = ctx.batch([phs[a] for a, _ in inst], [grids[c][0] for _, c in inst])
    n = len(inst)
    ang = rng.uniform(0, 2 * np.pi, n)  # lateral push of 0.03 > clearance 0.01 + col_th 0.01
    EA = np.stack([workloads.pose(workloads.rotvec_to_matrix(rng.normal(size=3) * 0.005),
                                  [0.03 * np.cos(a), 0.03 * np.sin(a), 0.2 * rng.normal()]) for a in ang])
    EB = np.stack([np.eye(4)] * n)
    phiA = rng.normal(size=(n, 6)) * 0.3
    phiB = np.zeros((n, 6))
    prm = [sdfc.Params(1e5, [1e3, 1e1][k % 2], 0.3, 1e3, 1.0, 1.0) for k in range(n)]
    fm, Km, Dm, nact, st = b.evaluate(EA, phiA, EB, phiB, prm, want_deriv=True)
    assert not st.any()
    for k, (a, c) in enumerate(inst):
        g = grids[c][1]
        og = oracle.Grid(g.values, g.min_box, g.max_box, g.dx, 0.01)
        op = oracle.Params(prm[k].kn, prm[k].kt, prm[k].mu, prm[k].damping, 1.0, 1.0)
        rf, rK, rD, rids = oracle.pair_eval(og, psets[a], EA[k], phiA[k], EB[k], phiB[k], op, True)
        assert nact[k] == len(rids) and len(rids) > 0
        assert_close(f"inst {k} fm", fm[k], rf, rel=FM_REL)
        assert_close(f"inst {k} Km", Km[k], rK, rel=JAC_REL)
        assert_close(f"inst {k} Dm", Dm[k], rD, rel=JAC_REL)
    b.close()


def test_edge_cases(sdfc, ctx, oracle, workloads):
    g = workloads.socket_grid(16, dtype=np.float32)
    grid = ctx.upload_grid(g.values, g.min_box, g.max_box, g.dx, 0.01, 1)
    og = oracle.Grid(g.values, g.min_box, g.max_box, g.dx, 0.01)
    prm = sdfc.Params(1e5, 1e3, 0.3, 1e3)
    op = oracle.Params(1e5, 1e3, 0.3, 1e3)
    I, z = np.eye(4), np.zeros(6)
    # empty point set
    empty = ctx.upload_points(np.zeros((0, 3)), 1)
    fm, Km, Dm, n = ctx.evaluate(empty, grid, I, z, I, z, prm)
    assert n == 0 and not fm.any() and not Km.any() and not Dm.any()
    # every point outside the grid box: nothing active
    far = ctx.upload_points(np.full((100, 3), 7.0), 1)
    fm, Km, Dm, n = ctx.evaluate(far, grid, I, z, I, z, prm)
    assert n == 0 and not fm.any()
    # points a few hundredths of a cell from grid nodes (their stencils stay in the cell; contacts
    # whose stencil crosses faces: test_contacts_near_cell_faces)
    ax = g.min_box[0] + g.dx[0] * np.arange(3, 13)
    P = np.array([[x, y, zz] for x in ax[::3] for y in ax[::3] for zz in ax]).astype(np.float32).astype(np.float64)
    P = P[np.abs(workloads.socket_sdf(P)) < 0.3]
    nodes = ctx.upload_points(P, 1)
    EA = workloads.pose(p=[0.004, -0.003, 0.002])
    fm, Km, Dm, n = ctx.evaluate(nodes, grid, EA, z, I, z, prm)
    rf, rK, rD, rids = oracle.pair_eval(og, P, EA, z, I, z, op, True)
    assert n == len(rids) and n > 0
    assert np.array_equal(ctx.active_ids(), rids)
    assert_close("nodes fm", fm, rf, rel=FM_REL)
    assert_close("nodes Km", Km, rK, rel=JAC_REL)
    assert_close("nodes Dm", Dm, rD, rel=JAC_REL)
    # mixed precision on the same contacts
    ctx.set_precision(sdfc.PRECISION_MIXED)
    for deriv in (True, False):
        fm, Km, Dm, n = ctx.evaluate(nodes, grid, EA, z, I, z, prm, want_deriv=deriv)
        assert n == len(rids)
        assert_close(f"nodes fm (mixed, deriv={deriv})", fm, rf, rel=MIXED_REL)
        if deriv:
            assert_close("nodes Km (mixed)", Km, rK, rel=MIXED_REL)
            assert_close("nodes Dm (mixed)", Dm, rD, rel=MIXED_REL)
    ctx.set_precision(sdfc.PRECISION_FP64)
    ctx.set_derivative_mode(sdfc.DERIV_STENCIL)
    fm, Km, Dm, n = ctx.evaluate(nodes, grid, EA, z, I, z, prm)
    ctx.set_derivative_mode(sdfc.DERIV_ANALYTIC)
    assert_close("nodes fm (stencil)", fm, rf, rel=FM_REL_STENCIL)
    assert_close("nodes Km (stencil)", Km, rK, rel=JAC_REL_STENCIL)
    assert_close("nodes Dm (stencil)", Dm, rD, rel=JAC_REL_STENCIL)
    # minimal 2x2x2 grid
    v = np.array([-0.1, 0.2, 0.1, 0.3, 0.0, 0.4, 0.2, 0.5]).reshape(2, 2, 2)
    tiny = ctx.upload_grid(v, [0, 0, 0], [1, 1, 1], [1, 1, 1], 0.0, 0)
    Q = np.random.default_rng(0).uniform(0, 1, (500, 3))
    qp = ctx.upload_points(Q, 0)
    fm, Km, Dm, n = ctx.evaluate(qp, tiny, I, z, I, z, prm)
    rf, rK, rD, rids = oracle.pair_eval(oracle.Grid(v, [0, 0, 0], [1, 1, 1], [1, 1, 1], 0.0), Q, I, z, I, z, op, True)
    assert n == len(rids)
    assert_close("tiny fm", fm, rf, rel=FM_REL)
    assert_close("tiny Km", Km, rK, rel=JAC_REL)


def near_face_cells(rng, shape, mn, dx, count):
    """Grid-frame points whose derivative stencil (BodySDFObj.cpp:176-205, steps 1e-5 and 5e-6)
    reaches across faces of their cell: on one, two or three axes (faces, edges, corners), on
    either side, at distances from the face of 0 to just past the stencil's reach (1e-5 and the
    1.0001e-5 band the FP32 classification rounds to), some in the grid's outermost cells, where
    the next layer of nodes does not exist."""
    dists = (0.0, 2.5e-6, 4.9e-6, 5.1e-6, 9.9e-6, 1e-5 - 1e-9, 1.00005e-5, 1.05e-5)
    pts = []
    for q in range(count):
        cell = np.array([rng.integers(0, n - 1) for n in shape])
        f = rng.uniform(0.15, 0.85, 3)
        axes = rng.choice(3, 1 + q % 3, replace=False)
        for m, a in enumerate(axes):
            d = dists[rng.integers(len(dists))] / dx[a]
            up = rng.random() < 0.5
            if q % 7 == 0 and m == 0:  # toward the grid's outside
                cell[a] = shape[a] - 2 if up else 0
            f[a] = 1.0 - d if up else d
        pts.append(mn + dx * (cell + f))
    return np.array(pts)


@pytest.mark.parametrize("point_storage", [0, 1])
@pytest.mark.parametrize("grid_storage", [0, 1, 3])
def test_contacts_near_cell_faces(sdfc, ctx, oracle, workloads, grid_storage, point_storage):
    """Single contacts whose derivative stencil crosses faces of their cell, each one instance of
    a batch, against the oracle (the reference's stencil) per contact.  The FP64 path takes the
    reference's own stencil there; the mixed path its closed form (cell derivatives plus the
    face-crossing terms).  The grid is anisotropic (12 x 10 x 14 nodes, three spacings) and its
    values curve along every axis, so every second difference the closed form uses is nonzero;
    every node lies below -col_th, so every contact inside the grid box is active."""
    rng = np.random.default_rng(1234)
    shape = (12, 10, 14)
    mn, mx = np.array([0.0, 0.0, 0.0]), np.array([0.25, 0.2, 0.3])
    dx = (mx - mn) / (np.array(shape) - 1)
    ax = [mn[a] + dx[a] * np.arange(shape[a]) for a in range(3)]
    Z, Y, X = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    S = np.array([1.0, 1.3, 0.8])
    c = np.array([0.11, 0.1, 0.16])
    vals = np.sqrt((((np.stack([X, Y, Z], -1) - c) * S) ** 2).sum(-1)) - 0.3
    vals = vals.astype(np.float32).astype(np.float64)  # (nk, nj, ni)
    assert vals.max() < -0.05
    gh = ctx.upload_grid(vals, mn, mx, dx, 0.01, grid_storage)
    og = oracle.Grid(vals, mn, mx, dx, 0.01)
    xs = near_face_cells(rng, shape, mn, dx, 180)
    n = len(xs)
    EB = np.stack([workloads.pose(workloads.rotvec_to_matrix(rng.normal(size=3) * 0.4), rng.normal(size=3))
                   for _ in range(n)])
    EA = np.stack([workloads.pose(workloads.rotvec_to_matrix(rng.normal(size=3) * 0.4), rng.normal(size=3))
                   for _ in range(n)])
    # body-A points that the poses carry onto the grid-frame points (x_B = E_B^-1 E_A p)
    P = np.einsum("nij,nj->ni", np.linalg.inv(EA) @ EB, np.c_[xs, np.ones(n)])[:, :3]
    if point_storage == 1:
        P = P.astype(np.float32).astype(np.float64)
    phs = [ctx.upload_points(P[k:k + 1], point_storage) for k in range(n)]
    phiA = rng.normal(size=(n, 6)) * 0.2
    phiB = rng.normal(size=(n, 6)) * 0.1
    prm = [sdfc.Params(1e5, 1e3, 0.3, 1e3, 1.0, 1.0)] * n
    op = oracle.Params(1e5, 1e3, 0.3, 1e3, 1.0, 1.0)
    ref = [oracle.pair_eval(og, P[k:k + 1], EA[k], phiA[k], EB[k], phiB[k], op, True) for k in range(n)]
    # (FP32 point storage can round a point on the grid box's face to outside it: no contact, as
    # in the reference)
    active = np.array([len(r[3]) for r in ref])
    assert active.sum() >= 0.95 * n
    b = ctx.batch(phs, [gh] * n)
    try:
        for precision, stencil, rel_f, rel_j in ((0, 0, FM_REL, JAC_REL), (0, 1, FM_REL_STENCIL, JAC_REL_STENCIL),
                                                 (1, 0, MIXED_REL, MIXED_REL)):
            b.set_precision(precision)
            b.set_derivative_mode(stencil)
            fm, Km, Dm, nact, st = b.evaluate(EA, phiA, EB, phiB, prm, want_deriv=True)
            assert np.array_equal(nact, active) and not st.any()
            for k in range(n):
                rf, rK, rD, _ = ref[k]
                tag = f"contact {k} at {xs[k]} (precision {precision}, stencil {stencil})"
                assert_close(f"{tag} fm", fm[k], rf, rel=rel_f)
                assert_close(f"{tag} Km", Km[k], rK, rel=rel_j)
                assert_close(f"{tag} Dm", Dm[k], rD, rel=rel_j)
            fv, _, _, nv, _ = b.evaluate(EA, phiA, EB, phiB, prm, want_deriv=False)
            assert np.array_equal(nv, active)
            for k in range(n):
                assert_close(f"value pass {k}", fv[k], ref[k][0], rel=rel_f)
    finally:
        b.close()


def test_invalid_arguments(sdfc, ctx):
    with pytest.raises(sdfc.SdfcError):
        ctx.upload_grid(np.zeros((4, 4, 4)), [0, 0, 0], [5, 5, 5], [1, 1, 1], 0.0)  # box past the last node
    with pytest.raises(sdfc.SdfcError):
        ctx.upload_grid(np.full((4, 4, 4), np.nan), [0, 0, 0], [3, 3, 3], [1, 1, 1], 0.0)
    with pytest.raises(sdfc.SdfcError):
        ctx.batch([12345], [0])


def test_mixed_precision_golden(sdfc, ctx, fx):
    grid = ctx.upload_grid(fx["grid"], fx["min_box"], fx["max_box"], fx["dx"], float(fx["col_th"]), 1)
    pts = ctx.upload_points(fx["points"], 1)
    n = len(fx["fm"])
    b = ctx.batch([pts] * n, [grid] * n)
    b.set_precision(sdfc.PRECISION_MIXED)
    prms = [params_of(sdfc, fx["params"][k]) for k in range(n)]
    fm, Km, Dm, nact, st = b.evaluate(fx["EA"], fx["phiA"], fx["EB"], fx["phiB"], prms, want_deriv=True)
    fmv, _, _, nactv, _ = b.evaluate(fx["EA"], fx["phiA"], fx["EB"], fx["phiB"], prms, want_deriv=False)
    assert not st.any()
    worst = {"fm": 0.0, "Km": 0.0, "Dm": 0.0}
    for k in range(n):
        assert nact[k] == nactv[k] == fx["n_active"][k]
        assert_close(f"mixed {k} fm value", fmv[k], fx["fm_v"][k], rel=MIXED_REL, abs_=1e-9)
        for name, a, ref in (("fm", fm[k], fx["fm"][k]), ("Km", Km[k], fx["Km"][k]), ("Dm", Dm[k], fx["Dm"][k])):
            assert_close(f"mixed {k} {name}", a, ref, rel=MIXED_REL, abs_=1e-9)
            worst[name] = max(worst[name], rel_err(a, ref)[0])
    print("mixed-precision worst relative error vs the reference:", worst)
    b.close()


def test_mixed_precision_uneven_batch(sdfc, ctx, oracle, workloads):
    rng = np.random.default_rng(7)
    g = workloads.socket_grid(96, dtype=np.float32)
    gh = ctx.upload_grid(g.values, g.min_box, g.max_box, g.dx, 0.01, 1)
    psets = [workloads.peg_points(n, seed=s) for n, s in ((30000, 4), (5000, 5))]
    phs = [ctx.upload_points(p, 1) for p in psets]
    n = 8
    which = [k % 2 for k in range(n)]
    b = ctx.batch([phs[w] for w in which], [gh] * n)
    b.set_precision(sdfc.PRECISION_MIXED)
    ang = rng.uniform(0, 2 * np.pi, n)
    rel = np.stack([workloads.pose(workloads.rotvec_to_matrix(rng.normal(size=3) * 0.003),
                                   [0.0202 * np.cos(a), 0.0202 * np.sin(a), 0.3 * rng.normal()]) for a in ang])
    # the socket placed in the world too (half the instances), so that the Km columns of
    # body B, which the FP32 path derives from body A's, are checked under a general pose
    EB = np.stack([workloads.pose(workloads.rotvec_to_matrix(rng.normal(size=3) * 0.3), rng.normal(size=3))
                   if k % 2 else np.eye(4) for k in range(n)])
    EA = EB @ rel
    phiA = rng.normal(size=(n, 6)) * 0.2
    phiB = rng.normal(size=(n, 6)) * 0.1
    prm = [sdfc.Params(1e5, [1e3, 1e1][k % 2], 0.3, 1e3, 1.0, 1.0) for k in range(n)]
    fm, Km, Dm, nact, st = b.evaluate(EA, phiA, EB, phiB, prm, want_deriv=True)
    og = oracle.Grid(g.values, g.min_box, g.max_box, g.dx, 0.01)
    for k in range(n):
        op = oracle.Params(prm[k].kn, prm[k].kt, prm[k].mu, prm[k].damping, 1.0, 1.0)
        rf, rK, rD, rids = oracle.pair_eval(og, psets[which[k]], EA[k], phiA[k], EB[k], phiB[k], op, True)
        assert nact[k] == len(rids) > 0
        assert_close(f"inst {k} fm", fm[k], rf, rel=MIXED_REL, abs_=1e-9)
        assert_close(f"inst {k} Km", Km[k], rK, rel=MIXED_REL, abs_=1e-9)
        assert_close(f"inst {k} Dm", Dm[k], rD, rel=MIXED_REL, abs_=1e-9)
    b.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_masked_requests(sdfc, ctx, workloads, precision):
    """Per-instance requests in one launch set (sdfc_batch_evaluate_masked_device):
    0 skip, 1 fm only, 2 fm, Km, Dm.  Every requested instance is bit-identical to a
    plain evaluation of its kind; skipped outputs stay untouched.  Many value
    requests follow derivative ones, so any overlap of the two passes' scratch would
    show; the poses of both bodies are general (rotated and offset)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(9)
    g = workloads.socket_grid(64, dtype=np.float32)
    gh = ctx.upload_grid(g.values, g.min_box, g.max_box, g.dx, 0.01, 1)
    ph = ctx.upload_points(workloads.peg_points(6000, seed=8), 1)
    n = 40
    b = ctx.batch([ph] * n, [gh] * n)
    b.set_precision(precision)
    ang = rng.uniform(0, 2 * np.pi, n)
    EB = np.stack([workloads.pose(workloads.rotvec_to_matrix(rng.normal(size=3) * 0.2), rng.normal(size=3) * 0.3)
                   for _ in range(n)])
    rel = np.stack([workloads.pose(workloads.rotvec_to_matrix(rng.normal(size=3) * 0.004),
                                   [0.025 * np.cos(a), 0.025 * np.sin(a), 0.3 * rng.normal()]) for a in ang])
    EA = EB @ rel  # the peg pressed into the socket, both placed in the world
    phiA = rng.normal(size=(n, 6)) * 0.2
    phiB = rng.normal(size=(n, 6)) * 0.1
    prm = [sdfc.Params(1e5, [1e3, 1e1][k % 2], 0.3, 1e3, 1.0, 1.0) for k in range(n)]
    req = np.array([2, 2] + [1] * 20 + [0, 2, 1] * 6, dtype=np.int32)
    assert len(req) == n
    fm2, Km2, Dm2, n2, _ = b.evaluate(EA, phiA, EB, phiB, prm, want_deriv=True)
    fm1, _, _, n1, _ = b.evaluate(EA, phiA, EB, phiB, prm, want_deriv=False)
    assert (n2 > 0).all()

    dev = torch.device("cuda", 0)
    t = lambda a: torch.tensor(np.ascontiguousarray(a, dtype=np.float64), device=dev)
    dEA, dphiA, dEB, dphiB = t(EA.reshape(n, 16)), t(phiA), t(EB.reshape(n, 16)), t(phiB)
    dprm = t([[p.kn, p.kt, p.mu, p.damping, p.scale, p.contact_scale] for p in prm])
    dreq = torch.tensor(req, device=dev)
    fm = torch.full((n, 12), float("nan"), dtype=torch.float64, device=dev)
    Km = torch.full((n, 144), float("nan"), dtype=torch.float64, device=dev)
    Dm = torch.full((n, 144), float("nan"), dtype=torch.float64, device=dev)
    nact = torch.full((n,), -7, dtype=torch.int32, device=dev)
    st = torch.zeros(n, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    b.evaluate_masked_device(dEA.data_ptr(), dphiA.data_ptr(), dEB.data_ptr(), dphiB.data_ptr(), dprm.data_ptr(),
                             dreq.data_ptr(), fm.data_ptr(), Km.data_ptr(), Dm.data_ptr(), nact.data_ptr(),
                             st.data_ptr(), torch.cuda.current_stream(dev).cuda_stream)
    torch.cuda.synchronize()
    fm, Km, Dm, nact, st = (x.cpu().numpy() for x in (fm, Km, Dm, nact, st))
    assert not st.any()
    for k in range(n):
        if req[k] == 2:
            assert np.array_equal(fm[k], fm2[k]) and nact[k] == n2[k], k
            assert np.array_equal(Km[k], Km2[k].ravel()) and np.array_equal(Dm[k], Dm2[k].ravel()), k
        elif req[k] == 1:
            assert np.array_equal(fm[k], fm1[k]) and nact[k] == n1[k], k
            assert np.isnan(Km[k]).all() and np.isnan(Dm[k]).all(), k
        else:
            assert np.isnan(fm[k]).all() and np.isnan(Km[k]).all() and nact[k] == -7, k
    b.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_f16_bricks_against_oracle(sdfc, ctx, oracle, workloads, precision):
    """FP16-brick grids (SDFC_STORAGE_F16_BRICKS): the evaluations see the decoded grid
    (sdfc_grid_values), so against the oracle on that grid they keep the bars of the other
    storages (identical active sets; FP64 path fm 1e-10, Km/Dm 1e-6; mixed 1e-5).  Against the
    original FP64 grid the error is FP16's; it is bounded loosely here and reported by the bench."""
    rng = np.random.default_rng(21)
    g = workloads.socket_grid(61, dtype=np.float64)  # 61 nodes per axis: partial bricks at the top
    gh = ctx.upload_grid(g.values, g.min_box, g.max_box, g.dx, 0.01, sdfc.STORAGE_F16_BRICKS)
    dec = ctx.grid_values(gh)
    assert np.abs(dec - g.values).max() <= 2.0 ** -11 * np.abs(g.values).max()
    pts = workloads.peg_points(8000, seed=11)
    ph = ctx.upload_points(pts, 1)
    n = 6
    b = ctx.batch([ph] * n, [gh] * n)
    b.set_precision(precision)
    ang = rng.uniform(0, 2 * np.pi, n)
    rel = np.stack([workloads.pose(workloads.rotvec_to_matrix(rng.normal(size=3) * 0.003),
                                   [0.025 * np.cos(a), 0.025 * np.sin(a), 0.3 * rng.normal()]) for a in ang])
    EB = np.stack([workloads.pose(workloads.rotvec_to_matrix(rng.normal(size=3) * 0.3), rng.normal(size=3))
                   for _ in range(n)])
    EA = EB @ rel
    phiA = rng.normal(size=(n, 6)) * 0.2
    phiB = rng.normal(size=(n, 6)) * 0.1
    prm = [sdfc.Params(1e5, 1e3, 0.3, 1e3, 1.0, 1.0) for _ in range(n)]
    fm, Km, Dm, nact, st = b.evaluate(EA, phiA, EB, phiB, prm, want_deriv=True)
    assert not st.any()
    og = oracle.Grid(dec, g.min_box, g.max_box, g.dx, 0.01)
    og64 = oracle.Grid(g.values, g.min_box, g.max_box, g.dx, 0.01)
    op = oracle.Params(1e5, 1e3, 0.3, 1e3, 1.0, 1.0)
    for k in range(n):
        rf, rK, rD, rids = oracle.pair_eval(og, pts, EA[k], phiA[k], EB[k], phiB[k], op, True)
        assert nact[k] == len(rids) > 0
        if precision == 0:
            assert_close(f"inst {k} fm", fm[k], rf, rel=FM_REL)
            assert_close(f"inst {k} Km", Km[k], rK, rel=JAC_REL)
            assert_close(f"inst {k} Dm", Dm[k], rD, rel=JAC_REL)
        else:
            assert_close(f"inst {k} fm", fm[k], rf, rel=MIXED_REL, abs_=1e-9)
            assert_close(f"inst {k} Km", Km[k], rK, rel=MIXED_REL, abs_=1e-9)
            assert_close(f"inst {k} Dm", Dm[k], rD, rel=MIXED_REL, abs_=1e-9)
        f64, _, _, _ = oracle.pair_eval(og64, pts, EA[k], phiA[k], EB[k], phiB[k], op, False)
        assert np.linalg.norm(fm[k] - f64) <= 0.05 * np.linalg.norm(f64)  # FP16 quantisation
    b.close()


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("stencil", [0, 1])
def test_mixed_storage_batch(sdfc, ctx, workloads, precision, stencil):
    """One batch over an FP32 grid, an FP64 grid and an FP16-brick grid: the kernels specialised
    on brick-free grids and the general ones split the instances; every instance equals its
    evaluation in a batch of its own storage alone (bit for bit)."""
    rng = np.random.default_rng(31)
    g = workloads.socket_grid(40, dtype=np.float64)
    hs = [ctx.upload_grid(g.values, g.min_box, g.max_box, g.dx, 0.01, st) for st in (1, 0, sdfc.STORAGE_F16_BRICKS)]
    ph = ctx.upload_points(workloads.peg_points(4000, seed=13), 1)
    n = 9
    grids = [hs[k % 3] for k in range(n)]
    ang = rng.uniform(0, 2 * np.pi, n)
    EA = np.stack([workloads.pose(workloads.rotvec_to_matrix(rng.normal(size=3) * 0.003),
                                  [0.025 * np.cos(a), 0.025 * np.sin(a), 0.3 * rng.normal()]) for a in ang])
    EB = np.tile(np.eye(4), (n, 1, 1))
    phiA = rng.normal(size=(n, 6)) * 0.2
    phiB = np.zeros((n, 6))
    prm = [sdfc.Params(1e5, 1e3, 0.3, 1e3, 1.0, 1.0) for _ in range(n)]

    def run(idx):
        b = ctx.batch([ph] * len(idx), [grids[k] for k in idx])
        b.set_precision(precision)
        b.set_derivative_mode(stencil)
        out = b.evaluate(EA[idx], phiA[idx], EB[idx], phiB[idx], [prm[k] for k in idx], want_deriv=True)
        b.close()
        return out

    fm, Km, Dm, nact, _ = run(list(range(n)))
    assert (nact > 0).all()
    for kind in range(3):
        idx = [k for k in range(n) if k % 3 == kind]
        f1, K1, D1, n1, _ = run(idx)
        assert np.array_equal(fm[idx], f1) and np.array_equal(Km[idx], K1) and np.array_equal(Dm[idx], D1)
        assert np.array_equal(nact[idx], n1)


@pytest.mark.parametrize("precision,bar", [(0, 1e-10), (1, 1e-5)])
def test_energy_against_oracle(sdfc, ctx, oracle, workloads, precision, bar):
    """Penetration energy (sdfc_batch_energy) and its twist gradient against the oracle's
    definition on the same inputs (the oracle's gradient is itself checked against central
    differences of the energy in the CPU tests)."""
    rng = np.random.default_rng(31)
    g = workloads.socket_grid(64, dtype=np.float32)
    gh = ctx.upload_grid(g.values, g.min_box, g.max_box, g.dx, 0.01, 1)
    pts = workloads.peg_points(6000, seed=12)
    ph = ctx.upload_points(pts, 1)
    n = 6
    b = ctx.batch([ph] * n, [gh] * n)
    b.set_precision(precision)
    ang = rng.uniform(0, 2 * np.pi, n)
    rel = np.stack([workloads.pose(workloads.rotvec_to_matrix(rng.normal(size=3) * 0.004),
                                   [0.026 * np.cos(a), 0.026 * np.sin(a), 0.3 * rng.normal()]) for a in ang])
    EB = np.stack([workloads.pose(workloads.rotvec_to_matrix(rng.normal(size=3) * 0.3), rng.normal(size=3))
                   for _ in range(n)])
    EA = EB @ rel
    prm = [sdfc.Params(1e5, 1e3, 0.3, 1e3, 2.0, 0.5) for _ in range(n)]
    e, dE = b.energy(EA, EB, prm)
    og = oracle.Grid(g.values, g.min_box, g.max_box, g.dx, 0.01)
    for k in range(n):
        re, rdE = oracle.pair_energy(og, pts, EA[k], EB[k], oracle.Params(1e5, 1e3, 0.3, 1e3, 2.0, 0.5))
        assert re > 0
        assert abs(e[k] - re) <= bar * re, (k, e[k], re)
        assert np.linalg.norm(dE[k] - rdE) <= bar * np.linalg.norm(rdE), (k, dE[k], rdE)
    b.close()


@pytest.mark.parametrize("precision,bar", [(0, 1e-10), (1, 1e-5)])
def test_energy_many_shares(sdfc, ctx, oracle, workloads, precision, bar):
    """Instances whose contacts fill more shares than the energy pass has CTAs per instance (12k
    active contacts in 1-chunk shares: 94 shares, 16 CTAs each taking several in turn), against
    the oracle.  Every node of the grid lies inside (values below -col_th) and every point in the
    grid box, so every point is an active contact."""
    rng = np.random.default_rng(41)
    shape = (20, 18, 22)
    mn, mx = np.array([0.0, 0.0, 0.0]), np.array([0.25, 0.2, 0.3])
    dx = (mx - mn) / (np.array(shape) - 1)
    ax = [mn[a] + dx[a] * np.arange(shape[a]) for a in range(3)]
    Z, Y, X = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    vals = np.sqrt((((np.stack([X, Y, Z], -1) - [0.11, 0.1, 0.16]) * [1.0, 1.3, 0.8]) ** 2).sum(-1)) - 0.3
    vals = vals.astype(np.float32).astype(np.float64)
    assert vals.max() < -0.05
    gh = ctx.upload_grid(vals, mn, mx, dx, 0.01, 1)
    og = oracle.Grid(vals, mn, mx, dx, 0.01)
    n = 2
    EB = np.stack([workloads.pose(workloads.rotvec_to_matrix(rng.normal(size=3) * 0.5), rng.normal(size=3))
                   for _ in range(n)])
    EA = EB @ np.stack([workloads.pose(workloads.rotvec_to_matrix(rng.normal(size=3) * 0.005), [0.01, -0.01, 0.02])
                        for _ in range(n)])
    # points that both poses carry into the grid box (margin 0.03 for the offsets above)
    xb = rng.uniform(mn + 0.03, mx - 0.03, size=(12000, 3))
    pts = np.einsum("ij,nj->ni", np.linalg.inv(EA[0]) @ EB[0], np.c_[xb, np.ones(len(xb))])[:, :3]
    ph = ctx.upload_points(pts, 0)
    b = ctx.batch([ph] * n, [gh] * n)
    try:
        b.set_precision(precision)
        b.set_tuning(128, sdfc.FORCE_CTAS, 0, 1)
        prm = [sdfc.Params(1e5, 1e3, 0.3, 1e3, 2.0, 0.5)] * n
        e, dE = b.energy(EA, EB, prm)
        for k in range(n):
            re, rdE = oracle.pair_energy(og, pts, EA[k], EB[k], oracle.Params(1e5, 1e3, 0.3, 1e3, 2.0, 0.5))
            nact = len(oracle.pair_eval(og, pts, EA[k], np.zeros(6), EB[k], np.zeros(6),
                                        oracle.Params(1e5, 1e3, 0.3, 1e3, 2.0, 0.5), False)[3])
            assert nact > 16 * 128, (k, nact)  # more 1-chunk shares than the pass's 16 CTAs per instance
            assert abs(e[k] - re) <= bar * re, (k, e[k], re)
            assert np.linalg.norm(dE[k] - rdE) <= bar * np.linalg.norm(rdE), (k, dE[k], rdE)
    finally:
        b.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_host_array_paths_agree(sdfc, workloads, precision):
    """sdfc_batch_evaluate's two host-array paths give the same bits: kernels that read the
    caller's arrays and write its result arrays themselves (where the device reads pageable
    memory), and inputs / results staged through pinned buffers (SDFC_STAGED_COPIES)."""
    import os
    g = workloads.socket_grid(64, dtype=np.float32)
    pts = workloads.peg_points(20000, seed=3)
    n = 16
    EA, phiA, EB, phiB = workloads.direction_sweep_states(n)
    prm = [sdfc.Params(1e5, 1e3, 0.3, 1e3, 1.0, 1.0)] * n
    outs = []
    for staged in (False, True):
        if staged:
            os.environ["SDFC_STAGED_COPIES"] = "1"
        try:
            c = sdfc.Context(0)
        finally:
            os.environ.pop("SDFC_STAGED_COPIES", None)
        gh = c.upload_grid(g.values, g.min_box, g.max_box, g.dx, 0.01, 1)
        ph = c.upload_points(pts, 1)
        b = c.batch([ph] * n, [gh] * n)
        b.set_precision(sdfc.PRECISION_MIXED if precision == "mixed" else sdfc.PRECISION_FP64)
        r = []
        for _ in range(2):  # the second call replays the captured graph
            r.append(b.evaluate(EA, phiA, EB, phiB, prm, want_deriv=True))
        r.append(b.evaluate(EA, phiA, EB, phiB, prm, want_deriv=False))
        outs.append(r)
        b.close()
        c.close()
    (d1, d2, dv), (s1, s2, sv) = outs
    assert d1[3].sum() > 0
    for a, b_ in ((d1, s1), (d2, s2), (d1, d2)):
        for x, y in zip(a, b_):
            np.testing.assert_array_equal(x, y)
    for x, y in zip((dv[0], dv[3], dv[4]), (sv[0], sv[3], sv[4])):
        np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(dv[3], d1[3])


def test_host_array_optional_outputs(sdfc, ctx, workloads):
    """sdfc_batch_evaluate with n_active and status left null (both optional in the ABI): the
    forces are the same as with them."""
    import ctypes
    g = workloads.socket_grid(64, dtype=np.float32)
    gh = ctx.upload_grid(g.values, g.min_box, g.max_box, g.dx, 0.01, 1)
    ph = ctx.upload_points(workloads.peg_points(8000, seed=5), 1)
    n = 8
    EA, phiA, EB, phiB = workloads.direction_sweep_states(n)
    b = ctx.batch([ph] * n, [gh] * n)
    rows = np.tile(sdfc.Params(1e5, 1e3, 0.3, 1e3, 1.0, 1.0).as_row(), (n, 1))
    fm, Km, Dm, nact, st = b.evaluate(EA, phiA, EB, phiB, rows, want_deriv=True)
    assert nact.sum() > 0 and not st.any()
    f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)  # noqa: E731
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
    ins = [f64(EA), f64(phiA), f64(EB), f64(phiB)]
    prm = f64(rows)
    fm2, Km2, Dm2 = np.zeros((n, 12)), np.zeros((n, 12, 12)), np.zeros((n, 12, 12))
    rc = sdfc.lib().sdfc_batch_evaluate(b._h, *(dp(a) for a in ins), prm.ctypes.data_as(ctypes.POINTER(sdfc.Params)),
                                        1, dp(fm2), dp(Km2), dp(Dm2), None, None)
    assert rc == 0
    for x, y in ((fm, fm2), (Km, Km2), (Dm, Dm2)):
        np.testing.assert_array_equal(x, y)
    b.close()
