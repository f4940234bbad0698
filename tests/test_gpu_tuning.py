"""Launch configurations of the force pass (sdfc_tuning) and the autotuner, through the C ABI.

Every configuration (persistent 128-thread CTAs or one-warp workers over the (instance, share)
items, or a grid of one CTA per item; at most 1-128 shares per instance, 1-32 chunks per share)
must give the reference's
results at the parity bars (FP64: fm 1e-10, Km and Dm 1e-6; mixed precision 1e-5, in the
reference's relative-error convention) with identical active sets, and be bit-reproducible run
to run, also when it replaces a configuration the batch already evaluated with.  The
autotuner must choose one of them, keep it for the batch and reuse it for batches of the same
shape; a sim must step the same trajectory with either force-pass form."""
import numpy as np
import pytest

from _helpers import assert_close
from conftest import submodule

pytestmark = pytest.mark.gpu

CONFIGS = [(variant, slots, per) for variant in (0, 1, 2) for slots, per in ((1, 1), (4, 1), (32, 1), (32, 4), (8, 32))]


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
def case(sdfc, ctx, oracle, workloads):
    """Uneven instances (two grids, three point sets) and the oracle's FP64 results."""
    rng = np.random.default_rng(4)
    g = workloads.socket_grid(56, dtype=np.float32)
    g2 = workloads.socket_grid(40, dtype=np.float32)
    gh = [ctx.upload_grid(g.values, g.min_box, g.max_box, g.dx, 0.01, 1),
          ctx.upload_grid(g2.values, g2.min_box, g2.max_box, g2.dx, 0.01, sdfc.STORAGE_F32_NODES)]
    psets = [workloads.peg_points(n, seed=s) for n, s in ((30000, 1), (2500, 2), (9000, 3))]
    ph = [ctx.upload_points(p, 1) for p in psets]
    inst = [(0, 0), (1, 1), (2, 0), (0, 1), (1, 0), (2, 1), (0, 0)]
    n = len(inst)
    ang = rng.uniform(0, 2 * np.pi, n)
    EA = np.stack([workloads.pose(workloads.rotvec_to_matrix(rng.normal(size=3) * 0.004),
                                  [0.027 * np.cos(a), 0.027 * np.sin(a), 0.25 * rng.normal()]) for a in ang])
    EB = np.tile(np.eye(4), (n, 1, 1))
    phiA = rng.normal(size=(n, 6)) * 0.3
    phiB = np.zeros((n, 6))
    prm = [sdfc.Params(1e5, [1e3, 1e1][k % 2], 0.3, 1e3, 1.0, 1.0) for k in range(n)]
    ogs = [oracle.Grid(x.values, x.min_box, x.max_box, x.dx, 0.01) for x in (g, g2)]
    ref = []
    for k, (a, c) in enumerate(inst):
        op = oracle.Params(prm[k].kn, prm[k].kt, prm[k].mu, prm[k].damping)
        ref.append(oracle.pair_eval(ogs[c], psets[a], EA[k], phiA[k], EB[k], phiB[k], op, True))
    return dict(points=[ph[a] for a, _ in inst], grids=[gh[c] for _, c in inst], states=(EA, phiA, EB, phiB),
                prm=prm, ref=ref)


@pytest.mark.parametrize("variant,slots,per", CONFIGS)
@pytest.mark.parametrize("precision", [0, 1])
def test_configuration_matches_oracle(sdfc, ctx, case, variant, slots, per, precision):
    b = ctx.batch(case["points"], case["grids"])
    try:
        b.set_precision(precision)
        EA, phiA, EB, phiB = case["states"]
        # an evaluation with the default configuration first: the new one must replace it
        b.evaluate(EA, phiA, EB, phiB, case["prm"], want_deriv=True)
        b.set_tuning(slots, variant, chunks_per_slot=per)
        t = b.tuning()
        assert (t["slots"], t["chunks_per_slot"]) == (slots, per)
        out = b.evaluate(EA, phiA, EB, phiB, case["prm"], want_deriv=True)
        fm, Km, Dm, nact, st = out
        assert not st.any()
        fbar, jbar = (1e-10, 1e-6) if precision == 0 else (1e-5, 1e-5)
        for k, (rf, rK, rD, rids) in enumerate(case["ref"]):
            assert nact[k] == len(rids) > 0
            assert_close(f"inst {k} fm", fm[k], rf, rel=fbar, abs_=1e-9)
            assert_close(f"inst {k} Km", Km[k], rK, rel=jbar, abs_=1e-9)
            assert_close(f"inst {k} Dm", Dm[k], rD, rel=jbar, abs_=1e-9)
        again = b.evaluate(EA, phiA, EB, phiB, case["prm"], want_deriv=True)
        assert all(np.array_equal(x, y) for x, y in zip(out, again))
        fv, _, _, nv, _ = b.evaluate(EA, phiA, EB, phiB, case["prm"], want_deriv=False)
        assert np.array_equal(nv, nact)
        for k, (rf, _, _, _) in enumerate(case["ref"]):
            assert_close(f"inst {k} fm value", fv[k], rf, rel=fbar, abs_=1e-9)
    finally:
        b.close()


def test_autotune_chooses_and_reuses(sdfc, ctx, case):
    torch = pytest.importorskip("torch")
    EA, phiA, EB, phiB = case["states"]
    n = len(case["points"])
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()  # noqa: E731
    dEA, dphiA, dEB, dphiB = dev(EA), dev(phiA), dev(EB), dev(phiB)
    dprm = dev(np.stack([p.as_row() for p in case["prm"]]))
    fm = torch.zeros(n, 12, dtype=torch.float64, device="cuda")
    Km = torch.zeros(n, 144, dtype=torch.float64, device="cuda")
    Dm = torch.zeros(n, 144, dtype=torch.float64, device="cuda")
    nact = torch.zeros(n, dtype=torch.int32, device="cuda")
    st = torch.zeros(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    ptrs = (dEA.data_ptr(), dphiA.data_ptr(), dEB.data_ptr(), dphiB.data_ptr(), dprm.data_ptr(), fm.data_ptr(),
            Km.data_ptr(), Dm.data_ptr(), nact.data_ptr(), st.data_ptr())
    chosen = []
    for _ in range(2):  # the second batch has the first's shape: it takes the same tuning
        b = ctx.batch(case["points"], case["grids"])
        b.set_precision(1)
        t = b.autotune(*ptrs, want_deriv=True)
        assert t["slots"] in (1, 2, 4, 8, 16, 32, 64, 128) and t["force_variant"] in ("ctas", "workers", "grid")
        assert t["ms"] > 0
        assert t["chunks_per_slot"] in (1, 2, 4, 8, 16, 32)
        assert b.tuning() == t
        torch.cuda.synchronize()
        out = b.evaluate(EA, phiA, EB, phiB, case["prm"], want_deriv=True)
        for k, (rf, rK, _, rids) in enumerate(case["ref"]):
            assert out[3][k] == len(rids)
            assert_close(f"inst {k} fm", out[0][k], rf, rel=1e-5, abs_=1e-9)
            assert_close(f"inst {k} Km", out[1][k], rK, rel=1e-5, abs_=1e-9)
        chosen.append(t)
        b.close()
    assert chosen[0] == chosen[1]


@pytest.mark.parametrize("precision,atol", [(0, 1e-10), (1, 1e-7)])
def test_sim_workers_match_ctas(sdfc, ctx, workloads, precision, atol):
    """A direction sweep stepped with each force-pass form (and after sdfc_sim_autotune): the
    same trajectories up to the sums' grouping."""
    g = workloads.socket_grid(48, dtype=np.float32)
    gh = ctx.upload_grid(g.values, g.min_box, g.max_box, g.dx, 0.01, 1)
    ph = ctx.upload_points(workloads.peg_points(8000, seed=6), 1)
    n = 24
    dirs = workloads.fibonacci_directions(n)
    m, inertia = workloads.cylinder_mass_props()
    H = float(np.float32(5e-3))
    mover = sdfc.Mover.make(m, inertia, np.eye(4), H, (0.0, 0.0, -9.8))
    prm = sdfc.Params(1e5, 1e3, 0.3, 1e3)
    F = np.zeros((n, 6))
    F[:, 3:] = dirs

    def run(tune):
        sim = ctx.sim([mover] * n, [sdfc.ScenePair.make(i, ph, gh, True, np.eye(4), prm) for i in range(n)])
        try:
            sim.set_precision(precision)
            sim.set_state(np.zeros((n, 3)), np.zeros((n, 3)))
            sim.set_external_force(F)
            t = tune(sim)
            qs = []
            for _ in range(4):
                sim.step(5)
                qs.append(sim.get_state()[0])
            return np.stack(qs), t
        finally:
            sim.close()

    q_ctas, _ = run(lambda s: s.set_tuning(4, sdfc.FORCE_CTAS))
    q_work, _ = run(lambda s: s.set_tuning(8, sdfc.FORCE_WORKERS, chunks_per_slot=2))
    q_grid, _ = run(lambda s: s.set_tuning(4, sdfc.FORCE_GRID))
    q_auto, t = run(lambda s: s.autotune())
    assert t["slots"] in (1, 2, 4, 8, 16, 32)
    assert np.abs(q_ctas).max() > 1e-3  # the pegs move
    np.testing.assert_allclose(q_work, q_ctas, rtol=0, atol=atol)
    np.testing.assert_allclose(q_grid, q_ctas, rtol=0, atol=atol)
    np.testing.assert_allclose(q_auto, q_ctas, rtol=0, atol=atol)


@pytest.mark.parametrize("variant,slots,per", [(0, 32, 1), (0, 32, 4), (1, 32, 2), (2, 4, 1), (2, 32, 1)])
def test_heavy_instance_among_empty_ones(sdfc, ctx, oracle, workloads, variant, slots, per):
    """One instance with tens of thousands of active contacts (spread over many shares), one
    with a few hundred, and 30 whose point sets lie away from the grid (no contact: no share, no
    item, zero outputs): every form gives the oracle's results."""
    rng = np.random.default_rng(9)
    g = workloads.socket_grid(64, dtype=np.float32)
    gh = ctx.upload_grid(g.values, g.min_box, g.max_box, g.dx, 0.01, 1)
    heavy = workloads.peg_points(120000, seed=5)
    light = workloads.peg_points(3000, seed=6)
    ph, pl = ctx.upload_points(heavy, 1), ctx.upload_points(light, 1)
    n = 32
    points = [ph, pl] + [pl] * (n - 2)
    EA = np.tile(np.eye(4), (n, 1, 1))
    EA[0] = workloads.pose(workloads.rotvec_to_matrix([0.0, 0.003, 0.0]), [0.028, 0.0, 0.0])
    EA[1] = workloads.pose(workloads.rotvec_to_matrix([0.002, 0.0, 0.0]), [0.0, 0.027, 0.1])
    for k in range(2, n):
        EA[k, :3, 3] = [5.0 + k, 3.0, -4.0]  # far outside the grid box
    EB = np.tile(np.eye(4), (n, 1, 1))
    phiA = rng.normal(size=(n, 6)) * 0.2
    phiB = np.zeros((n, 6))
    prm = [sdfc.Params(1e5, 1e3, 0.3, 1e3, 1.0, 1.0)] * n
    b = ctx.batch(points, [gh] * n)
    try:
        b.set_precision(1)
        b.set_tuning(slots, variant, chunks_per_slot=per)
        fm, Km, Dm, nact, st = b.evaluate(EA, phiA, EB, phiB, prm, want_deriv=True)
    finally:
        b.close()
    assert not st.any()
    assert nact[0] > 20000 and 0 < nact[1] < 5000 and not nact[2:].any(), nact[:3]
    assert not fm[2:].any() and not Km[2:].any() and not Dm[2:].any()
    og = oracle.Grid(g.values, g.min_box, g.max_box, g.dx, 0.01)
    op = oracle.Params(1e5, 1e3, 0.3, 1e3, 1.0, 1.0)
    for k, pts in ((0, heavy), (1, light)):
        rf, rK, rD, rids = oracle.pair_eval(og, pts, EA[k], phiA[k], EB[k], phiB[k], op, True)
        assert nact[k] == len(rids)
        assert_close(f"inst {k} fm", fm[k], rf, rel=1e-5, abs_=1e-9)
        assert_close(f"inst {k} Km", Km[k], rK, rel=1e-5, abs_=1e-9)
        assert_close(f"inst {k} Dm", Dm[k], rD, rel=1e-5, abs_=1e-9)
