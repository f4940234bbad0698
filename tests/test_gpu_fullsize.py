"""The headline evaluation at full size (1024 direction-sweep instances x 50k peg points on the
128^3 FP32 socket grid), checked through properties that hold at any size:

  * the mixed-precision path against the FP64 path on every instance: fm, Km, Dm within the
    1e-5 bar (the reference's relative-error convention), identical active counts;
  * determinism: two evaluations of the same inputs are bit-identical;
  * the host-array entry point (a captured graph) equals the device-array one;
  * rigid-motion invariance of the FP64 path: Km's body-B columns equal -(body-A columns) times
    Ad(E_A^-1 E_B) up to FP64 round-off (the identity the FP32 path uses to derive them)."""
import numpy as np
import pytest

from conftest import submodule

pytestmark = pytest.mark.gpu

N, POINTS, GRID = 1024, 50000, 128
PRM = (1e5, 1e3, 0.3, 1e3, 1.0, 1.0)


@pytest.fixture(scope="module")
def setup():
    submodule("build").build()
    sdfc = submodule("sdfc")
    W = submodule("workloads")
    ctx = sdfc.Context(0)
    g = W.socket_grid(GRID, dtype=np.float32)
    gh = ctx.upload_grid(g.values, g.min_box, g.max_box, g.dx, 0.01, sdfc.STORAGE_F32)
    ph = ctx.upload_points(W.peg_points(POINTS, seed=0), sdfc.STORAGE_F32)
    states = W.direction_sweep_states(N)
    yield sdfc, ctx, gh, ph, states
    ctx.close()


def rel(a, b):
    """|a - b| / max(min(|a|, |b|), 1e-4) per instance (Frobenius norms)."""
    a = a.reshape(len(a), -1)
    b = b.reshape(len(b), -1)
    d = np.linalg.norm(a - b, axis=1)
    return d / np.maximum(np.minimum(np.linalg.norm(a, axis=1), np.linalg.norm(b, axis=1)), 1e-4)


def evaluate(sdfc, ctx, gh, ph, states, precision):
    b = ctx.batch([ph] * N, [gh] * N)
    b.set_precision(precision)
    out = b.evaluate(*states, np.tile(np.array(PRM), (N, 1)), want_deriv=True)
    b.close()
    return out


def test_mixed_against_fp64_full_size(setup):
    sdfc, ctx, gh, ph, states = setup
    fm, Km, Dm, nact, st = evaluate(sdfc, ctx, gh, ph, states, sdfc.PRECISION_MIXED)
    fm64, Km64, Dm64, nact64, st64 = evaluate(sdfc, ctx, gh, ph, states, sdfc.PRECISION_FP64)
    assert not st.any() and not st64.any()
    assert np.array_equal(nact, nact64) and (nact > 0).all()
    assert nact.sum() > 1.5e6
    for name, a, b in (("fm", fm, fm64), ("Km", Km, Km64), ("Dm", Dm, Dm64)):
        r = rel(a, b)
        assert r.max() <= 1e-5, (name, r.max(), int(r.argmax()))


def test_deterministic_and_entry_points_agree(setup):
    sdfc, ctx, gh, ph, states = setup
    torch = pytest.importorskip("torch")
    a = evaluate(sdfc, ctx, gh, ph, states, sdfc.PRECISION_MIXED)
    b = evaluate(sdfc, ctx, gh, ph, states, sdfc.PRECISION_MIXED)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    batch = ctx.batch([ph] * N, [gh] * N)
    batch.set_precision(sdfc.PRECISION_MIXED)
    dev = [torch.tensor(np.ascontiguousarray(x, dtype=np.float64), device="cuda") for x in states]
    prm = torch.tensor(np.tile(np.array(PRM), (N, 1)), device="cuda")
    fm = torch.zeros((N, 12), dtype=torch.float64, device="cuda")
    Km = torch.zeros((N, 144), dtype=torch.float64, device="cuda")
    Dm = torch.zeros((N, 144), dtype=torch.float64, device="cuda")
    nact = torch.zeros(N, dtype=torch.int32, device="cuda")
    status = torch.zeros(N, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    batch.evaluate_device(*(t.data_ptr() for t in dev), prm.data_ptr(), fm.data_ptr(), Km.data_ptr(), Dm.data_ptr(),
                          nact.data_ptr(), status.data_ptr(), want_deriv=True,
                          stream=sdfc.torch_stream_handle(stream))
    torch.cuda.synchronize()
    batch.close()
    assert np.array_equal(fm.cpu().numpy(), a[0])
    assert np.array_equal(Km.cpu().numpy().reshape(N, 12, 12), a[1])
    assert np.array_equal(Dm.cpu().numpy().reshape(N, 12, 12), a[2])


def test_rigid_motion_invariance_full_size(setup):
    """d fm / d q_B = -(d fm / d q_A) Ad(E_A^-1 E_B) for the FP64 path (no derivation used there)."""
    sdfc, ctx, gh, ph, states = setup
    fm, Km, Dm, nact, st = evaluate(sdfc, ctx, gh, ph, states, sdfc.PRECISION_FP64)
    EA, _, EB, _ = states
    worst = 0.0
    for k in range(0, N, 37):
        E = np.linalg.inv(EA[k]) @ EB[k]
        R, p = E[:3, :3], E[:3, 3]
        px = np.array([[0, -p[2], p[1]], [p[2], 0, -p[0]], [-p[1], p[0], 0]])
        Ad = np.zeros((6, 6))
        Ad[:3, :3] = R
        Ad[3:, 3:] = R
        Ad[3:, :3] = px @ R
        KA, KB = Km[k][:, :6], Km[k][:, 6:]
        worst = max(worst, np.linalg.norm(KB + KA @ Ad) / np.linalg.norm(KA))
    assert worst <= 1e-8, worst
