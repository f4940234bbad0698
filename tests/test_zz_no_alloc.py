"""The allocation-free entry point sdfc_evaluate_noalloc, through the C ABI.

It is for callers that cannot allocate device memory when they need a contact
force (real-time loops, hosts that own all device memory, stream capture).  Its
results must equal the allocating entry point sdfc_evaluate's on the same
inputs, within the tolerances of the GPU parity tests, on consecutive calls
(its working memory is shared between calls and must not leak state)."""
import numpy as np
import pytest

from _helpers import assert_close, load
from conftest import submodule

pytestmark = pytest.mark.gpu

FM_REL = 1e-10  # the FP64 analytic-mode bars of test_gpu_parity.py
JAC_REL = 1e-6


def test_noalloc_matches_evaluate_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    submodule("build").build()
    sdfc = submodule("sdfc")
    fx = load("pair_eval.npz")
    ctx = sdfc.Context(0)
    try:
        grid = ctx.upload_grid(fx["grid"], fx["min_box"], fx["max_box"], fx["dx"], float(fx["col_th"]), 0)
        pts = ctx.upload_points(fx["points"], 0)
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()  # noqa: E731
        g = dev(fx["grid"])
        p = dev(fx["points"])
        shape = fx["grid"].shape[::-1]  # (ni, nj, nk)
        fm = torch.empty(12, dtype=torch.float64, device="cuda")
        Km = torch.empty(144, dtype=torch.float64, device="cuda")
        Dm = torch.empty(144, dtype=torch.float64, device="cuda")
        nact = torch.empty(1, dtype=torch.int32, device="cuda")
        cases = [1, 4, 4, 9]  # consecutive calls, one repeated
        seen = {}
        for k in cases:
            EA, phiA, EB, phiB = (dev(fx[key][k]) for key in ("EA", "phiA", "EB", "phiB"))
            prm = dev(fx["params"][k])
            fm.fill_(np.nan)
            Km.fill_(np.nan)
            Dm.fill_(np.nan)
            sdfc.evaluate_noalloc(g.data_ptr(), shape, fx["min_box"], fx["max_box"], fx["dx"], float(fx["col_th"]),
                                  p.data_ptr(), len(fx["points"]), EA.data_ptr(), phiA.data_ptr(), EB.data_ptr(),
                                  phiB.data_ptr(), prm.data_ptr(), fm.data_ptr(), Km.data_ptr(), Dm.data_ptr(),
                                  nact.data_ptr(), want_deriv=True)
            torch.cuda.synchronize()
            got = (fm.cpu().numpy(), Km.cpu().numpy().reshape(12, 12), Dm.cpu().numpy().reshape(12, 12),
                   int(nact.item()))
            ref = ctx.evaluate(pts, grid, fx["EA"][k], fx["phiA"][k], fx["EB"][k], fx["phiB"][k],
                               sdfc.Params(*[float(x) for x in fx["params"][k]]), want_deriv=True)
            assert got[3] == ref[3] == fx["n_active"][k]
            assert_close(f"case {k} fm", got[0], ref[0], rel=FM_REL)
            assert_close(f"case {k} Km", got[1], ref[1], rel=JAC_REL)
            assert_close(f"case {k} Dm", got[2], ref[2], rel=JAC_REL)
            if k in seen:
                assert all(np.array_equal(a, b) for a, b in zip(got[:3], seen[k]))
            seen[k] = got[:3]
        # value-only calls (Km, Dm not given) against the value form of sdfc_evaluate
        for k in (4, 9):
            EA, phiA, EB, phiB = (dev(fx[key][k]) for key in ("EA", "phiA", "EB", "phiB"))
            prm = dev(fx["params"][k])
            fm.fill_(np.nan)
            sdfc.evaluate_noalloc(g.data_ptr(), shape, fx["min_box"], fx["max_box"], fx["dx"], float(fx["col_th"]),
                                  p.data_ptr(), len(fx["points"]), EA.data_ptr(), phiA.data_ptr(), EB.data_ptr(),
                                  phiB.data_ptr(), prm.data_ptr(), fm.data_ptr(), None, None, nact.data_ptr(),
                                  want_deriv=False)
            torch.cuda.synchronize()
            ref = ctx.evaluate(pts, grid, fx["EA"][k], fx["phiA"][k], fx["EB"][k], fx["phiB"][k],
                               sdfc.Params(*[float(x) for x in fx["params"][k]]), want_deriv=False)
            assert int(nact.item()) == ref[3] == fx["n_active"][k]
            assert_close(f"case {k} fm (value form)", fm.cpu().numpy(), ref[0], rel=FM_REL)
        # an empty point set: no contact, zero force and Jacobians
        fm.fill_(np.nan)
        Km.fill_(np.nan)
        Dm.fill_(np.nan)
        nact.fill_(-1)
        sdfc.evaluate_noalloc(g.data_ptr(), shape, fx["min_box"], fx["max_box"], fx["dx"], float(fx["col_th"]),
                              p.data_ptr(), 0, EA.data_ptr(), phiA.data_ptr(), EB.data_ptr(), phiB.data_ptr(),
                              prm.data_ptr(), fm.data_ptr(), Km.data_ptr(), Dm.data_ptr(), nact.data_ptr(),
                              want_deriv=True)
        torch.cuda.synchronize()
        assert int(nact.item()) == 0
        assert not fm.cpu().numpy().any() and not Km.cpu().numpy().any() and not Dm.cpu().numpy().any()
        # sizes beyond the maximum, and negative ones, are refused before any launch
        for bad in (131073, -1):
            with pytest.raises(sdfc.SdfcError):
                sdfc.evaluate_noalloc(g.data_ptr(), shape, fx["min_box"], fx["max_box"], fx["dx"], 0.01,
                                      p.data_ptr(), bad, EA.data_ptr(), phiA.data_ptr(), EB.data_ptr(),
                                      phiB.data_ptr(), prm.data_ptr(), fm.data_ptr(), Km.data_ptr(), Dm.data_ptr(),
                                      nact.data_ptr(), want_deriv=True)
    finally:
        ctx.close()
