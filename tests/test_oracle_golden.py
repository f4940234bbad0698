"""The oracle restatement against golden vectors generated by the reference itself."""
import numpy as np
import pytest

from _helpers import assert_close, load


@pytest.fixture(scope="module")
def fx():
    return load("pair_eval.npz")


def grid_of(O, fx):
    return O.Grid(fx["grid"], fx["min_box"], fx["max_box"], fx["dx"], float(fx["col_th"]))


def test_pair_eval_golden(oracle, fx):
    g = grid_of(oracle, fx)
    for k in range(len(fx["fm"])):
        kn, kt, mu, kd, sc, cs = fx["params"][k]
        prm = oracle.Params(kn, kt, mu, kd, sc, cs)
        args = (g, fx["points"], fx["EA"][k], fx["phiA"][k], fx["EB"][k], fx["phiB"][k], prm)
        fm_v, _, _, ids_v = oracle.pair_eval(*args, want_deriv=False)
        fm, Km, Dm, ids = oracle.pair_eval(*args, want_deriv=True)
        ref_ids = fx["ids"][k][: fx["n_active"][k]]
        assert np.array_equal(ids, ref_ids), f"case {k}: active set differs"
        assert np.array_equal(ids_v, ref_ids)
        assert_close(f"case {k} fm (value)", fm_v, fx["fm_v"][k], rel=1e-12)
        assert_close(f"case {k} fm", fm, fx["fm"][k], rel=1e-12)
        assert_close(f"case {k} Km", Km, fx["Km"][k], rel=1e-12)
        assert_close(f"case {k} Dm", Dm, fx["Dm"][k], rel=1e-12)


def test_collision_golden(oracle):
    c = load("collision.npz")
    g = oracle.Grid(c["grid"], c["min_box"], c["max_box"], c["dx"], float(c["col_th"]))
    for k in range(len(c["xw"])):
        out = oracle.collision(g, c["EB"][k], c["phiB"][k], c["xw"][k], c["xw_dot"][k], want_deriv=True)
        ref = c["out"][k]
        assert_close(f"point {k} value part", out[:11], ref[:11], rel=1e-11)
        for name, off, shape in oracle.COLLISION_BLOCKS:
            n = int(np.prod(shape))
            assert_close(f"point {k} {name}", out[off:off + n], ref[off:off + n], rel=1e-9, abs_=1e-9)


def test_detect_matches_pair_ids(oracle, fx):
    g = grid_of(oracle, fx)
    for k in range(len(fx["fm"])):
        ids, dist = oracle.detect(g, fx["EA"][k], fx["EB"][k], fx["points"])
        assert np.array_equal(ids, fx["ids"][k][: fx["n_active"][k]])
        assert np.array_equal(ids, np.nonzero(dist < 0)[0])
