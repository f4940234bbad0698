"""Shared helpers of the parity tests."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel_err(a, b):
    """The reference's error convention (simulation/redmax/Utils.h:362-381):
    |a - b| / max(min(|a|, |b|), 1e-4), Frobenius norms; also returns |a - b|."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    err = np.linalg.norm(a - b)
    return err / max(min(np.linalg.norm(a), np.linalg.norm(b)), 1e-4), err


def assert_close(name, a, b, rel=1e-9, abs_=1e-9):
    """Fails when both the relative and the absolute error exceed their bounds
    (the reference reports a mismatch only when rel > 1e-5 and abs > 1e-5)."""
    r, e = rel_err(a, b)
    assert not (r > rel and e > abs_), f"{name}: rel {r:.3e} abs {e:.3e}"


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name)))
