"""The procedural assembly generator (CPU): seeded, interlocked without overlap, points on the
surface, sizes in the requested ranges."""
import numpy as np

from conftest import submodule


def test_procedural_assemblies():
    W = submodule("workloads")
    for seed in range(6):
        a = W.procedural_assembly(seed, points=(2000, 6000), grids=(24, 32))
        b = W.procedural_assembly(seed, points=(2000, 6000), grids=(24, 32))
        assert 2 <= len(a.parts) <= 12 and 0 <= a.mover < len(a.parts)
        assert a.n_points == b.n_points and a.grid_n == b.grid_n and np.array_equal(a.direction, b.direction)
        assert all(2000 <= n <= 6000 for n in a.n_points) and set(a.grid_n) <= {24, 32}
        assert np.abs(a.direction).sum() == 1.0
        pts = [p.surface_points(n, k) for k, (p, n) in enumerate(zip(a.parts, a.n_points))]
        near = 0
        for i, pi in enumerate(a.parts):
            assert np.abs(pi.sdf(pts[i])).max() <= 1e-9  # on the surface
            for j, pj in enumerate(a.parts):
                if i != j:
                    d = pj.sdf(pts[i] + pi.position - pj.position)
                    assert d.min() >= 0.0  # no overlap at rest
                    near += int(d.min() < 0.02)  # within a clearance or two: interlocked
        assert near >= 2
