"""Synthetic peg-in-hole inputs that stand in for the reference's assembly datasets.

The reference plans on download-only mesh datasets; these seeded procedural
inputs keep their shapes and sizes:
  * socket: the cube [-1, 1]^3 minus a z-axis bore of radius 0.5, as an analytic
    signed distance sampled on an n^3 grid over the bounding box padded by 10%;
  * peg: a cylinder of radius 0.49 and length 2, its contact points drawn
    uniformly (area-weighted) from its surface with a seed, rounded to FP32;
  * pull directions on a Fibonacci sphere or in a cone about +z.
Grids follow BodySDFObj's layout: values[k, j, i] (i fastest), min_box, max_box,
dx (simulation/redmax/Body/BodySDFObj.h:13-16).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class GridSpec:
    values: np.ndarray  # (nk, nj, ni) float64
    min_box: np.ndarray
    max_box: np.ndarray
    dx: np.ndarray

    @property
    def shape(self):
        return self.values.shape


def socket_sdf(p: np.ndarray, half: float = 1.0, bore: float = 0.5) -> np.ndarray:
    """Signed distance (negative inside material) of a cube of half-size `half` minus a z-axis bore."""
    q = np.abs(p) - half
    box = np.linalg.norm(np.maximum(q, 0.0), axis=-1) + np.minimum(q.max(axis=-1), 0.0)
    cyl = np.sqrt(p[..., 0] ** 2 + p[..., 1] ** 2) - bore
    return np.maximum(box, -cyl)


def cylinder_sdf(p: np.ndarray, radius: float = 0.49, half_len: float = 1.0) -> np.ndarray:
    """Signed distance of a z-axis capped cylinder."""
    r = np.sqrt(p[..., 0] ** 2 + p[..., 1] ** 2)
    d = np.stack([r - radius, np.abs(p[..., 2]) - half_len], axis=-1)
    return np.minimum(np.max(d, axis=-1), 0.0) + np.linalg.norm(np.maximum(d, 0.0), axis=-1)


def sample_grid(fn, lo, hi, n: int, pad: float = 0.1, dtype=np.float64) -> GridSpec:
    """Samples `fn` on an n^3 grid over the box [lo, hi] grown by `pad` x its extent (half on each side).

    dtype=np.float32 rounds the values to FP32 (the precision sdfgen generates, BodySDFObj.cpp:72-83)."""
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    ext = hi - lo
    mn = lo - pad * ext / 2.0
    mx = hi + pad * ext / 2.0
    dx = (mx - mn) / (n - 1)
    mx = mn + (n - 1) * dx
    ax = [mn[a] + dx[a] * np.arange(n) for a in range(3)]
    Z, Y, X = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    vals = fn(np.stack([X, Y, Z], axis=-1))
    vals = vals.astype(dtype).astype(np.float64)
    return GridSpec(np.ascontiguousarray(vals), mn, mx, dx)


def socket_grid(n: int = 64, dtype=np.float64) -> GridSpec:
    return sample_grid(socket_sdf, [-1, -1, -1], [1, 1, 1], n, pad=0.1, dtype=dtype)


def peg_grid(n: int = 64, dtype=np.float64) -> GridSpec:
    return sample_grid(cylinder_sdf, [-0.49, -0.49, -1.0], [0.49, 0.49, 1.0], n, pad=0.1, dtype=dtype)


def peg_points(n: int, radius: float = 0.49, length: float = 2.0, seed: int = 0) -> np.ndarray:
    """n points uniform on the closed cylinder surface (lateral + caps), FP32-representable, body frame
    (centre of mass at the origin, axis along z)."""
    g = np.random.default_rng(seed)
    side = 2.0 * np.pi * radius * length
    cap = np.pi * radius * radius
    u = g.uniform(0.0, side + 2.0 * cap, n)
    th = g.uniform(0.0, 2.0 * np.pi, n)
    z = g.uniform(-length / 2, length / 2, n)
    rr = radius * np.sqrt(g.uniform(0.0, 1.0, n))
    zc = np.where(g.uniform(0.0, 1.0, n) < 0.5, -length / 2, length / 2)
    lat = u < side
    pts = np.where(lat[:, None], np.stack([radius * np.cos(th), radius * np.sin(th), z], -1),
                   np.stack([rr * np.cos(th), rr * np.sin(th), zc], -1))
    return pts.astype(np.float32).astype(np.float64)


def cylinder_mass_props(radius: float = 0.49, length: float = 2.0, density: float = 1.0):
    """Mass and principal inertia diagonal (Ixx, Iyy, Izz, m, m, m) of a solid cylinder
    (the layout of Body::_Inertia, simulation/redmax/Body/Body.h)."""
    m = density * np.pi * radius * radius * length
    ixx = m * (3 * radius * radius + length * length) / 12.0
    izz = m * radius * radius / 2.0
    return m, np.array([ixx, ixx, izz, m, m, m])


def fibonacci_directions(n: int) -> np.ndarray:
    """n unit vectors on a Fibonacci sphere."""
    k = np.arange(n) + 0.5
    phi = np.arccos(1.0 - 2.0 * k / n)
    theta = np.pi * (1.0 + 5.0 ** 0.5) * k
    return np.stack([np.cos(theta) * np.sin(phi), np.sin(theta) * np.sin(phi), np.cos(phi)], axis=-1)


def cone_directions(n: int, half_angle_deg: float = 30.0, seed: int = 0) -> np.ndarray:
    """n unit vectors uniform in a cone about +z."""
    g = np.random.default_rng(seed)
    c = np.cos(np.deg2rad(half_angle_deg))
    z = g.uniform(c, 1.0, n)
    th = g.uniform(0.0, 2.0 * np.pi, n)
    s = np.sqrt(1.0 - z * z)
    return np.stack([s * np.cos(th), s * np.sin(th), z], axis=-1)


def rotvec_to_matrix(w) -> np.ndarray:
    """Rodrigues' formula (the same map as math::exp(Vector3), simulation/redmax/Utils.h:108-124)."""
    w = np.asarray(w, dtype=np.float64)
    th = np.linalg.norm(w)
    if th < 1e-12:
        return np.eye(3)
    k = w / th
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K


def pose(R=None, p=None) -> np.ndarray:
    E = np.eye(4)
    if R is not None:
        E[:3, :3] = R
    if p is not None:
        E[:3, 3] = p
    return E
