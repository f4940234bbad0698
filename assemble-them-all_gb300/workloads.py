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
    vals = np.empty((n, n, n))
    Y, X = np.meshgrid(ax[1], ax[0], indexing="ij")

    def slab(k):  # one z slab at a time bounds the memory of large grids
        vals[k] = fn(np.stack([X, Y, np.full_like(X, ax[2][k])], axis=-1))

    if n >= 128:  # NumPy releases the GIL inside its kernels: slabs in threads
        import concurrent.futures as cf
        import os
        with cf.ThreadPoolExecutor(max_workers=min(32, os.cpu_count() or 1)) as ex:
            list(ex.map(slab, range(n)))
    else:
        for k in range(n):
            slab(k)
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


def direction_sweep_states(n, rank=0, world=1):
    """The direction sweep of the planner (one instance per pull direction): the peg fully inserted
    in the socket, shifted 0.0201 toward the direction's lateral part (pressed 1e-4 into the bore
    wall past col_th 0.01), tilted 0.002 rad about the perpendicular axis, raised 0.25 d_z, moving
    at 0.01 d.  Returns (E_A, phi_A, E_B, phi_B) for n instances.  With `world` replicas the sweep
    is one Fibonacci sphere of n * world directions and replica `rank` takes its rank-th block of
    n, so the replicas' instances are disjoint and together cover the sphere."""
    if not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    dirs = fibonacci_directions(n * world)[rank * n:(rank + 1) * n]
    EA = np.zeros((n, 4, 4))
    phiA = np.zeros((n, 6))
    for k, d in enumerate(dirs):
        lat = np.array([d[0], d[1], 0.0])
        ln = np.linalg.norm(lat)
        lat = lat / ln if ln > 1e-6 else np.array([1.0, 0.0, 0.0])
        R = rotvec_to_matrix(0.002 * np.array([-lat[1], lat[0], 0.0]))
        EA[k] = pose(R, 0.0201 * lat + np.array([0.0, 0.0, 0.25 * d[2]]))
        phiA[k, 3:] = 0.01 * d
    EB = np.broadcast_to(np.eye(4), (n, 4, 4)).copy()
    phiB = np.zeros((n, 6))
    return EA, phiA, EB, phiB


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


# --------------------------------------------------------------------------- procedural multi-part assemblies
#
# Stand-ins for the reference's multi-part assembly datasets: a chain of box blocks along x, each
# joined to the next by a tab on its +x face that sits in a slot of the next block's -x face, and
# some blocks pierced by a z bore holding a pin (a part of its own).  Sizes are jittered by +-2%
# (inside the 0.01 clearances) so the parts stay interlocked without overlapping.
# Every part is a CSG of boxes and z cylinders in its own frame (centred at its placement); its
# signed distance is the min/max composition of the primitives'.

def _box_sdf(p, c, h):
    q = np.abs(p - np.asarray(c)) - np.asarray(h)
    return np.linalg.norm(np.maximum(q, 0.0), axis=-1) + np.minimum(q.max(axis=-1), 0.0)


def _zcyl_sdf(p, c, r, hl):
    d = p - np.asarray(c)
    rr = np.sqrt(d[..., 0] ** 2 + d[..., 1] ** 2)
    e = np.stack([rr - r, np.abs(d[..., 2]) - hl], axis=-1)
    return np.minimum(np.max(e, axis=-1), 0.0) + np.linalg.norm(np.maximum(e, 0.0), axis=-1)


@dataclass
class Primitive:
    kind: str     # "box" or "zcyl"
    c: tuple      # centre in the part frame
    size: tuple   # box half-extents, or (radius, half-length)
    sign: int     # +1 union (material), -1 subtraction (cut)

    def sdf(self, p):
        return _box_sdf(p, self.c, self.size) if self.kind == "box" else _zcyl_sdf(p, self.c, *self.size)

    def area(self):
        if self.kind == "box":
            hx, hy, hz = self.size
            return 8.0 * (hx * hy + hy * hz + hx * hz)
        r, hl = self.size
        return 2.0 * np.pi * r * 2.0 * hl + 2.0 * np.pi * r * r

    def sample_surface(self, g, n):
        c = np.asarray(self.c, dtype=np.float64)
        if self.kind == "box":
            h = np.asarray(self.size, dtype=np.float64)
            areas = np.array([h[1] * h[2], h[1] * h[2], h[0] * h[2], h[0] * h[2], h[0] * h[1], h[0] * h[1]])
            face = g.choice(6, size=n, p=areas / areas.sum())
            u = g.uniform(-1.0, 1.0, (n, 3)) * h
            ax = face // 2
            u[np.arange(n), ax] = np.where(face % 2 == 0, -h[ax], h[ax])
            return c + u
        r, hl = self.size
        side, cap = 2 * np.pi * r * 2 * hl, np.pi * r * r
        which = g.uniform(0.0, side + 2 * cap, n)
        th = g.uniform(0.0, 2 * np.pi, n)
        z = g.uniform(-hl, hl, n)
        rr = r * np.sqrt(g.uniform(0.0, 1.0, n))
        zc = np.where(which < side + cap, -hl, hl)
        lat = which < side
        pts = np.where(lat[:, None], np.stack([r * np.cos(th), r * np.sin(th), z], -1),
                       np.stack([rr * np.cos(th), rr * np.sin(th), zc], -1))
        return c + pts


@dataclass
class Part:
    prims: list        # Primitive list: the material ones first, then the cuts
    position: np.ndarray  # placement of the part frame in the world (translation only)

    def sdf(self, p):
        d = None
        for pr in self.prims:
            if pr.sign > 0:
                s = pr.sdf(p)
                d = s if d is None else np.minimum(d, s)
        for pr in self.prims:
            if pr.sign < 0:
                d = np.maximum(d, -pr.sdf(p))
        return d

    def bounds(self):
        lo = np.full(3, np.inf)
        hi = np.full(3, -np.inf)
        for pr in self.prims:
            if pr.sign < 0:
                continue
            c = np.asarray(pr.c)
            h = np.asarray(pr.size) if pr.kind == "box" else np.array([pr.size[0], pr.size[0], pr.size[1]])
            lo = np.minimum(lo, c - h)
            hi = np.maximum(hi, c + h)
        return lo, hi

    def surface_points(self, n, seed, tol=1e-9):
        """n points uniform (area-weighted) on the part's surface, part frame."""
        g = np.random.default_rng(seed)
        areas = np.array([pr.area() for pr in self.prims])
        out = []
        have = 0
        while have < n:
            m = max(2 * (n - have), 256)
            which = g.choice(len(self.prims), size=m, p=areas / areas.sum())
            cand = np.concatenate([self.prims[k].sample_surface(g, int((which == k).sum()))
                                   for k in range(len(self.prims))])
            keep = cand[np.abs(self.sdf(cand)) <= tol]
            out.append(keep)
            have += len(keep)
        pts = np.concatenate(out)[:n]
        return pts[g.permutation(len(pts))]

    def mass_props(self, density=1.0):
        """Mass and principal inertia diagonal (Ixx, Iyy, Izz, m, m, m) of the part's material
        primitives taken as solids about the part frame (the cuts ignored: a stand-in for the
        mesh integrals of BodyMeshObj)."""
        m_tot, I = 0.0, np.zeros(3)
        for pr in self.prims:
            if pr.sign < 0:
                continue
            c = np.asarray(pr.c)
            if pr.kind == "box":
                a, b, cz = 2 * np.asarray(pr.size)
                m = density * a * b * cz
                Ic = m / 12.0 * np.array([b * b + cz * cz, a * a + cz * cz, a * a + b * b])
            else:
                r, hl = pr.size
                m = density * np.pi * r * r * 2 * hl
                L = 2 * hl
                Ic = np.array([m * (3 * r * r + L * L) / 12, m * (3 * r * r + L * L) / 12, m * r * r / 2])
            Ic = Ic + m * np.array([c[1] ** 2 + c[2] ** 2, c[0] ** 2 + c[2] ** 2, c[0] ** 2 + c[1] ** 2])
            m_tot += m
            I += Ic
        return m_tot, np.array([I[0], I[1], I[2], m_tot, m_tot, m_tot])

    def grid(self, n, dtype=np.float64, pad=0.1):
        lo, hi = self.bounds()
        return sample_grid(self.sdf, lo, hi, n, pad=pad, dtype=dtype)

    # ---- the same definitions evaluated on the GPU (torch, FP64), for workloads too large to
    # generate on the host (hundreds of 256^3 grids, tens of millions of surface points)
    def sdf_device(self, p):
        """sdf() of (..., 3) FP64 points on the device."""
        d = None
        for pr in self.prims:
            if pr.sign > 0:
                s = _prim_sdf_t(pr, p)
                d = s if d is None else _torch().minimum(d, s)
        for pr in self.prims:
            if pr.sign < 0:
                d = _torch().maximum(d, -_prim_sdf_t(pr, p))
        return d

    def grid_device(self, n, pad=0.1):
        """grid(n, FP32) sampled on the device: (FP32 values (nk, nj, ni) on the device, min_box,
        max_box, dx), the box and spacing computed as sample_grid computes them."""
        torch = _torch()
        lo, hi = self.bounds()
        ext = hi - lo
        mn = lo - pad * ext / 2.0
        mx = hi + pad * ext / 2.0
        dx = (mx - mn) / (n - 1)
        mx = mn + (n - 1) * dx
        ax = [torch.tensor(mn[a] + dx[a] * np.arange(n), dtype=torch.float64, device="cuda") for a in range(3)]
        Y, X = torch.meshgrid(ax[1], ax[0], indexing="ij")
        vals = torch.empty((n, n, n), dtype=torch.float32, device="cuda")
        for k0 in range(0, n, 32):  # slabs of 32 planes bound the temporaries
            k1 = min(n, k0 + 32)
            Z = ax[2][k0:k1].view(-1, 1, 1).expand(k1 - k0, n, n)
            P = torch.stack([X.expand(k1 - k0, n, n), Y.expand(k1 - k0, n, n), Z], dim=-1)
            vals[k0:k1] = self.sdf_device(P).to(torch.float32)
        return vals, mn, mx, dx

    def surface_points_device(self, n, seed, tol=1e-9):
        """surface_points(n) drawn on the device (its own seeded stream): n points uniform
        (area-weighted) on the part's surface, rounded to FP32, returned as a host (n, 3) FP64 array."""
        torch = _torch()
        g = torch.Generator(device="cuda")
        g.manual_seed(int(seed))
        areas = torch.tensor([pr.area() for pr in self.prims], dtype=torch.float64, device="cuda")
        out, have = [], 0
        while have < n:
            m = max(2 * (n - have), 256)
            which = torch.multinomial(areas / areas.sum(), m, replacement=True, generator=g)
            counts = torch.bincount(which, minlength=len(self.prims)).tolist()
            cand = torch.cat([_prim_sample_t(pr, g, c) for pr, c in zip(self.prims, counts) if c > 0])
            keep = cand[self.sdf_device(cand).abs() <= tol]
            out.append(keep)
            have += len(keep)
        pts = torch.cat(out)[:n]
        pts = pts[torch.randperm(len(pts), generator=g, device="cuda")]
        return pts.to(torch.float32).to(torch.float64).cpu().numpy()


def _torch():
    import torch
    return torch


def _prim_sdf_t(pr, p):
    torch = _torch()
    c = torch.tensor(pr.c, dtype=torch.float64, device=p.device)
    if pr.kind == "box":
        q = (p - c).abs() - torch.tensor(pr.size, dtype=torch.float64, device=p.device)
        return q.clamp_min(0.0).norm(dim=-1) + q.amax(dim=-1).clamp_max(0.0)
    r, hl = pr.size
    d = p - c
    rr = torch.sqrt(d[..., 0] ** 2 + d[..., 1] ** 2)
    e = torch.stack([rr - r, d[..., 2].abs() - hl], dim=-1)
    return e.amax(dim=-1).clamp_max(0.0) + e.clamp_min(0.0).norm(dim=-1)


def _prim_sample_t(pr, g, n):
    """Primitive.sample_surface on the device."""
    torch = _torch()
    dev = "cuda"
    c = torch.tensor(pr.c, dtype=torch.float64, device=dev)
    if pr.kind == "box":
        h = torch.tensor(pr.size, dtype=torch.float64, device=dev)
        areas = torch.stack([h[1] * h[2], h[1] * h[2], h[0] * h[2], h[0] * h[2], h[0] * h[1], h[0] * h[1]])
        face = torch.multinomial(areas / areas.sum(), n, replacement=True, generator=g)
        u = (torch.rand((n, 3), dtype=torch.float64, device=dev, generator=g) * 2.0 - 1.0) * h
        ax = face // 2
        idx = torch.arange(n, device=dev)
        u[idx, ax] = torch.where(face % 2 == 0, -h[ax], h[ax])
        return c + u
    r, hl = pr.size
    side, cap = 2 * np.pi * r * 2 * hl, np.pi * r * r
    rnd = lambda: torch.rand(n, dtype=torch.float64, device=dev, generator=g)  # noqa: E731
    which = rnd() * (side + 2 * cap)
    th = rnd() * (2 * np.pi)
    z = rnd() * (2 * hl) - hl
    rr = r * torch.sqrt(rnd())
    zc = torch.where(which < side + cap, torch.full_like(z, -hl), torch.full_like(z, hl))
    lat = (which < side).unsqueeze(-1)
    a = torch.stack([r * torch.cos(th), r * torch.sin(th), z], dim=-1)
    b = torch.stack([rr * torch.cos(th), rr * torch.sin(th), zc], dim=-1)
    return c + torch.where(lat, a, b)


@dataclass
class Assembly:
    parts: list
    n_points: list   # contact points per part
    grid_n: list     # grid resolution per part
    mover: int       # the pulled part
    direction: np.ndarray


def procedural_assembly(seed: int, n_parts: int = None, points=(2000, 200000), grids=(64, 128, 256),
                        clearance: float = 0.01, jitter: float = 0.02) -> Assembly:
    """A seeded interlocked assembly of 2-12 parts: boxes chained by tab-in-slot joints along x,
    some with a z bore holding a pin.  Per part: contact points log-uniform in `points`, grid
    resolution uniform over `grids`.  One part is pulled along a random axis direction."""
    g = np.random.default_rng(seed)
    n_parts = int(g.integers(2, 13)) if n_parts is None else int(n_parts)
    n_pins = int(g.integers(0, n_parts // 2 + 1)) if n_parts > 2 else 0
    n_blocks = max(n_parts - n_pins, 1 if n_parts == 1 else 2)
    n_pins = n_parts - n_blocks
    J = lambda v: v * (1.0 + g.uniform(-jitter, jitter))
    tab_h = 0.15  # tab half-width / half-height
    tab_t = 0.3   # tab protrusion (= slot depth)
    parts = []
    for k in range(n_blocks):
        h = (0.5, J(0.5), J(0.5))
        prims = [Primitive("box", (0.0, 0.0, 0.0), h, +1)]
        if k + 1 < n_blocks:  # tab into the next block
            prims.append(Primitive("box", (0.5 + tab_t / 2, 0.0, 0.0), (tab_t / 2, J(tab_h), J(tab_h)), +1))
        if k > 0:  # slot for the previous block's tab
            prims.append(Primitive("box", (-0.5 + tab_t / 2, 0.0, 0.0),
                                   (tab_t / 2 + clearance, tab_h * (1 + jitter) + clearance,
                                    tab_h * (1 + jitter) + clearance), -1))
        # blocks half a clearance apart (placement jitter a tenth of it): no part overlaps another
        # at rest, contacts come from the pull
        parts.append(Part(prims, np.array([k * (1.0 + 0.5 * clearance) + g.uniform(-0.1, 0.1) * clearance,
                                           0.0, 0.0])))
    bored = sorted(g.choice(n_blocks, size=n_pins, replace=n_pins > n_blocks))
    for b in bored:
        blk = parts[b]
        bx = g.uniform(-0.1, 0.1)  # bore away from the tab/slot axis in y
        by = 0.3 * (1 if g.uniform() < 0.5 else -1)
        r = J(0.1)
        blk.prims.append(Primitive("zcyl", (bx, by, 0.0), (r + clearance, 2.0), -1))
        pin = Part([Primitive("zcyl", (0.0, 0.0, 0.0), (r, J(0.7)), +1)],
                   blk.position + np.array([bx, by, 0.0]))
        parts.append(pin)
    n_pts = [int(round(np.exp(g.uniform(np.log(points[0]), np.log(points[1]))))) for _ in parts]
    grid_n = [int(g.choice(grids)) for _ in parts]
    mover = int(g.integers(len(parts)))
    axis = int(g.integers(3))
    d = np.zeros(3)
    d[axis] = 1.0 if g.uniform() < 0.5 else -1.0
    return Assembly(parts, n_pts, grid_n, mover, d)


# ----------------------------------------------------------------------------- triangle meshes
# Closed triangle meshes for building SDF grids (BodySDFObj::precompute_SDF): the parts of an
# assembly arrive as OBJ meshes; these procedural ones stand in for them.  Vertices (nv, 3)
# float64, faces (nt, 3) int32, outward-facing.

def box_mesh(half=(0.5, 0.5, 0.5), center=(0.0, 0.0, 0.0)):
    h = np.asarray(half, float)
    c = np.asarray(center, float)
    V = np.array([[sx, sy, sz] for sz in (-1, 1) for sy in (-1, 1) for sx in (-1, 1)], float) * h + c
    F = np.array([[0, 2, 1], [1, 2, 3], [4, 5, 6], [5, 7, 6], [0, 1, 4], [1, 5, 4],
                  [2, 6, 3], [3, 6, 7], [0, 4, 2], [2, 4, 6], [1, 3, 5], [3, 7, 5]], np.int32)
    return V, F


def cylinder_mesh(radius=0.4, half_len=0.5, segments=24):
    """A z-axis cylinder: `segments` side quads and two fans."""
    n = segments
    t = 2 * np.pi * np.arange(n) / n
    ring = np.stack([radius * np.cos(t), radius * np.sin(t)], 1)
    V = np.concatenate([np.c_[ring, np.full(n, -half_len)], np.c_[ring, np.full(n, half_len)],
                        [[0, 0, -half_len], [0, 0, half_len]]])
    F = []
    for a in range(n):
        b = (a + 1) % n
        F += [(a, b, n + b), (a, n + b, n + a), (2 * n, b, a), (2 * n + 1, n + a, n + b)]
    return V, np.array(F, np.int32)


def torus_mesh(R=0.6, r=0.25, n=32, m=16):
    """A torus about z: n segments around the axis, m around the tube."""
    u = 2 * np.pi * np.arange(n) / n
    v = 2 * np.pi * np.arange(m) / m
    U, Vv = np.meshgrid(u, v, indexing="ij")
    V = np.stack([(R + r * np.cos(Vv)) * np.cos(U), (R + r * np.cos(Vv)) * np.sin(U), r * np.sin(Vv)], -1)
    F = []
    for a in range(n):
        for b in range(m):
            i, j = a * m + b, ((a + 1) % n) * m + b
            k, l = ((a + 1) % n) * m + (b + 1) % m, a * m + (b + 1) % m
            F += [(i, j, k), (i, k, l)]
    return V.reshape(-1, 3), np.array(F, np.int32)


def socket_mesh(outer=1.0, inner=0.5, half_len=1.0):
    """A square socket: the box [-outer, outer]^2 x [-half_len, half_len] minus a square z-bore
    of half-width `inner` (32 large triangles)."""
    sq = np.array([[-1, -1], [1, -1], [1, 1], [-1, 1]], float)
    rings = [np.c_[sq * s, np.full(4, z)] for s in (outer, inner) for z in (-half_len, half_len)]
    V = np.concatenate(rings)  # outer bottom 0-3, outer top 4-7, inner bottom 8-11, inner top 12-15
    F = []
    for c in range(4):
        d = (c + 1) % 4
        F += [(c, d, 4 + d), (c, 4 + d, 4 + c)]                  # outer side
        F += [(8 + d, 8 + c, 12 + c), (8 + d, 12 + c, 12 + d)]    # bore side
        F += [(4 + c, 4 + d, 12 + d), (4 + c, 12 + d, 12 + c)]    # top ring
        F += [(d, c, 8 + c), (d, 8 + c, 8 + d)]                   # bottom ring
    return V, np.array(F, np.int32)


def level_set_grid(V, dx, pad=2):
    """A grid covering the mesh with `pad` cells of margin: (origin float32, shape (ni, nj, nk))."""
    V = np.asarray(V, np.float32)
    h = np.float32(dx)
    lo, hi = V.min(0), V.max(0)
    origin = (lo - pad * h).astype(np.float32)
    shape = tuple(int(np.ceil((hi[a] - lo[a]) / h)) + 2 * pad + 1 for a in range(3))
    return origin, shape
