"""ORACLE — test infrastructure, not the product.

ctypes front end of the plain-C restatement in ``oracle/sdfc_oracle.c`` of the
reference redmax point-vs-SDF contact path.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg import this
module, as the checker; the product never does.

Every function cites the reference function it restates (paths relative to the
reference project root, ``rm/`` = ``simulation/redmax/``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "sdfc_oracle.c")
_LIB = os.path.join(_HERE, "_build", "libsdfc_oracle.so")

COLLISION_VALUE = 11
COLLISION_DERIV = 146
# (name, offset, shape) of the derivative blocks of orc_collision's output
COLLISION_BLOCKS = [
    ("dd_dxw", 11, (3,)), ("dd_dq2", 14, (6,)), ("dn_dxw", 20, (3, 3)), ("dn_dq2", 29, (3, 6)),
    ("dddot_dxw", 47, (3,)), ("dddot_dxwdot", 50, (3,)), ("dddot_dq2", 53, (6,)),
    ("dddot_dphi2", 59, (6,)), ("dtdot_dxw", 65, (3, 3)), ("dtdot_dxwdot", 74, (3, 3)),
    ("dtdot_dq2", 83, (3, 6)), ("dtdot_dphi2", 101, (3, 6)), ("dxi2_dxw", 119, (3, 3)),
    ("dxi2_dq2", 128, (3, 6)),
]


def build(force: bool = False) -> str:
    """Compile the restatement (no FMA contraction, see the C file header)."""
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(_SRC):
        os.makedirs(os.path.dirname(_LIB), exist_ok=True)
        tmp = _LIB + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", tmp, _SRC, "-lm"])
        os.replace(tmp, _LIB)
    return _LIB


class _Grid(ctypes.Structure):
    _fields_ = [("ni", ctypes.c_int), ("nj", ctypes.c_int), ("nk", ctypes.c_int),
                ("min_box", ctypes.c_double * 3), ("max_box", ctypes.c_double * 3),
                ("dx", ctypes.c_double * 3), ("col_th", ctypes.c_double),
                ("v", ctypes.POINTER(ctypes.c_double))]


class _Params(ctypes.Structure):
    _fields_ = [("kn", ctypes.c_double), ("kt", ctypes.c_double), ("mu", ctypes.c_double),
                ("damping", ctypes.c_double), ("scale", ctypes.c_double), ("contact_scale", ctypes.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        d = ctypes.c_double
        P = ctypes.POINTER
        _lib.orc_query_sdf.restype = d
        _lib.orc_query_sdf.argtypes = [P(_Grid), P(d), ctypes.c_int]
        _lib.orc_distance.restype = d
        _lib.orc_distance.argtypes = [P(_Grid), P(d), P(d)]
        _lib.orc_collision.restype = None
        _lib.orc_collision.argtypes = [P(_Grid), P(d), P(d), P(d), P(d), ctypes.c_int, P(d)]
        _lib.orc_detect.restype = ctypes.c_int
        _lib.orc_detect.argtypes = [P(_Grid), P(d), P(d), P(d), ctypes.c_int, P(ctypes.c_int), P(d)]
        _lib.orc_pair_eval.restype = ctypes.c_int
        _lib.orc_pair_eval.argtypes = [P(_Grid), P(d), ctypes.c_int, P(d), P(d), P(d), P(d), P(_Params),
                                       ctypes.c_int, P(d), P(d), P(d), P(ctypes.c_int)]
        _lib.orc_query_dsdf.argtypes = [P(_Grid), P(d), P(d)]
        _lib.orc_query_ddsdf.argtypes = [P(_Grid), P(d), P(d)]
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


@dataclass
class Grid:
    """An SDF body's grid (rm/Body/BodySDFObj.h:13-16); values indexed [k, j, i] (i fastest)."""
    values: np.ndarray  # shape (nk, nj, ni), float64
    min_box: np.ndarray
    max_box: np.ndarray
    dx: np.ndarray
    col_th: float

    def _c(self):
        v = _f64(self.values)
        self._keep = v
        nk, nj, ni = v.shape
        g = _Grid(ni, nj, nk, (ctypes.c_double * 3)(*self.min_box), (ctypes.c_double * 3)(*self.max_box),
                  (ctypes.c_double * 3)(*self.dx), float(self.col_th), _dp(v))
        return g


@dataclass
class Params:
    """ForceGeneralSDFContact coefficients (rm/Force/ForceGeneralSDFContact.h:16-20)."""
    kn: float = 1.0
    kt: float = 0.0
    mu: float = 0.0
    damping: float = 0.0
    scale: float = 1.0
    contact_scale: float = 1.0

    def _c(self):
        return _Params(self.kn, self.kt, self.mu, self.damping, self.scale, self.contact_scale)


def query_sdf(grid: Grid, x, outside_accurate=False) -> float:
    """BodySDFObj::query_SDF (rm/Body/BodySDFObj.cpp:123-174)."""
    g = grid._c()
    return lib().orc_query_sdf(ctypes.byref(g), _dp(_f64(x)), int(outside_accurate))


def query_dsdf(grid: Grid, x) -> np.ndarray:
    """BodySDFObj::query_dSDF (rm/Body/BodySDFObj.cpp:176-187)."""
    g = grid._c()
    out = np.zeros(3)
    lib().orc_query_dsdf(ctypes.byref(g), _dp(_f64(x)), _dp(out))
    return out


def query_ddsdf(grid: Grid, x) -> np.ndarray:
    """BodySDFObj::query_ddSDF (rm/Body/BodySDFObj.cpp:189-205)."""
    g = grid._c()
    out = np.zeros(9)
    lib().orc_query_ddsdf(ctypes.byref(g), _dp(_f64(x)), _dp(out))
    return out.reshape(3, 3)


def distance(grid: Grid, E_B, xw) -> float:
    """BodySDFObj::distance (rm/Body/BodySDFObj.cpp:207-213)."""
    g = grid._c()
    return lib().orc_distance(ctypes.byref(g), _dp(_f64(E_B)), _dp(_f64(xw)))


def collision(grid: Grid, E_B, phi_B, xw, xw_dot, want_deriv=True) -> np.ndarray:
    """BodySDFObj::collision (rm/Body/BodySDFObj.cpp:239-377); flat output, see COLLISION_BLOCKS."""
    g = grid._c()
    out = np.zeros(COLLISION_DERIV)
    lib().orc_collision(ctypes.byref(g), _dp(_f64(E_B)), _dp(_f64(phi_B)), _dp(_f64(xw)), _dp(_f64(xw_dot)),
                        int(want_deriv), _dp(out))
    return out if want_deriv else out[:COLLISION_VALUE]


def detect(grid: Grid, E_A, E_B, pts):
    """collision_detection_general_SDF (rm/CollisionDetection/CollisionDetection.cpp:124-147).

    Returns (active ids ascending, per-point distance)."""
    g = grid._c()
    p = _f64(pts).reshape(-1, 3)
    ids = np.zeros(max(len(p), 1), dtype=np.int32)
    dist = np.zeros(len(p))
    n = lib().orc_detect(ctypes.byref(g), _dp(_f64(E_A)), _dp(_f64(E_B)), _dp(p), len(p),
                         ids.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _dp(dist))
    return ids[:n].copy(), dist


def pair_eval(grid: Grid, pts, E_A, phi_A, E_B, phi_B, params: Params, want_deriv=True):
    """ForceGeneralSDFContact::computeForce[WithDerivative] (rm/Force/ForceGeneralSDFContact.cpp:46-105,
    147-447) for one (contact body A, SDF body B) pair.  Returns (fm[12], Km[12,12], Dm[12,12], ids)."""
    g = grid._c()
    p = _f64(pts).reshape(-1, 3)
    fm = np.zeros(12)
    Km = np.zeros(144)
    Dm = np.zeros(144)
    ids = np.zeros(max(len(p), 1), dtype=np.int32)
    prm = params._c()
    n = lib().orc_pair_eval(ctypes.byref(g), _dp(p), len(p), _dp(_f64(E_A)), _dp(_f64(phi_A)), _dp(_f64(E_B)),
                            _dp(_f64(phi_B)), ctypes.byref(prm), int(want_deriv), _dp(fm), _dp(Km), _dp(Dm),
                            ids.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    return fm, Km.reshape(12, 12), Dm.reshape(12, 12), ids[:n].copy()


def pair_force_norm_sum(grid: Grid, pts, E_A, phi_A, E_B, phi_B, params: Params) -> float:
    """Sum over the active contacts of |fm_i|, each contact's own 12-vector term of fm
    (rm/Force/ForceGeneralSDFContact.cpp:147-219 for one contact): the error scale of fm where
    contact forces cancel."""
    L = lib()
    if not hasattr(L, "_norm_ready"):
        L.orc_pair_force_norm_sum.restype = ctypes.c_double
        L.orc_pair_force_norm_sum.argtypes = [ctypes.POINTER(_Grid), ctypes.POINTER(ctypes.c_double), ctypes.c_int] + \
            [ctypes.POINTER(ctypes.c_double)] * 4 + [ctypes.POINTER(_Params)]
        L._norm_ready = True
    g = grid._c()
    p = _f64(pts).reshape(-1, 3)
    prm = params._c()
    return L.orc_pair_force_norm_sum(ctypes.byref(g), _dp(p), len(p), _dp(_f64(E_A)), _dp(_f64(phi_A)),
                                     _dp(_f64(E_B)), _dp(_f64(phi_B)), ctypes.byref(prm))


# --------------------------------------------------------------------------- BDF1 of one translational mover

class _Mover(ctypes.Structure):
    _fields_ = [("mass", ctypes.c_double), ("inertia", ctypes.c_double * 6), ("E_pj0", ctypes.c_double * 16),
                ("E_ji", ctypes.c_double * 16), ("gravity", ctypes.c_double * 3), ("h", ctypes.c_double),
                ("f_ext", ctypes.c_double * 6), ("joint_stiffness", ctypes.c_double),
                ("joint_damping", ctypes.c_double), ("q_rest", ctypes.c_double * 6), ("ndof", ctypes.c_int),
                ("newton_tol", ctypes.c_double)]


class _Pair(ctypes.Structure):
    _fields_ = [("grid", ctypes.POINTER(_Grid)), ("pts", ctypes.POINTER(ctypes.c_double)), ("n_pts", ctypes.c_int),
                ("mover_is_contact", ctypes.c_int), ("E_fixed", ctypes.c_double * 16), ("prm", _Params)]


@dataclass
class Mover:
    """One body on a joint to the world (Body::_mass/_Inertia/_E_ji, Joint::_E_pj_0, options):
    ndof 3 = translational, 6 = free3d-exp (q = (p, r), r exponential rotation coordinates)."""
    mass: float
    inertia: np.ndarray
    E_ji: np.ndarray
    E_pj0: np.ndarray = None
    gravity: tuple = (0.0, 0.0, -9.8)
    h: float = 5e-3
    f_ext: np.ndarray = None
    joint_stiffness: float = 0.0
    joint_damping: float = 0.0
    ndof: int = 3
    newton_tol: float = 0.0  # 0: the reference's 1e-8; smaller for finite-difference checks

    def _c(self):
        E_pj0 = np.eye(4) if self.E_pj0 is None else self.E_pj0
        f = np.zeros(6) if self.f_ext is None else self.f_ext
        return _Mover(float(self.mass), (ctypes.c_double * 6)(*_f64(self.inertia)),
                      (ctypes.c_double * 16)(*_f64(E_pj0).ravel()), (ctypes.c_double * 16)(*_f64(self.E_ji).ravel()),
                      (ctypes.c_double * 3)(*self.gravity), float(self.h), (ctypes.c_double * 6)(*_f64(f)),
                      float(self.joint_stiffness), float(self.joint_damping), (ctypes.c_double * 6)(*([0.0] * 6)),
                      int(self.ndof), float(self.newton_tol))


@dataclass
class ScenePair:
    """One contact of the mover with a fixed body (grid of the SDF body, points of the contact body)."""
    grid: Grid
    pts: np.ndarray
    mover_is_contact: bool
    E_fixed: np.ndarray
    params: Params


def _lib_sim():
    L = lib()
    if not hasattr(L, "_sim_ready"):
        P = ctypes.POINTER
        d = ctypes.c_double
        L.orc_bdf1_step.restype = ctypes.c_int
        L.orc_bdf1_step.argtypes = [P(_Mover), P(_Pair), ctypes.c_int, P(d), P(d), P(ctypes.c_int), P(ctypes.c_int)]
        L.orc_bdf1_eval.restype = None
        L.orc_bdf1_eval.argtypes = [P(_Mover), P(_Pair), ctypes.c_int, P(d), P(d), P(d), P(d), P(d)]
        L.orc_bdf1_eval_full.restype = None
        L.orc_bdf1_eval_full.argtypes = [P(_Mover), P(_Pair), ctypes.c_int, P(d), P(d), P(d), P(d), P(d), P(d),
                                         P(d)]
        L.orc_bdf1_backward.restype = None
        L.orc_bdf1_backward.argtypes = [P(_Mover), P(_Pair), ctypes.c_int, P(d), P(d), ctypes.c_int, P(d), P(d),
                                        P(d), P(d)]
        L._sim_ready = True
    return L


def _pairs_c(pairs):
    keep = []
    arr = (_Pair * max(1, len(pairs)))()
    for k, sp in enumerate(pairs):
        g = sp.grid._c()
        p = _f64(sp.pts).reshape(-1, 3)
        keep += [g, p, sp.grid]
        arr[k] = _Pair(ctypes.pointer(g), _dp(p), len(p), int(bool(sp.mover_is_contact)),
                       (ctypes.c_double * 16)(*_f64(sp.E_fixed).ravel()), sp.params._c())
    return arr, keep


def bdf1_steps(mover: Mover, pairs, q, qdot, steps=1):
    """Simulation::forward with BDF1 (Simulation.cpp:914-990, 1248-1270) for one moving part:
    returns (q_his[steps+1, ndof], qdot_his, converged[steps], iters[steps], evals[steps])."""
    L = _lib_sim()
    m = mover._c()
    arr, keep = _pairs_c(pairs)
    q = _f64(q).copy()
    qd = _f64(qdot).copy()
    qs, qds, conv, its, evs = [q.copy()], [qd.copy()], [], [], []
    it, ev = ctypes.c_int(), ctypes.c_int()
    for _ in range(steps):
        c = L.orc_bdf1_step(ctypes.byref(m), arr, len(pairs), _dp(q), _dp(qd), ctypes.byref(it), ctypes.byref(ev))
        qs.append(q.copy())
        qds.append(qd.copy())
        conv.append(bool(c))
        its.append(it.value)
        evs.append(ev.value)
    return np.array(qs), np.array(qds), np.array(conv), np.array(its), np.array(evs)


def bdf1_eval(mover: Mover, pairs, q0, qdot0, q1, want_H=True):
    """g and H of BDF1 at q1 (Simulation::evaluate_g_with_derivatives_BDF1, Simulation.cpp:1094-1165)."""
    L = _lib_sim()
    m = mover._c()
    arr, keep = _pairs_c(pairs)
    n = mover.ndof
    g = np.zeros(n)
    H = np.zeros(n * n)
    L.orc_bdf1_eval(ctypes.byref(m), arr, len(pairs), _dp(_f64(q0)), _dp(_f64(qdot0)), _dp(_f64(q1)), _dp(g),
                    _dp(H) if want_H else None)
    return g, H.reshape(n, n)


def bdf1_matrices(mover: Mover, pairs, q0, qdot0, q1):
    """g, H, M, D of BDF1 at q1: the step data integration_BDF1 saves for the adjoint
    (Simulation.cpp:1114-1163, 1262-1269)."""
    L = _lib_sim()
    m = mover._c()
    arr, keep = _pairs_c(pairs)
    n = mover.ndof
    g, H, M, D = np.zeros(n), np.zeros(n * n), np.zeros(n * n), np.zeros(n * n)
    L.orc_bdf1_eval_full(ctypes.byref(m), arr, len(pairs), _dp(_f64(q0)), _dp(_f64(qdot0)), _dp(_f64(q1)), _dp(g),
                         _dp(H), _dp(M), _dp(D))
    return g, H.reshape(n, n), M.reshape(n, n), D.reshape(n, n)


def bdf1_backward(mover: Mover, pairs, q_his, qdot0, df_dq):
    """Simulation::backward_BDF1 (Simulation.cpp:1559-1634) from a trajectory q_his[T+1, 3]
    and dL/dq_k[T, 3]; returns (dL/dq0, dL/dqdot0, dL/df_ext[6])."""
    L = _lib_sim()
    m = mover._c()
    arr, keep = _pairs_c(pairs)
    n = mover.ndof
    q_his = _f64(q_his).reshape(-1, n)
    T = len(q_his) - 1
    df_dq = _f64(df_dq).reshape(T, n)
    g0, gd0, gf = np.zeros(n), np.zeros(n), np.zeros(6)
    L.orc_bdf1_backward(ctypes.byref(m), arr, len(pairs), _dp(q_his), _dp(_f64(qdot0)), T, _dp(df_dq), _dp(g0),
                        _dp(gd0), _dp(gf))
    return g0, gd0, gf


def pair_energy(grid: Grid, pts, E_A, E_B, params: Params):
    """Penetration energy of a pair and its gradient (12) wrt the twists of A then B."""
    L = lib()
    if not hasattr(L, "_energy_ready"):
        L.orc_pair_energy.restype = ctypes.c_double
        L.orc_pair_energy.argtypes = [ctypes.POINTER(_Grid), ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                      ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                      ctypes.POINTER(_Params), ctypes.POINTER(ctypes.c_double)]
        L._energy_ready = True
    g = grid._c()
    p = _f64(pts).reshape(-1, 3)
    dE = np.zeros(12)
    prm = params._c()
    e = L.orc_pair_energy(ctypes.byref(g), _dp(p), len(p), _dp(_f64(E_A)), _dp(_f64(E_B)), ctypes.byref(prm), _dp(dE))
    return e, dE


def make_level_set3(verts, tris, origin, dx, shape, exact_band=1) -> np.ndarray:
    """sdfgen::make_level_set3 (simulation/externals/sdfgen/makelevelset3.cpp:161-227):
    phi[k, j, i] of the closed mesh (verts (nv, 3), tris (nt, 3)) on the grid with
    node (i, j, k) at origin + (i dx, j dy, k dz), shape = (ni, nj, nk)."""
    L = lib()
    fp = ctypes.POINTER(ctypes.c_float)
    L.orc_make_level_set3.restype = None
    L.orc_make_level_set3.argtypes = [fp, ctypes.c_int, ctypes.POINTER(ctypes.c_uint), ctypes.c_int, fp,
                                      ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_int, fp]
    V = np.ascontiguousarray(verts, np.float32)
    T = np.ascontiguousarray(tris, np.uint32)
    o = np.ascontiguousarray(origin, np.float32)
    d = np.broadcast_to(np.asarray(dx, np.float32), (3,))
    ni, nj, nk = (int(s) for s in shape)
    phi = np.empty((nk, nj, ni), np.float32)
    L.orc_make_level_set3(V.ctypes.data_as(fp), len(V), T.ctypes.data_as(ctypes.POINTER(ctypes.c_uint)), len(T),
                          o.ctypes.data_as(fp), float(d[0]), float(d[1]), float(d[2]), ni, nj, nk, int(exact_band),
                          phi.ctypes.data_as(fp))
    return phi


def body_distance(grid: Grid, E_from, E_to, V, per_point=False):
    """Simulation::get_body_distance (rm/Simulation.cpp:276-296): the `to` body's grid, both
    poses, the `from` body's vertices (n, 3) -> minimum (and every vertex's distance)."""
    L = lib()
    L.orc_body_distance.restype = ctypes.c_double
    L.orc_body_distance.argtypes = [ctypes.POINTER(_Grid), ctypes.POINTER(ctypes.c_double),
                                    ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                    ctypes.POINTER(ctypes.c_double)]
    g = grid._c()
    v = _f64(V).reshape(-1, 3)
    d = np.zeros(len(v))
    m = L.orc_body_distance(ctypes.byref(g), _dp(_f64(E_from)), _dp(_f64(E_to)), _dp(v), len(v), _dp(d))
    return (m, d) if per_point else m
