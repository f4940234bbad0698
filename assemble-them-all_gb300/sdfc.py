"""Python host side of libsdfcontact (include/sdfc.h), through ctypes.

The GPU path is the only path: if the shared library is missing this module
raises on import, and every call goes to the CUDA kernels.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsdfcontact.so")

SDFC_OK = 0
SDFC_ERR_NOT_FOUND = -3
STORAGE_F64 = 0
STORAGE_F32 = 1
STORAGE_F16_BRICKS = 2
STORAGE_F32_NODES = 3

# every symbol include/sdfc.h declares
EXPORTS = (
    "sdfc_create", "sdfc_destroy", "sdfc_last_error", "sdfc_upload_grid", "sdfc_upload_points",
    "sdfc_evaluate", "sdfc_active_ids", "sdfc_batch_create", "sdfc_batch_destroy", "sdfc_batch_evaluate",
    "sdfc_batch_evaluate_device", "sdfc_batch_evaluate_masked_device", "sdfc_batch_recheck_count", "sdfc_set_derivative_mode",
    "sdfc_batch_set_derivative_mode", "sdfc_batch_set_timing", "sdfc_batch_last_timing", "sdfc_set_precision",
    "sdfc_batch_set_precision", "sdfc_evaluate_noalloc", "sdfc_sim_create", "sdfc_sim_destroy",
    "sdfc_sim_set_precision", "sdfc_sim_set_state", "sdfc_sim_get_state", "sdfc_sim_set_external_force",
    "sdfc_sim_step", "sdfc_sim_stats", "sdfc_sim_record", "sdfc_sim_history", "sdfc_sim_backward",
    "sdfc_grid_values", "sdfc_f16_brick_encode", "sdfc_f16_brick_decode", "sdfc_batch_energy",
    "sdfc_batch_energy_device", "sdfc_sim_record_energy", "sdfc_sim_energy", "sdfc_sim_backward_energy",
    "sdfc_sim_set_tolerance", "sdfc_make_level_set3", "sdfc_make_level_set3_device", "sdfc_sdf_grid_layout",
    "sdfc_batch_distance", "sdfc_batch_distance_device", "sdfc_grid_distance", "sdfc_sdf_save_text",
    "sdfc_sdf_load_text", "sdfc_sdf_save_bricks", "sdfc_sdf_load_bricks", "sdfc_upload_grid_bricks",
    "sdfc_upload_hull", "sdfc_disassembled", "sdfc_disassembled_device", "sdfc_upload_grid_device",
    "sdfc_sim_scene_evaluations", "sdfc_batch_autotune", "sdfc_batch_get_tuning", "sdfc_batch_set_tuning",
    "sdfc_sim_autotune", "sdfc_sim_get_tuning", "sdfc_sim_set_tuning",
)
JOINT_TRANSLATIONAL = 3
JOINT_FREE3D_EXP = 6
PRECISION_FP64 = 0
PRECISION_MIXED = 1
DERIV_ANALYTIC = 0
DERIV_STENCIL = 1


class SdfcError(RuntimeError):
    pass


class Mover(ctypes.Structure):
    """sdfc_mover: the moving part (Body::_mass, _Inertia, Joint::_E_pj_0, Body::_E_ji, gravity, timestep)."""
    _fields_ = [("joint", ctypes.c_int), ("mass", ctypes.c_double), ("inertia", ctypes.c_double * 6),
                ("E_pj0", ctypes.c_double * 16), ("E_ji", ctypes.c_double * 16), ("gravity", ctypes.c_double * 3),
                ("h", ctypes.c_double), ("joint_stiffness", ctypes.c_double), ("joint_damping", ctypes.c_double)]

    @classmethod
    def make(cls, mass, inertia, E_ji, h, gravity=(0.0, 0.0, -9.8), E_pj0=None, joint=3, joint_stiffness=0.0,
             joint_damping=0.0):
        E_pj0 = np.eye(4) if E_pj0 is None else np.asarray(E_pj0, dtype=np.float64)
        return cls(joint, float(mass), (ctypes.c_double * 6)(*np.asarray(inertia, dtype=np.float64)),
                   (ctypes.c_double * 16)(*E_pj0.ravel()),
                   (ctypes.c_double * 16)(*np.asarray(E_ji, dtype=np.float64).ravel()),
                   (ctypes.c_double * 3)(*gravity), float(h), float(joint_stiffness), float(joint_damping))


FORCE_CTAS = 0
FORCE_WORKERS = 1
FORCE_GRID = 2


class Tuning(ctypes.Structure):
    """sdfc_tuning: the launch configuration of a batch's force pass."""
    _fields_ = [("slots", ctypes.c_int), ("force_variant", ctypes.c_int), ("worker_ctas", ctypes.c_int),
                ("chunks_per_slot", ctypes.c_int), ("ms", ctypes.c_float)]

    def as_dict(self):
        return {"slots": self.slots, "force_variant": ("ctas", "workers", "grid")[self.force_variant],
                "worker_ctas": self.worker_ctas, "chunks_per_slot": self.chunks_per_slot, "ms": float(self.ms)}


class Params(ctypes.Structure):
    """sdfc_params: ForceGeneralSDFContact's kn, kt, mu, damping, scale and the contact body's contact_scale."""
    _fields_ = [("kn", ctypes.c_double), ("kt", ctypes.c_double), ("mu", ctypes.c_double),
                ("damping", ctypes.c_double), ("scale", ctypes.c_double), ("contact_scale", ctypes.c_double)]

    def __init__(self, kn=1.0, kt=0.0, mu=0.0, damping=0.0, scale=1.0, contact_scale=1.0):
        super().__init__(kn, kt, mu, damping, scale, contact_scale)

    def as_row(self):
        return np.array([self.kn, self.kt, self.mu, self.damping, self.scale, self.contact_scale])


class ScenePair(ctypes.Structure):
    """sdfc_scene_pair: one contact of scene `instance`'s mover with a fixed part."""
    _fields_ = [("instance", ctypes.c_int), ("points", ctypes.c_int), ("grid", ctypes.c_int),
                ("mover_is_contact", ctypes.c_int), ("E_fixed", ctypes.c_double * 16), ("params", Params)]

    @classmethod
    def make(cls, instance, points, grid, mover_is_contact, E_fixed, params):
        return cls(int(instance), int(points), int(grid), int(bool(mover_is_contact)),
                   (ctypes.c_double * 16)(*np.asarray(E_fixed, dtype=np.float64).ravel()), params)


_lib = None


def lib():
    """Loads libsdfcontact.so; raises if it was not built (no fallback exists)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise SdfcError(f"{LIB_PATH} is missing: run the package build (build.build()) first")
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER
        d, i, v = P(ctypes.c_double), ctypes.c_int, ctypes.c_void_p
        L.sdfc_create.argtypes = [P(v), i]
        L.sdfc_destroy.argtypes = [v]
        L.sdfc_destroy.restype = None
        L.sdfc_last_error.argtypes = [v]
        L.sdfc_last_error.restype = ctypes.c_char_p
        L.sdfc_upload_grid.argtypes = [v, d, i, i, i, d, d, d, ctypes.c_double, i, P(i)]
        L.sdfc_upload_grid_device.argtypes = [v, v, i, i, i, d, d, d, ctypes.c_double, i, P(i)]
        L.sdfc_upload_points.argtypes = [v, d, i, i, P(i)]
        L.sdfc_evaluate.argtypes = [v, i, i, d, d, d, d, P(Params), i, d, d, d, P(i)]
        L.sdfc_active_ids.argtypes = [v, P(i), i, P(i)]
        L.sdfc_batch_create.argtypes = [v, i, P(i), P(i), P(v)]
        L.sdfc_batch_destroy.argtypes = [v]
        L.sdfc_batch_destroy.restype = None
        L.sdfc_batch_evaluate.argtypes = [v, d, d, d, d, P(Params), i, d, d, d, P(i), P(i)]
        L.sdfc_batch_evaluate_device.argtypes = [v, v, v, v, v, v, i, v, v, v, v, v, v]
        L.sdfc_batch_evaluate_masked_device.argtypes = [v, v, v, v, v, v, v, v, v, v, v, v, v]
        L.sdfc_batch_recheck_count.argtypes = [v, P(ctypes.c_ulonglong), i]
        L.sdfc_set_derivative_mode.argtypes = [v, i]
        L.sdfc_batch_set_derivative_mode.argtypes = [v, i]
        L.sdfc_batch_set_timing.argtypes = [v, i]
        L.sdfc_set_precision.argtypes = [v, i]
        L.sdfc_sim_create.argtypes = [v, i, P(Mover), i, P(ScenePair), P(v)]
        L.sdfc_sim_destroy.argtypes = [v]
        L.sdfc_sim_destroy.restype = None
        L.sdfc_sim_set_precision.argtypes = [v, i]
        L.sdfc_sim_set_state.argtypes = [v, d, d]
        L.sdfc_sim_get_state.argtypes = [v, d, d]
        L.sdfc_sim_set_external_force.argtypes = [v, d]
        L.sdfc_sim_step.argtypes = [v, i, P(i)]
        L.sdfc_sim_stats.argtypes = [v, P(ctypes.c_longlong), P(ctypes.c_longlong)]
        L.sdfc_sim_scene_evaluations.argtypes = [v, P(ctypes.c_longlong)]
        L.sdfc_batch_autotune.argtypes = [v, v, v, v, v, v, i, v, v, v, v, v, v, P(Tuning)]
        L.sdfc_batch_get_tuning.argtypes = [v, P(Tuning)]
        L.sdfc_batch_set_tuning.argtypes = [v, P(Tuning)]
        L.sdfc_sim_autotune.argtypes = [v, P(Tuning)]
        L.sdfc_sim_get_tuning.argtypes = [v, P(Tuning)]
        L.sdfc_sim_set_tuning.argtypes = [v, P(Tuning)]
        L.sdfc_sim_record.argtypes = [v, i]
        L.sdfc_grid_values.argtypes = [v, i, d]
        L.sdfc_batch_energy.argtypes = [v, d, d, P(Params), d, d]
        L.sdfc_sim_record_energy.argtypes = [v, i]
        L.sdfc_sim_energy.argtypes = [v, d, d]
        L.sdfc_sim_backward_energy.argtypes = [v, d, d, d, d, d]
        L.sdfc_sim_set_tolerance.argtypes = [v, ctypes.c_double]
        L.sdfc_batch_energy_device.argtypes = [v, v, v, v, v, v, v, v, v]
        L.sdfc_f16_brick_encode.argtypes = [d, i, i, i, v, v]
        L.sdfc_f16_brick_decode.argtypes = [v, v, i, i, i, d]
        L.sdfc_sim_history.argtypes = [v, P(i), d]
        L.sdfc_sim_backward.argtypes = [v, d, d, d, d]
        L.sdfc_evaluate_noalloc.argtypes = [v, i, i, i, d, d, d, ctypes.c_double, v, i, v, v, v, v, v, i, v, v, v,
                                            v, v]
        L.sdfc_batch_set_precision.argtypes = [v, i]
        L.sdfc_batch_last_timing.argtypes = [v, P(ctypes.c_float)]
        f, f32 = P(ctypes.c_float), ctypes.c_float
        L.sdfc_make_level_set3.argtypes = [v, f, i, P(ctypes.c_uint), i, f, f32, f32, f32, i, i, i, i, f]
        L.sdfc_make_level_set3_device.argtypes = [v, v, i, v, i, f, f32, f32, f32, i, i, i, i, v, v]
        L.sdfc_sdf_grid_layout.argtypes = [d, i, ctypes.c_double, i, P(i), d, d, d, f]
        L.sdfc_batch_distance.argtypes = [v, d, d, d, d]
        L.sdfc_batch_distance_device.argtypes = [v, v, v, v, v, v]
        L.sdfc_grid_distance.argtypes = [v, i, d, i, d, d]
        cp = ctypes.c_char_p
        L.sdfc_sdf_save_text.argtypes = [cp, d, i, i, i, d, d, d]
        L.sdfc_sdf_load_text.argtypes = [cp, P(i), d, d, d, d, ctypes.c_longlong]
        L.sdfc_sdf_save_bricks.argtypes = [cp, d, i, i, i, d, d, d]
        L.sdfc_sdf_load_bricks.argtypes = [cp, P(i), d, d, d, v, v]
        L.sdfc_upload_grid_bricks.argtypes = [v, v, v, i, i, i, d, d, d, ctypes.c_double, P(i)]
        L.sdfc_upload_hull.argtypes = [v, d, i, d, i, P(i)]
        L.sdfc_disassembled.argtypes = [v, i, i, d, i, P(i), P(i)]
        L.sdfc_disassembled_device.argtypes = [v, i, i, v, i, v, v, v]
        _lib = L
    return _lib


CUDA_STREAM_LEGACY = 1  # cudaStreamLegacy: the legacy default stream named explicitly


def torch_stream_handle(stream) -> int:
    """The handle to pass for a torch stream.  torch's default stream has handle 0, which the
    library reads as "the context's own stream"; name the legacy default stream instead."""
    h = int(stream.cuda_stream)
    return h if h else CUDA_STREAM_LEGACY


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _f64(a, shape=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    if shape is not None:
        a = a.reshape(shape)
    return a


class Context:
    """A device context (sdfc_create): owns uploaded grids and point sets."""

    def __init__(self, device: int = 0):
        self._h = ctypes.c_void_p()
        rc = lib().sdfc_create(ctypes.byref(self._h), int(device))
        if rc != SDFC_OK:
            raise SdfcError(f"sdfc_create failed ({rc}): no usable CUDA device {device}")
        self.device = device
        self._npoints = {}
        self._grid_shapes = {}
        self._batches = []

    def _check(self, rc, what):
        if rc != SDFC_OK:
            raise SdfcError(f"{what} failed ({rc}): {lib().sdfc_last_error(self._h).decode()}")

    def close(self):
        if self._h:
            lib().sdfc_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload_grid(self, values, min_box, max_box, dx, col_th, storage=STORAGE_F32) -> int:
        """values: (nk, nj, ni) array (i fastest), as BodySDFObj::_SDF."""
        v = _f64(values)
        nk, nj, ni = v.shape
        h = ctypes.c_int()
        self._check(lib().sdfc_upload_grid(self._h, _dp(v), ni, nj, nk, _dp(_f64(min_box, 3)), _dp(_f64(max_box, 3)),
                                           _dp(_f64(dx, 3)), float(col_th), int(storage), ctypes.byref(h)),
                    "sdfc_upload_grid")
        self._grid_shapes[h.value] = (nk, nj, ni)
        return h.value

    def upload_grid_device(self, values_ptr, shape, min_box, max_box, dx, col_th, storage=STORAGE_F32_NODES) -> int:
        """sdfc_upload_grid_device: FP32 node values already on the device (values_ptr, an int
        address of (nk, nj, ni) floats, i fastest); shape = (nk, nj, ni)."""
        nk, nj, ni = shape
        h = ctypes.c_int()
        self._check(lib().sdfc_upload_grid_device(self._h, int(values_ptr), ni, nj, nk, _dp(_f64(min_box, 3)),
                                                  _dp(_f64(max_box, 3)), _dp(_f64(dx, 3)), float(col_th),
                                                  int(storage), ctypes.byref(h)), "sdfc_upload_grid_device")
        self._grid_shapes[h.value] = (nk, nj, ni)
        return h.value

    def upload_grid_bricks(self, codes, so, shape, min_box, max_box, dx, col_th) -> int:
        """sdfc_upload_grid_bricks: an FP16-brick grid from its codes and (scale, offset) pairs
        (as f16_brick_encode / load_sdf_bricks give them); shape = (nk, nj, ni)."""
        nk, nj, ni = shape
        codes = np.ascontiguousarray(codes, np.uint16)
        so = np.ascontiguousarray(so, np.float32)
        nb = ((ni + 7) // 8) * ((nj + 7) // 8) * ((nk + 7) // 8)
        if codes.size != nb * 512 or so.size != 2 * nb:
            raise ValueError("codes / so do not match the grid's bricks")
        h = ctypes.c_int()
        self._check(lib().sdfc_upload_grid_bricks(self._h, codes.ctypes.data, so.ctypes.data, ni, nj, nk,
                                                  _dp(_f64(min_box, 3)), _dp(_f64(max_box, 3)), _dp(_f64(dx, 3)),
                                                  float(col_th), ctypes.byref(h)), "sdfc_upload_grid_bricks")
        self._grid_shapes[h.value] = (nk, nj, ni)
        return h.value

    def grid_distance(self, grid: int, X, want_values=True):
        """sdfc_grid_distance: SDFMesh::query_SDF at X (n, 3) in the grid's frame ->
        (d (n,) or None, minimum)."""
        Xc = _f64(X).reshape(-1, 3)
        d = np.zeros(len(Xc)) if want_values else None
        m = np.zeros(1)
        self._check(lib().sdfc_grid_distance(self._h, int(grid), _dp(Xc), len(Xc), None if d is None else _dp(d),
                                             _dp(m)), "sdfc_grid_distance")
        return d, float(m[0])

    def upload_hull(self, points) -> int:
        """The convex hull of points (n, 3) for the disassembly check (sdfc_upload_hull): its
        vertices and facet planes from qhull, as trimesh.convex.convex_hull builds it."""
        from scipy.spatial import ConvexHull
        pts = _f64(points).reshape(-1, 3)
        hull = ConvexHull(pts)
        verts = np.ascontiguousarray(pts[hull.vertices])
        planes = np.ascontiguousarray(hull.equations, dtype=np.float64)
        h = ctypes.c_int()
        self._check(lib().sdfc_upload_hull(self._h, _dp(verts), len(verts), _dp(planes), len(planes),
                                           ctypes.byref(h)), "sdfc_upload_hull")
        return h.value

    def disassembled(self, hull_move: int, hull_still: int, E, with_flags=False):
        """sdfc_disassembled for poses E (n, 4, 4) of the moving part -> bool (n,) [, flags]."""
        Ec = _f64(E).reshape(-1, 16)
        n = len(Ec)
        out = np.zeros(n, np.int32)
        flags = np.zeros(n, np.int32)
        self._check(lib().sdfc_disassembled(self._h, int(hull_move), int(hull_still), _dp(Ec), n, _ip(out),
                                            _ip(flags)), "sdfc_disassembled")
        return (out.astype(bool), flags) if with_flags else out.astype(bool)

    def grid_values(self, grid: int) -> np.ndarray:
        """The grid as the evaluations see it, (nk, nj, ni) (sdfc_grid_values)."""
        out = np.zeros(self._grid_shapes[grid])
        self._check(lib().sdfc_grid_values(self._h, int(grid), _dp(out)), "sdfc_grid_values")
        return out

    def upload_points(self, xyz, storage=STORAGE_F32) -> int:
        p = _f64(xyz).reshape(-1, 3)
        h = ctypes.c_int()
        self._check(lib().sdfc_upload_points(self._h, _dp(p), len(p), int(storage), ctypes.byref(h)),
                    "sdfc_upload_points")
        self._npoints[h.value] = len(p)
        return h.value

    def evaluate(self, points, grid, E_A, phi_A, E_B, phi_B, params: Params, want_deriv=True):
        """One ForceGeneralSDFContact call; returns (fm[12], Km[12,12], Dm[12,12], n_active)."""
        fm = np.zeros(12)
        Km = np.zeros(144)
        Dm = np.zeros(144)
        n = ctypes.c_int()
        self._check(lib().sdfc_evaluate(self._h, int(points), int(grid), _dp(_f64(E_A, 16)), _dp(_f64(phi_A, 6)),
                                        _dp(_f64(E_B, 16)), _dp(_f64(phi_B, 6)), ctypes.byref(params),
                                        int(bool(want_deriv)), _dp(fm), _dp(Km), _dp(Dm), ctypes.byref(n)),
                    "sdfc_evaluate")
        return fm, Km.reshape(12, 12), Dm.reshape(12, 12), n.value

    def active_ids(self, cap=None):
        n = ctypes.c_int()
        if cap is None:
            self._check(lib().sdfc_active_ids(self._h, None, 0, ctypes.byref(n)), "sdfc_active_ids")
            cap = n.value
        ids = np.zeros(max(cap, 1), dtype=np.int32)
        self._check(lib().sdfc_active_ids(self._h, _ip(ids), cap, ctypes.byref(n)), "sdfc_active_ids")
        return ids[:min(cap, n.value)].copy()

    def set_derivative_mode(self, mode: int):
        """DERIV_ANALYTIC or DERIV_STENCIL for sdfc_evaluate and later batches."""
        self._check(lib().sdfc_set_derivative_mode(self._h, int(mode)), "sdfc_set_derivative_mode")

    def set_precision(self, precision: int):
        """PRECISION_FP64 or PRECISION_MIXED for sdfc_evaluate and later batches."""
        self._check(lib().sdfc_set_precision(self._h, int(precision)), "sdfc_set_precision")

    def make_level_set3(self, verts, tris, origin, dx, shape, exact_band=1) -> np.ndarray:
        """sdfgen::make_level_set3 on the GPU (sdfc_make_level_set3): phi (nk, nj, ni) float32 of
        the closed mesh (verts (nv, 3) float32, tris (nt, 3)) on the grid with node (i, j, k) at
        origin + (i dx, j dy, k dz), shape = (ni, nj, nk)."""
        V = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
        T = np.ascontiguousarray(tris, np.uint32).reshape(-1, 3)
        o = np.ascontiguousarray(origin, np.float32).reshape(3)
        d = np.broadcast_to(np.asarray(dx, np.float32), (3,))
        ni, nj, nk = (int(x) for x in shape)
        phi = np.empty((nk, nj, ni), np.float32)
        fp = ctypes.POINTER(ctypes.c_float)
        self._check(lib().sdfc_make_level_set3(self._h, V.ctypes.data_as(fp), len(V),
                                               T.ctypes.data_as(ctypes.POINTER(ctypes.c_uint)), len(T),
                                               o.ctypes.data_as(fp), float(d[0]), float(d[1]), float(d[2]), ni, nj,
                                               nk, int(exact_band), phi.ctypes.data_as(fp)), "sdfc_make_level_set3")
        return phi

    def make_level_set3_device(self, verts, tris, origin, dx, shape, exact_band=1, stream=None):
        """sdfc_make_level_set3_device on torch CUDA tensors: verts (nv, 3) float32, tris (nt, 3)
        int32 (read as unsigned); returns phi (nk, nj, ni) float32 on the same device, queued on
        `stream` (default: torch's current stream)."""
        import torch
        V = verts.contiguous()
        T = tris.contiguous()
        if V.dtype != torch.float32 or T.dtype != torch.int32 or not V.is_cuda or not T.is_cuda:
            raise ValueError("verts: CUDA float32 (nv, 3); tris: CUDA int32 (nt, 3)")
        o = np.ascontiguousarray(origin, np.float32).reshape(3)
        d = np.broadcast_to(np.asarray(dx, np.float32), (3,))
        ni, nj, nk = (int(x) for x in shape)
        phi = torch.empty((nk, nj, ni), dtype=torch.float32, device=V.device)
        st = torch_stream_handle(stream or torch.cuda.current_stream(V.device))
        fp = ctypes.POINTER(ctypes.c_float)
        self._check(lib().sdfc_make_level_set3_device(self._h, V.data_ptr(), V.shape[0], T.data_ptr(), T.shape[0],
                                                      o.ctypes.data_as(fp), float(d[0]), float(d[1]), float(d[2]), ni,
                                                      nj, nk, int(exact_band), phi.data_ptr(), st),
                    "sdfc_make_level_set3_device")
        return phi

    def precompute_sdf(self, V, F, dx, res):
        """BodySDFObj::precompute_SDF (simulation/redmax/Body/BodySDFObj.cpp:38-84) with the level set
        built on the GPU: the body-frame mesh (V (nv, 3), F (nt, 3)) with the body's dx and res ->
        (values (nk, nj, ni) float64, min_box, max_box, spacing), the arguments of upload_grid."""
        shape, min_box, max_box, spacing, origin = sdf_grid_layout(V, dx, res)
        phi = self.make_level_set3(np.asarray(V, np.float64).astype(np.float32), F, origin,
                                   spacing.astype(np.float32), shape)
        return phi.astype(np.float64), min_box, max_box, spacing

    def batch(self, points, grids) -> "Batch":
        return Batch(self, points, grids)

    def sim(self, movers, pairs) -> "Sim":
        return Sim(self, movers, pairs)


class Batch:
    """sdfc_batch: n pair instances evaluated by one set of launches."""

    def __init__(self, ctx: Context, points, grids):
        pts = np.ascontiguousarray(np.asarray(points, dtype=np.int32))
        grd = np.ascontiguousarray(np.asarray(grids, dtype=np.int32))
        if pts.shape != grd.shape or pts.ndim != 1:
            raise ValueError("points and grids must be equal-length 1-D handle arrays")
        self.ctx = ctx
        self.n = len(pts)
        self._points = [int(x) for x in pts]
        self._h = ctypes.c_void_p()
        ctx._check(lib().sdfc_batch_create(ctx._h, self.n, _ip(pts), _ip(grd), ctypes.byref(self._h)),
                   "sdfc_batch_create")

    def close(self):
        if self._h and self.ctx._h:
            lib().sdfc_batch_destroy(self._h)
        self._h = ctypes.c_void_p()

    def set_derivative_mode(self, mode: int):
        self.ctx._check(lib().sdfc_batch_set_derivative_mode(self._h, int(mode)), "sdfc_batch_set_derivative_mode")

    def distance(self, E_A, E_B, per_point=False):
        """sdfc_batch_distance: each instance's minimum distance of A's points to B's grid (n,);
        with per_point, also every point's distance (a list of n arrays, caller order)."""
        n = self.n
        mn = np.zeros(n)
        counts = [self.ctx._npoints[p] for p in self._points]
        d = np.zeros(max(1, sum(counts))) if per_point else None
        self.ctx._check(lib().sdfc_batch_distance(self._h, _dp(_f64(E_A, 16 * n)), _dp(_f64(E_B, 16 * n)), _dp(mn),
                                                  None if d is None else _dp(d)), "sdfc_batch_distance")
        if not per_point:
            return mn
        off = np.concatenate([[0], np.cumsum(counts)])
        return mn, [d[off[k]:off[k + 1]].copy() for k in range(n)]

    def evaluate(self, E_A, phi_A, E_B, phi_B, params, want_deriv=True, out=None):
        """Host arrays in, host arrays out: (fm[n,12], Km[n,12,12], Dm[n,12,12], n_active[n], status[n]).
        params: one Params for every instance, a sequence of n Params, or an (n, 6) array of
        (kn, kt, mu, damping, scale, contact_scale) rows (sdfc_params' layout).  out: optional
        (fm, Km, Dm, n_active, status) arrays of those shapes (float64 / int32, C-contiguous) to
        write into and return, for callers that keep their result buffers across calls."""
        n = self.n
        if out is not None:
            fm, Km, Dm, nact, st = out
            ok = (fm.dtype == np.float64 and fm.shape == (n, 12) and fm.flags.c_contiguous and
                  nact.dtype == np.int32 and nact.shape == (n,) and st.dtype == np.int32 and st.shape == (n,) and
                  (not want_deriv or all(a.dtype == np.float64 and a.shape == (n, 12, 12) and a.flags.c_contiguous
                                         for a in (Km, Dm))))
            if not ok:
                raise ValueError("out: fm (n, 12), Km and Dm (n, 12, 12) float64, n_active and status (n,) int32")
        if isinstance(params, Params):
            rows = np.tile(params.as_row(), (n, 1))
        elif isinstance(params, np.ndarray):
            rows = params
        else:
            rows = np.array([p.as_row() for p in params])
        rows = _f64(rows, (n, 6))
        prm = rows.ctypes.data_as(ctypes.POINTER(Params))
        if out is None:
            fm = np.zeros((n, 12))
            Km = np.zeros((n, 12, 12)) if want_deriv else np.zeros(1)
            Dm = np.zeros((n, 12, 12)) if want_deriv else np.zeros(1)
            nact = np.zeros(n, dtype=np.int32)
            st = np.zeros(n, dtype=np.int32)
        self.ctx._check(lib().sdfc_batch_evaluate(self._h, _dp(_f64(E_A, 16 * n)), _dp(_f64(phi_A, 6 * n)),
                                                  _dp(_f64(E_B, 16 * n)), _dp(_f64(phi_B, 6 * n)), prm,
                                                  int(bool(want_deriv)), _dp(fm), _dp(Km) if want_deriv else None,
                                                  _dp(Dm) if want_deriv else None, _ip(nact), _ip(st)),
                        "sdfc_batch_evaluate")
        if want_deriv:
            return fm, Km, Dm, nact, st
        return fm, None, None, nact, st

    def evaluate_device(self, E_A, phi_A, E_B, phi_B, params, fm, Km, Dm, n_active, status, want_deriv=True,
                        stream=0):
        """Device pointers (ints, e.g. torch tensor.data_ptr()); enqueued on `stream` without syncing."""
        self.ctx._check(lib().sdfc_batch_evaluate_device(self._h, E_A, phi_A, E_B, phi_B, params,
                                                         int(bool(want_deriv)), fm, Km or 0, Dm or 0, n_active,
                                                         status, stream), "sdfc_batch_evaluate_device")

    def autotune(self, E_A, phi_A, E_B, phi_B, params, fm, Km, Dm, n_active, status, want_deriv=True,
                 stream=0) -> dict:
        """sdfc_batch_autotune on device inputs (pointers as for evaluate_device); returns the
        chosen launch configuration, which the batch keeps."""
        t = Tuning()
        self.ctx._check(lib().sdfc_batch_autotune(self._h, E_A, phi_A, E_B, phi_B, params, int(bool(want_deriv)), fm,
                                                  Km or 0, Dm or 0, n_active, status, stream, ctypes.byref(t)),
                        "sdfc_batch_autotune")
        return t.as_dict()

    def tuning(self) -> dict:
        t = Tuning()
        self.ctx._check(lib().sdfc_batch_get_tuning(self._h, ctypes.byref(t)), "sdfc_batch_get_tuning")
        return t.as_dict()

    def set_tuning(self, slots: int, force_variant: int, worker_ctas: int = 0, chunks_per_slot: int = 1):
        t = Tuning(int(slots), int(force_variant), int(worker_ctas), int(chunks_per_slot), 0.0)
        self.ctx._check(lib().sdfc_batch_set_tuning(self._h, ctypes.byref(t)), "sdfc_batch_set_tuning")

    def energy(self, E_A, E_B, params):
        """Penetration energy per instance (n,) and its gradient wrt both bodies' twists (n, 12)."""
        n = self.n
        pa = (Params * n)()
        for k in range(n):
            pa[k] = params[k] if isinstance(params, (list, tuple)) else params
        e, dE = np.zeros(n), np.zeros((n, 12))
        self.ctx._check(lib().sdfc_batch_energy(self._h, _dp(_f64(E_A, 16 * n)), _dp(_f64(E_B, 16 * n)), pa, _dp(e),
                                                _dp(dE)), "sdfc_batch_energy")
        return e, dE

    def evaluate_masked_device(self, E_A, phi_A, E_B, phi_B, params, request, fm, Km, Dm, n_active, status,
                               stream=0):
        """Device pointers; request (device int32[n]): 0 skip, 1 fm only, 2 fm, Km, Dm."""
        self.ctx._check(lib().sdfc_batch_evaluate_masked_device(self._h, E_A, phi_A, E_B, phi_B, params, request,
                                                                fm, Km, Dm, n_active, status, stream),
                        "sdfc_batch_evaluate_masked_device")

    def set_precision(self, precision: int):
        self.ctx._check(lib().sdfc_batch_set_precision(self._h, int(precision)), "sdfc_batch_set_precision")

    def set_timing(self, enable=True):
        self.ctx._check(lib().sdfc_batch_set_timing(self._h, int(bool(enable))), "sdfc_batch_set_timing")

    def last_timing(self):
        """(detect_ms, force_ms, reduce_ms) of the last evaluation."""
        ms = (ctypes.c_float * 3)()
        self.ctx._check(lib().sdfc_batch_last_timing(self._h, ms), "sdfc_batch_last_timing")
        return tuple(float(x) for x in ms)

    def recheck_count(self, reset=False) -> int:
        c = ctypes.c_ulonglong()
        self.ctx._check(lib().sdfc_batch_recheck_count(self._h, ctypes.byref(c), int(bool(reset))),
                        "sdfc_batch_recheck_count")
        return c.value


def evaluate_noalloc(grid_values_dev, shape, min_box, max_box, dx, col_th, points_dev, n, E_A, phi_A, E_B, phi_B,
                     params, fm, Km, Dm, n_active, want_deriv=True, stream=0):
    """sdfc_evaluate_noalloc: every array argument except min_box / max_box / dx is a device pointer (int).

    For callers that must not allocate device memory at call time; see include/sdfc.h."""
    ni, nj, nk = shape
    rc = lib().sdfc_evaluate_noalloc(grid_values_dev, ni, nj, nk, _dp(_f64(min_box, 3)), _dp(_f64(max_box, 3)),
                                     _dp(_f64(dx, 3)), float(col_th), points_dev, int(n), E_A, phi_A, E_B, phi_B,
                                     params, int(bool(want_deriv)), fm, Km or 0, Dm or 0, n_active, stream)
    if rc != SDFC_OK:
        raise SdfcError(f"sdfc_evaluate_noalloc failed ({rc})")


class Sim:
    """sdfc_sim: n planner scenes (one moving part each) stepped by batched BDF1 Newton."""

    def __init__(self, ctx: Context, movers, pairs):
        self.ctx = ctx
        self.n = len(movers)
        self.ndof = 6 if movers[0].joint == JOINT_FREE3D_EXP else 3
        marr = (Mover * self.n)(*movers)
        parr = (ScenePair * max(1, len(pairs)))(*pairs)
        self._h = ctypes.c_void_p()
        ctx._check(lib().sdfc_sim_create(ctx._h, self.n, marr, len(pairs), parr, ctypes.byref(self._h)),
                   "sdfc_sim_create")
        self.generation = 0  # bumped by every call that changes the state or the recording

    def close(self):
        if self._h and self.ctx._h:
            lib().sdfc_sim_destroy(self._h)
        self._h = ctypes.c_void_p()

    def set_precision(self, precision: int):
        self.ctx._check(lib().sdfc_sim_set_precision(self._h, int(precision)), "sdfc_sim_set_precision")

    def autotune(self) -> dict:
        """sdfc_sim_autotune: the fastest launch configuration for the sim's batch of pairs."""
        t = Tuning()
        self.ctx._check(lib().sdfc_sim_autotune(self._h, ctypes.byref(t)), "sdfc_sim_autotune")
        return t.as_dict()

    def tuning(self) -> dict:
        t = Tuning()
        self.ctx._check(lib().sdfc_sim_get_tuning(self._h, ctypes.byref(t)), "sdfc_sim_get_tuning")
        return t.as_dict()

    def set_tuning(self, slots: int, force_variant: int, worker_ctas: int = 0, chunks_per_slot: int = 1):
        t = Tuning(int(slots), int(force_variant), int(worker_ctas), int(chunks_per_slot), 0.0)
        self.ctx._check(lib().sdfc_sim_set_tuning(self._h, ctypes.byref(t)), "sdfc_sim_set_tuning")

    def set_state(self, q, qdot):
        self.generation += 1
        k = self.ndof * self.n
        self.ctx._check(lib().sdfc_sim_set_state(self._h, _dp(_f64(q, k)), _dp(_f64(qdot, k))), "sdfc_sim_set_state")

    def get_state(self):
        q, qd = np.zeros(self.ndof * self.n), np.zeros(self.ndof * self.n)
        self.ctx._check(lib().sdfc_sim_get_state(self._h, _dp(q), _dp(qd)), "sdfc_sim_get_state")
        return q.reshape(self.n, self.ndof), qd.reshape(self.n, self.ndof)

    def set_external_force(self, f):
        self.generation += 1
        self.ctx._check(lib().sdfc_sim_set_external_force(self._h, _dp(_f64(f, 6 * self.n))),
                        "sdfc_sim_set_external_force")

    def step(self, num_steps=1):
        self.generation += 1
        conv = np.zeros(self.n, dtype=np.int32)
        self.ctx._check(lib().sdfc_sim_step(self._h, int(num_steps), _ip(conv)), "sdfc_sim_step")
        return conv.astype(bool)

    def stats(self):
        r, e = ctypes.c_longlong(), ctypes.c_longlong()
        self.ctx._check(lib().sdfc_sim_stats(self._h, ctypes.byref(r), ctypes.byref(e)), "sdfc_sim_stats")
        return r.value, e.value

    def scene_evaluations(self) -> np.ndarray:
        """Force evaluations of each scene since creation (sdfc_sim_scene_evaluations)."""
        out = np.zeros(self.n, dtype=np.int64)
        self.ctx._check(lib().sdfc_sim_scene_evaluations(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))),
                        "sdfc_sim_scene_evaluations")
        return out

    # adjoint (Simulation::reset(backward_flag=True) / get_q_his / backward)
    def record(self, max_steps: int):
        """Record the trajectory from the current state for up to max_steps steps (0 stops)."""
        self.generation += 1
        self.ctx._check(lib().sdfc_sim_record(self._h, int(max_steps)), "sdfc_sim_record")

    def history(self):
        """Recorded joint trajectory, shape (n, T+1, ndof), q_0 first."""
        T = ctypes.c_int()
        self.ctx._check(lib().sdfc_sim_history(self._h, ctypes.byref(T), None), "sdfc_sim_history")
        q = np.zeros((self.n, T.value + 1, self.ndof))
        self.ctx._check(lib().sdfc_sim_history(self._h, ctypes.byref(T), _dp(q)), "sdfc_sim_history")
        return q

    def record_energy(self, on=True):
        """Also record each step's penetration energy (call before record(); stops a recording)."""
        self.generation += 1
        self.ctx._check(lib().sdfc_sim_record_energy(self._h, int(bool(on))), "sdfc_sim_record_energy")

    def energy(self):
        """Recorded penetration energies: per step (n, T) and their sum (n,)."""
        T = ctypes.c_int()
        self.ctx._check(lib().sdfc_sim_history(self._h, ctypes.byref(T), None), "sdfc_sim_history")
        per, tot = np.zeros((self.n, T.value)), np.zeros(self.n)
        self.ctx._check(lib().sdfc_sim_energy(self._h, _dp(per), _dp(tot)), "sdfc_sim_energy")
        return per, tot

    def set_tolerance(self, tol: float):
        """Newton tolerance on |g| (the reference's 1e-8 by default)."""
        self.ctx._check(lib().sdfc_sim_set_tolerance(self._h, float(tol)), "sdfc_sim_set_tolerance")

    def backward(self, df_dq, df_dE=None):
        """Simulation::backward_BDF1 over the recorded steps for dL/dq_k (n, T, ndof) and, with
        energy recording, dL/d(sum of the steps' penetration energies) df_dE (n,):
        returns dL/dq0 (n, ndof), dL/dqdot0 (n, ndof), dL/d(external force) (n, 6)."""
        df_dq = np.ascontiguousarray(df_dq, dtype=np.float64)
        if df_dq.ndim != 3 or df_dq.shape[0] != self.n or df_dq.shape[2] != self.ndof:
            raise ValueError(f"df_dq must have shape (n, T, {self.ndof})")
        T = ctypes.c_int()
        self.ctx._check(lib().sdfc_sim_history(self._h, ctypes.byref(T), None), "sdfc_sim_history")
        if df_dq.shape[1] != T.value:
            raise ValueError(f"df_dq covers {df_dq.shape[1]} steps, {T.value} recorded")
        g0, gd0, gf = np.zeros((self.n, self.ndof)), np.zeros((self.n, self.ndof)), np.zeros((self.n, 6))
        dfE = None if df_dE is None else _f64(df_dE, self.n)
        self.ctx._check(lib().sdfc_sim_backward_energy(self._h, _dp(df_dq), None if dfE is None else _dp(dfE), _dp(g0),
                                                       _dp(gd0), _dp(gf)), "sdfc_sim_backward_energy")
        return g0, gd0, gf


def f16_brick_encode(values):
    """sdfc_f16_brick_encode (host only): values (nk, nj, ni) -> (codes uint16 [nb*512], so float32 [nb, 2])."""
    v = _f64(values)
    nk, nj, ni = v.shape
    nb = ((ni + 7) // 8) * ((nj + 7) // 8) * ((nk + 7) // 8)
    codes = np.zeros(nb * 512, dtype=np.uint16)
    so = np.zeros((nb, 2), dtype=np.float32)
    rc = lib().sdfc_f16_brick_encode(_dp(v), ni, nj, nk, codes.ctypes.data, so.ctypes.data)
    if rc != SDFC_OK:
        raise SdfcError(f"sdfc_f16_brick_encode failed ({rc})")
    return codes, so


def f16_brick_decode(codes, so, shape):
    """sdfc_f16_brick_decode (host only): the FP64 grid (nk, nj, ni) the codes stand for."""
    nk, nj, ni = shape
    codes = np.ascontiguousarray(codes, dtype=np.uint16)
    so = np.ascontiguousarray(so, dtype=np.float32)
    out = np.zeros(shape)
    rc = lib().sdfc_f16_brick_decode(codes.ctypes.data, so.ctypes.data, ni, nj, nk, _dp(out))
    if rc != SDFC_OK:
        raise SdfcError(f"sdfc_f16_brick_decode failed ({rc})")
    return out


def sdf_grid_layout(V, dx, res):
    """sdfc_sdf_grid_layout (host only): BodySDFObj::precompute_SDF's grid for the body-frame
    vertices V (nv, 3) -> (shape (ni, nj, nk), min_box, max_box, spacing, origin float32)."""
    v = _f64(V).reshape(-1, 3)
    shape = (ctypes.c_int * 3)()
    mn, mx, sp = np.zeros(3), np.zeros(3), np.zeros(3)
    org = np.zeros(3, np.float32)
    rc = lib().sdfc_sdf_grid_layout(_dp(v), len(v), float(dx), int(res), shape, _dp(mn), _dp(mx), _dp(sp),
                                    org.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    if rc != SDFC_OK:
        raise SdfcError(f"sdfc_sdf_grid_layout failed ({rc})")
    return tuple(shape), mn, mx, sp, org


def save_sdf_text(path, values, min_box, max_box, dx):
    """sdfc_sdf_save_text: the reference's .sdf text cache of a grid (values (nk, nj, ni))."""
    v = _f64(values)
    nk, nj, ni = v.shape
    rc = lib().sdfc_sdf_save_text(str(path).encode(), _dp(v), ni, nj, nk, _dp(_f64(min_box, 3)),
                                  _dp(_f64(max_box, 3)), _dp(_f64(dx, 3)))
    if rc != SDFC_OK:
        raise SdfcError(f"sdfc_sdf_save_text failed ({rc}): {path}")


def load_sdf_text(path):
    """sdfc_sdf_load_text: (values (nk, nj, ni), min_box, max_box, dx) of a .sdf text cache,
    or None when the file does not open (as the reference's load_SDF reports)."""
    shape = (ctypes.c_int * 3)()
    mn, mx, dx = np.zeros(3), np.zeros(3), np.zeros(3)
    rc = lib().sdfc_sdf_load_text(str(path).encode(), shape, _dp(mn), _dp(mx), _dp(dx), None, 0)
    if rc == SDFC_ERR_NOT_FOUND:
        return None
    if rc != SDFC_OK:
        raise SdfcError(f"sdfc_sdf_load_text failed ({rc}): {path}")
    ni, nj, nk = shape
    v = np.zeros((nk, nj, ni))
    rc = lib().sdfc_sdf_load_text(str(path).encode(), shape, _dp(mn), _dp(mx), _dp(dx), _dp(v), v.size)
    if rc != SDFC_OK:
        raise SdfcError(f"sdfc_sdf_load_text failed ({rc}): {path}")
    return v, mn, mx, dx


def save_sdf_bricks(path, values, min_box, max_box, dx):
    """sdfc_sdf_save_bricks: the binary FP16-brick cache of a grid (values (nk, nj, ni))."""
    v = _f64(values)
    nk, nj, ni = v.shape
    rc = lib().sdfc_sdf_save_bricks(str(path).encode(), _dp(v), ni, nj, nk, _dp(_f64(min_box, 3)),
                                    _dp(_f64(max_box, 3)), _dp(_f64(dx, 3)))
    if rc != SDFC_OK:
        raise SdfcError(f"sdfc_sdf_save_bricks failed ({rc}): {path}")


def load_sdf_bricks(path):
    """sdfc_sdf_load_bricks: (codes, so, shape (nk, nj, ni), min_box, max_box, dx), or None when the
    file does not open."""
    shape = (ctypes.c_int * 3)()
    mn, mx, dx = np.zeros(3), np.zeros(3), np.zeros(3)
    rc = lib().sdfc_sdf_load_bricks(str(path).encode(), shape, _dp(mn), _dp(mx), _dp(dx), None, None)
    if rc == SDFC_ERR_NOT_FOUND:
        return None
    if rc != SDFC_OK:
        raise SdfcError(f"sdfc_sdf_load_bricks failed ({rc}): {path}")
    ni, nj, nk = shape
    nb = ((ni + 7) // 8) * ((nj + 7) // 8) * ((nk + 7) // 8)
    codes = np.zeros(nb * 512, np.uint16)
    so = np.zeros((nb, 2), np.float32)
    rc = lib().sdfc_sdf_load_bricks(str(path).encode(), shape, _dp(mn), _dp(mx), _dp(dx), codes.ctypes.data,
                                    so.ctypes.data)
    if rc != SDFC_OK:
        raise SdfcError(f"sdfc_sdf_load_bricks failed ({rc}): {path}")
    return codes, so, (nk, nj, ni), mn, mx, dx
