"""ORACLE — test infrastructure, not the product.

ctypes front end of ``oracle/_ref/libredmax_ref.so``: the reference redmax
simulator compiled from its own sources (``oracle/ref/Makefile``) plus the
extern "C" harness ``oracle/ref/ref_harness.cpp``.  It exists only where the
reference sources are present; it pins the C restatement and generates the
golden fixtures.  Nothing outside ``tests/`` and ``tests/golden/`` uses it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_ref", "libredmax_ref.so")
PLUGIN_LIB_PATH = os.path.join(_HERE, "_ref", "libredmax_gpu_plugin.so")
# The reference project's root: SDFC_REFERENCE_ROOT, else the copy of its sources that
# `make -C oracle/ref stage` puts under baseline/_ref/src (git-ignored); None where neither exists.
_STAGED = os.path.join(os.path.dirname(_HERE), "baseline", "_ref", "src")


def reference_root():
    for root in (os.environ.get("SDFC_REFERENCE_ROOT"), _STAGED):
        if root and os.path.isdir(os.path.join(root, "simulation", "redmax")):
            return root
    return None


def available() -> bool:
    return os.path.exists(LIB_PATH)


def build(jobs: int = None) -> bool:
    """Compile the reference + harness if the reference sources are present."""
    root = reference_root()
    if root is None:
        return False
    jobs = jobs or max(1, min(16, os.cpu_count() or 1))
    subprocess.check_call(["make", "-s", "-C", os.path.join(_HERE, "ref"), f"REF={root}", f"-j{jobs}"])
    return available()


def build_plugin(jobs: int = None) -> bool:
    """Compile the reference objects with the GPU Force plugin and its swap hook
    (oracle/_ref/libredmax_gpu_plugin.so; libsdfcontact must be built)."""
    root = reference_root()
    if root is None:
        return False
    jobs = jobs or max(1, min(16, os.cpu_count() or 1))
    subprocess.check_call(["make", "-s", "-C", os.path.join(_HERE, "ref"), f"REF={root}", f"-j{jobs}",
                           "plugin-check"])
    return os.path.exists(PLUGIN_LIB_PATH)


_lib = None


def use_plugin_library():
    """Makes this module drive libredmax_gpu_plugin.so (the reference objects, the harness and the
    GPU plugin in one library) instead of libredmax_ref.so; the two are never loaded together.
    Afterwards RefSim.use_gpu_contacts is available."""
    global _lib
    if _lib is not None and getattr(_lib, "_path", None) == PLUGIN_LIB_PATH:
        return _lib
    if _lib is not None:
        raise RuntimeError("the reference library is already loaded in this process")
    L = _declare(ctypes.CDLL(PLUGIN_LIB_PATH))
    L.ref_sim_use_gpu_contacts.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L._path = PLUGIN_LIB_PATH
    _lib = L
    return L


def lib():
    global _lib
    if _lib is None:
        _lib = _declare(ctypes.CDLL(LIB_PATH))
    return _lib


def _declare(L):
    if True:
        d, i, c = ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_char_p
        v = ctypes.c_void_p
        L.ref_sim_create.restype = v
        L.ref_sim_create.argtypes = [c, c]
        L.ref_sim_destroy.argtypes = [v]
        L.ref_sim_ndof.argtypes = [v, ctypes.POINTER(i), ctypes.POINTER(i)]
        L.ref_body_index.argtypes = [v, c]
        L.ref_body_mass_props.argtypes = [v, c, d, d, d, d]
        L.ref_body_num_contact_points.argtypes = [v, c]
        L.ref_body_get_contact_points.argtypes = [v, c, d, i]
        L.ref_body_set_contact_points.argtypes = [v, c, d, i]
        L.ref_body_set_sdf.argtypes = [v, c, i, i, i, d, d, d, ctypes.c_double, d]
        L.ref_body_get_sdf_shape.argtypes = [v, c, ctypes.POINTER(i), d, d, d, d]
        L.ref_body_get_sdf_values.argtypes = [v, c, d]
        L.ref_body_set_pose.argtypes = [v, c, d, d]
        L.ref_body_set_contact_scale.argtypes = [v, c, ctypes.c_double]
        L.ref_collision.argtypes = [v, c, d, d, i, d]
        L.ref_distance.argtypes = [v, c, d, i, d]
        L.ref_pair_eval.argtypes = [v, c, c] + [ctypes.c_double] * 5 + [i, d, d, d, ctypes.POINTER(i), i,
                                                                         ctypes.POINTER(i)]
        L.ref_sim_reset.argtypes = [v, i]
        L.ref_sim_set_state_init.argtypes = [v, d, d]
        L.ref_sim_set_external_force.argtypes = [v, c, d]
        L.ref_sim_forward.argtypes = [v, i]
        L.ref_sim_is_converged.argtypes = [v]
        L.ref_sim_get_state.argtypes = [v, d, d]
        L.ref_sim_backward.argtypes = [v, d, i, d, d]
        L.ref_body_mesh.argtypes = [v, c, ctypes.POINTER(i), ctypes.POINTER(i), d, ctypes.POINTER(i)]
        L.ref_sdfmesh_create.restype = v
        L.ref_sdfmesh_create.argtypes = [d, i, ctypes.POINTER(i), i, ctypes.c_double, c, c]
        L.ref_sdfmesh_destroy.argtypes = [v]
        L.ref_sdfmesh_shape.argtypes = [v, ctypes.POINTER(i), d, d, d]
        L.ref_sdfmesh_values.argtypes = [v, d]
        L.ref_sdfmesh_distance.argtypes = [v, d, i, d, d]
        L.ref_body_distance.argtypes = [v, c, c, d]
        L.ref_body_in_contact.argtypes = [v, c, c, ctypes.c_double]
        f = ctypes.POINTER(ctypes.c_float)
        L.ref_make_level_set3.argtypes = [f, i, ctypes.POINTER(ctypes.c_uint), i, f, ctypes.c_float,
                                          ctypes.c_float, ctypes.c_float, i, i, i, i, f]
    return L


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _f64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"reference harness: {what} failed ({rc})")


# --------------------------------------------------------------------------- scene files

def write_obj(path, V, F):
    with open(path, "w") as f:
        for v in V:
            f.write(f"v {v[0]:.9g} {v[1]:.9g} {v[2]:.9g}\n")
        for t in F:
            f.write(f"f {t[0] + 1} {t[1] + 1} {t[2] + 1}\n")


def box_mesh(half=(0.5, 0.5, 0.5), center=(0.0, 0.0, 0.0)):
    hx, hy, hz = half
    cx, cy, cz = center
    V = np.array([[cx + sx * hx, cy + sy * hy, cz + sz * hz]
                  for sz in (-1, 1) for sy in (-1, 1) for sx in (-1, 1)])
    F = np.array([[0, 2, 1], [1, 2, 3], [4, 5, 6], [5, 7, 6], [0, 1, 4], [1, 5, 4],
                  [2, 6, 3], [3, 6, 7], [0, 4, 2], [2, 4, 6], [1, 3, 5], [3, 7, 5]])
    return V, F


def two_body_xml(obj_a, obj_b, joint_a="free3d-exp", dx=0.1, col_th=0.01, kn=1e5, kt=1e3, mu=0.3, damping=1e3,
                 timestep=5e-3, gravity=(0.0, 0.0, -9.8), pos_a=(0.0, 0.0, 0.0), res=20):
    """XML for a moving contact body A ("A", joint `joint_a`) against a fixed SDF body B ("B").

    Follows the planner's scene layout (examples/run_joint_plan.py:140-178): both bodies are SDF bodies
    with OBJ_TO_JOINT transforms; only the A-points-vs-B-grid contact is listed."""
    g = " ".join(repr(float(x)) for x in gravity)
    pa = " ".join(repr(float(x)) for x in pos_a)
    return f"""
<redmax model="pair">
<option integrator="BDF1" timestep="{timestep!r}" gravity="{g}"/>
<robot>
  <link name="A">
    <joint name="A" type="{joint_a}" axis="0. 0. 0." pos="{pa}" quat="1 0 0 0" frame="WORLD" damping="0"/>
    <body name="A" type="SDF" filename="{obj_a}" pos="0 0 0" quat="1 0 0 0" scale="1 1 1"
          transform_type="OBJ_TO_JOINT" density="1" dx="{dx!r}" res="{res}" col_th="{col_th!r}" mu="0"
          rgba="1 1 1 1"/>
  </link>
</robot>
<robot>
  <link name="B">
    <joint name="B" type="fixed" pos="0 0 0" quat="1 0 0 0" frame="WORLD" damping="0"/>
    <body name="B" type="SDF" filename="{obj_b}" pos="0 0 0" quat="1 0 0 0" scale="1 1 1"
          transform_type="OBJ_TO_JOINT" density="1" dx="{dx!r}" res="{res}" col_th="{col_th!r}" mu="0"
          rgba="1 1 1 1"/>
  </link>
</robot>
<contact>
  <general_SDF_contact general_body="A" SDF_body="B" kn="{kn!r}" kt="{kt!r}" mu="{mu!r}" damping="{damping!r}"/>
</contact>
</redmax>
"""


class RefSim:
    """One reference Simulation built from an XML string (rm/Simulation_Constructor.cpp:123)."""

    def __init__(self, xml: str, asset_folder: str):
        self._h = lib().ref_sim_create(xml.encode(), asset_folder.encode())
        if not self._h:
            raise RuntimeError("reference Simulation construction failed")
        nr, nm = ctypes.c_int(), ctypes.c_int()
        lib().ref_sim_ndof(self._h, ctypes.byref(nr), ctypes.byref(nm))
        self.ndof_r, self.ndof_m = nr.value, nm.value

    def close(self):
        if self._h:
            lib().ref_sim_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # bodies -------------------------------------------------------------
    def mass_props(self, name):
        m = np.zeros(1)
        I = np.zeros(6)
        Eji = np.zeros(16)
        E0i = np.zeros(16)
        _check(lib().ref_body_mass_props(self._h, name.encode(), _dp(m), _dp(I), _dp(Eji), _dp(E0i)), "mass_props")
        return float(m[0]), I, Eji.reshape(4, 4), E0i.reshape(4, 4)

    def contact_points(self, name):
        n = lib().ref_body_num_contact_points(self._h, name.encode())
        out = np.zeros((n, 3))
        lib().ref_body_get_contact_points(self._h, name.encode(), _dp(out), n)
        return out

    def set_contact_points(self, name, pts):
        p = _f64(pts).reshape(-1, 3)
        _check(lib().ref_body_set_contact_points(self._h, name.encode(), _dp(p), len(p)), "set_contact_points")

    def set_sdf(self, name, values, min_box, max_box, dx, col_th):
        v = _f64(values)
        nk, nj, ni = v.shape
        _check(lib().ref_body_set_sdf(self._h, name.encode(), ni, nj, nk, _dp(_f64(min_box)), _dp(_f64(max_box)),
                                      _dp(_f64(dx)), float(col_th), _dp(v)), "set_sdf")

    def sdf(self, name):
        nijk = (ctypes.c_int * 3)()
        mn, mx, dx, ct = np.zeros(3), np.zeros(3), np.zeros(3), np.zeros(1)
        _check(lib().ref_body_get_sdf_shape(self._h, name.encode(), nijk, _dp(mn), _dp(mx), _dp(dx), _dp(ct)),
               "sdf_shape")
        ni, nj, nk = nijk
        v = np.zeros((nk, nj, ni))
        lib().ref_body_get_sdf_values(self._h, name.encode(), _dp(v))
        return v, mn, mx, dx, float(ct[0])

    def mesh(self, name):
        """The body-frame vertices (nv, 3) and faces (nt, 3) the body's SDF was built from."""
        nv, nt = ctypes.c_int(), ctypes.c_int()
        _check(lib().ref_body_mesh(self._h, name.encode(), ctypes.byref(nv), ctypes.byref(nt), None, None), "mesh")
        V = np.zeros((nv.value, 3))
        F = np.zeros((nt.value, 3), np.int32)
        _check(lib().ref_body_mesh(self._h, name.encode(), ctypes.byref(nv), ctypes.byref(nt), _dp(V),
                                   F.ctypes.data_as(ctypes.POINTER(ctypes.c_int))), "mesh")
        return V, F

    def body_distance(self, name_from, name_to):
        """Simulation::get_body_distance (rm/Simulation.cpp:276-296)."""
        out = np.zeros(1)
        _check(lib().ref_body_distance(self._h, name_from.encode(), name_to.encode(), _dp(out)), "body_distance")
        return float(out[0])

    def body_in_contact(self, a, b, eps):
        r = lib().ref_body_in_contact(self._h, a.encode(), b.encode(), float(eps))
        if r < 0:
            raise RuntimeError("reference harness: body_in_contact failed")
        return bool(r)

    def set_pose(self, name, E, phi):
        _check(lib().ref_body_set_pose(self._h, name.encode(), _dp(_f64(E)), _dp(_f64(phi))), "set_pose")

    def set_contact_scale(self, name, s):
        _check(lib().ref_body_set_contact_scale(self._h, name.encode(), float(s)), "set_contact_scale")

    # queries ------------------------------------------------------------
    def collision(self, name, xw, xw_dot, want_deriv=True):
        out = np.zeros(146)
        _check(lib().ref_collision(self._h, name.encode(), _dp(_f64(xw)), _dp(_f64(xw_dot)), int(want_deriv),
                                   _dp(out)), "collision")
        return out if want_deriv else out[:11]

    def distance(self, name, xw):
        p = _f64(xw).reshape(-1, 3)
        out = np.zeros(len(p))
        _check(lib().ref_distance(self._h, name.encode(), _dp(p), len(p), _dp(out)), "distance")
        return out

    def pair_eval(self, a, b, kn, kt, mu, damping, scale=1.0, want_deriv=True):
        fm, Km, Dm = np.zeros(12), np.zeros(144), np.zeros(144)
        cap = max(lib().ref_body_num_contact_points(self._h, a.encode()), 1)
        ids = np.zeros(cap, dtype=np.int32)
        n = ctypes.c_int()
        _check(lib().ref_pair_eval(self._h, a.encode(), b.encode(), kn, kt, mu, damping, scale, int(want_deriv),
                                   _dp(fm), _dp(Km), _dp(Dm), ids.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                   cap, ctypes.byref(n)), "pair_eval")
        return fm, Km.reshape(12, 12), Dm.reshape(12, 12), ids[:n.value].copy()

    def pair_force(self, a, b, kn, kt, mu, damping, scale=1.0, want_deriv=True):
        """One ForceGeneralSDFContact call (pair_eval without the active-id listing)."""
        fm, Km, Dm = np.zeros(12), np.zeros(144), np.zeros(144)
        n = ctypes.c_int()
        _check(lib().ref_pair_eval(self._h, a.encode(), b.encode(), kn, kt, mu, damping, scale, int(want_deriv),
                                   _dp(fm), _dp(Km), _dp(Dm), None, 0, ctypes.byref(n)), "pair_force")
        return fm, Km.reshape(12, 12), Dm.reshape(12, 12)

    # stepping -----------------------------------------------------------
    def reset(self, backward=False):
        _check(lib().ref_sim_reset(self._h, int(backward)), "reset")

    def set_state_init(self, q, qdot):
        _check(lib().ref_sim_set_state_init(self._h, _dp(_f64(q)), _dp(_f64(qdot))), "set_state_init")

    def set_external_force(self, name, f6):
        _check(lib().ref_sim_set_external_force(self._h, name.encode(), _dp(_f64(f6))), "set_external_force")

    def forward(self, n):
        _check(lib().ref_sim_forward(self._h, int(n)), "forward")

    def is_converged(self):
        return bool(lib().ref_sim_is_converged(self._h))

    def state(self):
        q, qd = np.zeros(self.ndof_r), np.zeros(self.ndof_r)
        _check(lib().ref_sim_get_state(self._h, _dp(q), _dp(qd)), "get_state")
        return q, qd

    def use_gpu_contacts(self, deriv_mode=0):
        """Puts ForceGeneralSDFContactGPU in place of every ForceGeneralSDFContact of this
        simulation (use_plugin_library first); returns how many were replaced."""
        n = lib().ref_sim_use_gpu_contacts(self._h, int(deriv_mode))
        if n < 0:
            raise RuntimeError("reference harness: use_gpu_contacts failed")
        return n

    def backward(self, df_dq, T):
        g0, gd0 = np.zeros(self.ndof_r), np.zeros(self.ndof_r)
        _check(lib().ref_sim_backward(self._h, _dp(_f64(df_dq)), int(T), _dp(g0), _dp(gd0)), "backward")
        return g0, gd0


def make_pair_sim(joint_a="free3d-exp", half_a=(0.3, 0.3, 0.3), half_b=(0.5, 0.5, 0.5), workdir=None, **kw):
    """A two-box reference scene whose grid / points the caller overwrites."""
    workdir = workdir or tempfile.mkdtemp(prefix="refsim_")
    Va, Fa = box_mesh(half_a)
    Vb, Fb = box_mesh(half_b)
    write_obj(os.path.join(workdir, "a.obj"), Va, Fa)
    write_obj(os.path.join(workdir, "b.obj"), Vb, Fb)
    xml = two_body_xml("a.obj", "b.obj", joint_a=joint_a, **kw)
    return RefSim(xml, workdir), workdir


def make_level_set3(verts, tris, origin, dx, shape, exact_band=1) -> np.ndarray:
    """The reference's own sdfgen::make_level_set3 (FP32 inputs, phi[k, j, i])."""
    L = lib()
    fp = ctypes.POINTER(ctypes.c_float)
    V = np.ascontiguousarray(verts, np.float32)
    T = np.ascontiguousarray(tris, np.uint32)
    o = np.ascontiguousarray(origin, np.float32)
    d = np.broadcast_to(np.asarray(dx, np.float32), (3,))
    ni, nj, nk = (int(s) for s in shape)
    phi = np.empty((nk, nj, ni), np.float32)
    _check(L.ref_make_level_set3(V.ctypes.data_as(fp), len(V), T.ctypes.data_as(ctypes.POINTER(ctypes.c_uint)),
                                 len(T), o.ctypes.data_as(fp), float(d[0]), float(d[1]), float(d[2]), ni, nj, nk,
                                 int(exact_band), phi.ctypes.data_as(fp)), "make_level_set3")
    return phi


class RefSDFMesh:
    """The reference's redmax::SDFMesh (rm/Mesh.cpp:41-198): V (nv, 3), F (nt, 3)."""

    def __init__(self, V, F, dx, load_path="", save_path=""):
        V = _f64(V).reshape(-1, 3)
        F = np.ascontiguousarray(F, np.int32).reshape(-1, 3)
        self._h = lib().ref_sdfmesh_create(_dp(V), len(V), F.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(F),
                                           float(dx), load_path.encode(), save_path.encode())
        if not self._h:
            raise RuntimeError("reference SDFMesh construction failed")

    def close(self):
        if self._h:
            lib().ref_sdfmesh_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def grid(self):
        nijk = (ctypes.c_int * 3)()
        mn, mx, dx = np.zeros(3), np.zeros(3), np.zeros(3)
        lib().ref_sdfmesh_shape(self._h, nijk, _dp(mn), _dp(mx), _dp(dx))
        ni, nj, nk = nijk
        v = np.zeros((nk, nj, ni))
        lib().ref_sdfmesh_values(self._h, _dp(v))
        return v, mn, mx, dx

    def distance(self, X):
        """SDFMesh::distance and min_distance of X (n, 3)."""
        X = _f64(X).reshape(-1, 3)
        d = np.zeros(len(X))
        m = np.zeros(1)
        _check(lib().ref_sdfmesh_distance(self._h, _dp(X), len(X), _dp(d), _dp(m)), "sdfmesh_distance")
        return d, float(m[0])
