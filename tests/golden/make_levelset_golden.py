"""Generates tests/golden/levelset.npz from the reference's own mesh-to-SDF code.

Runs sdfgen::make_level_set3 (simulation/externals/sdfgen/makelevelset3.cpp:161-227) and a
whole BodySDFObj::precompute_SDF (simulation/redmax/Body/BodySDFObj.cpp:38-84, reached by
loading an SDF body from an OBJ file), compiled from the reference sources by
oracle/ref/Makefile (oracle/_ref/libredmax_ref.so), on procedural meshes:

  case_<name>_*  make_level_set3 inputs (verts, tris, origin, dx[3], shape, band) and phi
  body_*         a torus body loaded by the reference: its body-frame mesh V, F, the body's
                 dx and res, and the reference's grid (shape, min_box, max_box, spacing, values)

Usage (where the reference sources are present):
    make -C oracle/ref REF=<reference root> -j8 && python tests/golden/make_levelset_golden.py
"""
import importlib
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import refsim  # noqa: E402

W = importlib.import_module("assemble-them-all_gb300.workloads")


def cases():
    """(name, V, F, origin, dx3, shape, band): edge cases of the reference's loops."""
    out = []
    # vertices exactly on grid nodes and crossing rays through edges and vertices: the
    # orientation test's tie-breaking decides the parity
    V, F = W.box_mesh((0.5, 0.25, 0.25))
    out.append(("box_on_nodes", V, F, np.float32([-0.75, -0.5, -0.5]), [0.125] * 3, (13, 9, 9), 1))
    # anisotropic spacing, many thin side triangles
    V, F = W.cylinder_mesh(0.4, 0.5, 24)
    o, _ = W.level_set_grid(V, 0.05)
    out.append(("cylinder_aniso", V, F, o, [0.05, 0.04, 0.06], (21, 26, 22), 1))
    # a non-convex body with large triangles, band 2
    V, F = W.socket_mesh(1.0, 0.5, 1.0)
    o, s = W.level_set_grid(V, 0.1)
    out.append(("socket_band2", V, F, o, [0.1] * 3, s, 2))
    # a grid that holds only part of the mesh (vertices at negative grid coordinates,
    # crossings before the first node), band 0
    V, F = W.torus_mesh(0.6, 0.25, 32, 16)
    out.append(("torus_partial_band0", V, F, np.float32([-0.3, -0.95, -0.3]), [0.05] * 3, (30, 40, 13), 0))
    # a zero-area triangle (three collinear vertices) among the faces
    V, F = W.box_mesh((0.4, 0.4, 0.4))
    V = np.vstack([V, [[-0.2, 0.0, 0.1], [0.0, 0.0, 0.1], [0.2, 0.0, 0.1]]])
    F = np.vstack([F, [[8, 9, 10]]]).astype(np.int32)
    o, s = W.level_set_grid(V, 0.07)
    out.append(("box_degenerate", V, F, o, [0.07] * 3, s, 1))
    return out


def main():
    if not refsim.available():
        raise SystemExit("oracle/_ref/libredmax_ref.so missing: build it with make -C oracle/ref REF=<reference root>")
    blob = {}
    names = []
    for name, V, F, o, d, shape, band in cases():
        V32 = np.asarray(V, np.float32)
        phi = refsim.make_level_set3(V32, F, o, np.float32(d), shape, band)
        names.append(name)
        blob[f"case_{name}_verts"] = V32
        blob[f"case_{name}_tris"] = np.asarray(F, np.uint32)
        blob[f"case_{name}_origin"] = np.asarray(o, np.float32)
        blob[f"case_{name}_dx"] = np.asarray(d, np.float32)
        blob[f"case_{name}_shape"] = np.asarray(shape, np.int32)
        blob[f"case_{name}_band"] = np.int32(band)
        blob[f"case_{name}_phi"] = phi
        print(name, shape, "inside nodes", int((phi < 0).sum()))
    blob["cases"] = np.array(names)

    # a whole precompute_SDF through the reference's body loader
    wd = tempfile.mkdtemp(prefix="golden_ls_")
    V, F = W.torus_mesh(0.6, 0.25, 40, 20)
    Vb, Fb = W.box_mesh((0.5, 0.5, 0.5))
    refsim.write_obj(os.path.join(wd, "a.obj"), V, F)
    refsim.write_obj(os.path.join(wd, "b.obj"), Vb, Fb)
    dx, res = 0.04, 30
    sim = refsim.RefSim(refsim.two_body_xml("b.obj", "a.obj", dx=dx, res=res), wd)
    Vr, Fr = sim.mesh("B")
    vals, mn, mx, sp, _ = sim.sdf("B")
    # the scene loader reads dx as a float (rm/Simulation_Constructor.cpp:565-566)
    blob.update(body_V=Vr, body_F=Fr, body_dx=float(np.float32(dx)), body_res=res, body_shape=np.array(vals.shape[::-1]),
                body_min_box=mn, body_max_box=mx, body_spacing=sp, body_values=vals.astype(np.float32))
    assert np.array_equal(vals.astype(np.float32).astype(np.float64), vals)
    print("body grid", vals.shape[::-1], "spacing", sp)
    np.savez_compressed(os.path.join(HERE, "levelset.npz"), **blob)


if __name__ == "__main__":
    main()
