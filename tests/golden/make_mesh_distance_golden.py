"""Generates tests/golden/mesh_distance.npz from the reference's own distance queries and
SDF cache files.

Runs, from the reference build (oracle/_ref/libredmax_ref.so, compiled from the reference
sources by oracle/ref/Makefile):

  sdfmesh_*   redmax::SDFMesh (simulation/redmax/Mesh.cpp:41-198) of a socket mesh: its grid,
              distance() and min_distance() at seeded points inside, outside and on the box
  body_*      Simulation::get_body_distance both ways and body_in_contact
              (simulation/redmax/Simulation.cpp:276-303) for a torus body and a socket body at
              seeded poses
  text_*      the reference's .sdf text cache of a small SDFMesh (SDFMesh::save_SDF, Mesh.cpp:
              124-135) as bytes, and the grid the reference reads back from it (load_SDF)

Usage (where the reference sources are present):
    make -C oracle/ref REF=<reference root> -j8 && python tests/golden/make_mesh_distance_golden.py
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


def main():
    if not refsim.available():
        raise SystemExit("oracle/_ref/libredmax_ref.so missing: build it with make -C oracle/ref REF=<reference root>")
    rng = np.random.default_rng(20261204)
    blob = {}

    V, F = W.socket_mesh(1.0, 0.5, 1.0)
    m = refsim.RefSDFMesh(V, F, 0.05)
    vals, mn, mx, sp = m.grid()
    X = np.concatenate([rng.uniform(-1.15, 1.15, (3000, 3)),          # mostly inside the box
                        rng.uniform(-2.0, 2.0, (500, 3)),             # many outside
                        mn + sp * rng.integers(0, 40, (200, 3)),      # on grid nodes
                        np.array([mn, mx, [mx[0], 0.0, 0.0]])])       # box corners and a face
    d, dmin = m.distance(X)
    blob.update(sdfmesh_V=V, sdfmesh_F=F, sdfmesh_dx=0.05, sdfmesh_values=vals, sdfmesh_min_box=mn,
                sdfmesh_max_box=mx, sdfmesh_spacing=sp, sdfmesh_X=X, sdfmesh_d=d, sdfmesh_min=dmin)
    print("sdfmesh grid", vals.shape[::-1], "min distance", dmin)

    wd = tempfile.mkdtemp(prefix="golden_md_")
    Va, Fa = W.torus_mesh(0.45, 0.12, 24, 12)
    Vb, Fb = W.socket_mesh(1.0, 0.5, 1.0)
    refsim.write_obj(os.path.join(wd, "a.obj"), Va, Fa)
    refsim.write_obj(os.path.join(wd, "b.obj"), Vb, Fb)
    sim = refsim.RefSim(refsim.two_body_xml("a.obj", "b.obj", dx=0.05, res=20), wd)
    VA, _ = sim.mesh("A")
    VB, _ = sim.mesh("B")
    gA = sim.sdf("A")
    gB = sim.sdf("B")
    EA, EB, dab, dba, inc = [], [], [], [], []
    for k in range(24):
        # the torus hovering over the socket's top face (z = 1): overlapping, touching, apart
        R = W.rotvec_to_matrix(rng.normal(size=3) * 0.2)
        p = np.array([rng.normal() * 0.2, rng.normal() * 0.2, 1.0 + rng.uniform(-0.1, 0.35)])
        Ea = W.pose(R, p)
        Eb = W.pose(W.rotvec_to_matrix(rng.normal(size=3) * 0.1), rng.normal(size=3) * 0.05)
        sim.set_pose("A", Ea, np.zeros(6))
        sim.set_pose("B", Eb, np.zeros(6))
        EA.append(Ea)
        EB.append(Eb)
        dab.append(sim.body_distance("A", "B"))
        dba.append(sim.body_distance("B", "A"))
        inc.append(sim.body_in_contact("A", "B", 0.02))
    blob.update(body_VA=VA, body_VB=VB, body_gridA=gA[0], body_minA=gA[1], body_maxA=gA[2], body_dxA=gA[3],
                body_colA=gA[4], body_gridB=gB[0], body_minB=gB[1], body_maxB=gB[2], body_dxB=gB[3],
                body_colB=gB[4], body_EA=np.array(EA), body_EB=np.array(EB), body_dab=np.array(dab),
                body_dba=np.array(dba), body_in_contact=np.array(inc), body_eps=0.02)
    print("body distances", np.round(dab, 4), "in contact", sum(inc))

    V, F = W.box_mesh((0.5, 0.3, 0.2))
    path = os.path.join(wd, "box.sdf")
    m2 = refsim.RefSDFMesh(V, F, 0.06, "", path)
    with open(path, "rb") as f:
        text = f.read()
    back = refsim.RefSDFMesh(V, F, 0.06, path, "")
    tv, tmn, tmx, tsp = back.grid()
    gv, gmn, gmx, gsp = m2.grid()
    blob.update(text_bytes=np.frombuffer(text, np.uint8), text_values=gv, text_min_box=gmn, text_max_box=gmx,
                text_spacing=gsp, text_read_values=tv, text_read_min_box=tmn, text_read_max_box=tmx,
                text_read_spacing=tsp)
    print("text cache", len(text), "bytes; values changed by the round trip:", int((tv != gv).sum()))
    np.savez_compressed(os.path.join(HERE, "mesh_distance.npz"), **blob)


if __name__ == "__main__":
    main()
