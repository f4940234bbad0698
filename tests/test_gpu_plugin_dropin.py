"""The GPU Force plugin as a drop-in: one reference Simulation (the reference built from its own
sources with the plugin, oracle/_ref/libredmax_gpu_plugin.so) is stepped twice from the same
XML scene, once with the stock ForceGeneralSDFContact the XML parser creates
(simulation/redmax/Simulation_Constructor.cpp:300-312) and once with ForceGeneralSDFContactGPU
swapped in for it (same bodies, coefficients and scale).

  * a peg on a free3d-exp joint pushed into a socket: with the reference's derivative stencil
    (SDFC_DERIV_STENCIL) the trajectories agree to 1e-9 over 40 steps, including after the
    contact points and the SDF values are edited in place mid-run (the plugin must see edits);
    with the analytic cell derivatives (the default) to 1e-6;
  * a cuboid contact body (its contact points are BodyCuboid::get_general_contact_points,
    CollisionDetection.cpp:126-131) dropped onto an SDF box: 1e-9 with the stencil.

Runs in a spawned process, which loads the plugin library alone.  Skipped where the reference
sources are not present (neither SDFC_REFERENCE_ROOT nor a staged copy under baseline/_ref)."""
import multiprocessing as mp
import os
import sys

import numpy as np
import pytest

from conftest import ROOT, submodule
from oracle import refsim

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(refsim.reference_root() is None, reason="reference sources not present")]

STEPS = 40
CUBOID_XML = """
<redmax model="cuboid">
<option integrator="BDF1" timestep="0.005" gravity="0. 0. -9.8"/>
<robot>
  <link name="A">
    <joint name="A" type="free3d-exp" axis="0. 0. 0." pos="0.05 -0.03 0.72" quat="1 0 0 0" frame="WORLD" damping="0"/>
    <body name="A" type="cuboid" size="0.4 0.3 0.4" pos="0 0 0" quat="1 0 0 0" density="1" mu="0" rgba="1 1 1 1"/>
  </link>
</robot>
<robot>
  <link name="B">
    <joint name="B" type="fixed" pos="0 0 0" quat="1 0 0 0" frame="WORLD" damping="0"/>
    <body name="B" type="SDF" filename="b.obj" pos="0 0 0" quat="1 0 0 0" scale="1 1 1"
          transform_type="OBJ_TO_JOINT" density="1" dx="0.1" res="20" col_th="0.01" mu="0" rgba="1 1 1 1"/>
  </link>
</robot>
<contact>
  <general_SDF_contact general_body="A" SDF_body="B" kn="1e5" kt="1e3" mu="0.3" damping="1e3"/>
</contact>
</redmax>
"""


def _peg_scene(R, W, wd):
    """The peg-in-socket scene of the reference's simulation fixtures (tests/golden/make_golden.py)."""
    Va, Fa = R.box_mesh((0.3, 0.25, 0.9))
    Vb, Fb = R.box_mesh((1.0, 1.0, 1.0))
    R.write_obj(os.path.join(wd, "a.obj"), Va, Fa)
    R.write_obj(os.path.join(wd, "b.obj"), Vb, Fb)
    xml = R.two_body_xml("a.obj", "b.obj", joint_a="free3d-exp", kn=1e5, kt=1e3, mu=0.3, damping=1e3, timestep=5e-3,
                         gravity=(0.0, 0.0, -9.8), col_th=0.01)
    sim = R.RefSim(xml, wd)
    _, _, _, E0iA = sim.mass_props("A")
    _, _, _, E0iB = sim.mass_props("B")
    grid = W.socket_grid(48, dtype=np.float32)
    mn, mx, dx = grid.min_box, grid.max_box, grid.dx
    n = grid.values.shape[0]
    ax = [mn[a] + dx[a] * np.arange(n) for a in range(3)]
    Z, Y, X = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    world = np.stack([X, Y, Z], -1) @ E0iB[:3, :3].T + E0iB[:3, 3]
    vals = W.socket_sdf(world).astype(np.float32).astype(np.float64)
    sim.set_sdf("B", vals, mn, mx, dx, 0.01)
    pts = (W.peg_points(3000, seed=2) - E0iA[:3, 3]) @ E0iA[:3, :3]
    sim.set_contact_points("A", pts)
    return sim, (vals, mn, mx, dx, pts)


def _drive(args):
    """Child process: both simulations of one scene, stepped in lockstep."""
    kind, deriv_mode = args
    sys.path.insert(0, ROOT)
    import importlib
    import tempfile
    from oracle import refsim as R
    W = importlib.import_module("assemble-them-all_gb300.workloads")
    R.use_plugin_library()
    sims = []
    for gpu in (False, True):
        wd = tempfile.mkdtemp(prefix="dropin_")
        if kind == "peg":
            sim, data = _peg_scene(R, W, wd)
            q0 = np.array([0.012, 0.0, 0.0, 0.002, -0.003, 0.01])
            qd0 = np.array([0.5, 0.0, -0.2, 0.3, -0.1, 0.5])
            F = np.array([0.05, -0.1, 0.02, 2.0, 0.5, 1.0])
        else:
            Vb, Fb = R.box_mesh((0.5, 0.5, 0.5))
            R.write_obj(os.path.join(wd, "b.obj"), Vb, Fb)
            sim, data = R.RefSim(CUBOID_XML, wd), None
            q0 = np.zeros(6)
            qd0 = np.array([0.1, -0.2, -0.5, 0.4, 0.2, -0.3])
            F = np.zeros(6)
        if gpu:
            assert sim.use_gpu_contacts(deriv_mode) == 1
        sim.set_state_init(q0, qd0)
        sim.reset(False)
        sim.set_external_force("A", F)
        sims.append((sim, data))
    qs = [[], []]
    for step in range(STEPS):
        if kind == "peg" and step == STEPS // 2:
            # edits in place: every contact point moved, every SDF value shifted
            for sim, (vals, mn, mx, dx, pts) in sims:
                sim.set_contact_points("A", pts * 0.998 + 0.001)
                sim.set_sdf("B", vals - 2e-3, mn, mx, dx, 0.01)
        for k, (sim, _) in enumerate(sims):
            sim.forward(1)
            qs[k].append(sim.state()[0])
    return np.array(qs[0]), np.array(qs[1])


@pytest.fixture(scope="module")
def plugin_built():
    submodule("build").build()
    assert refsim.build_plugin()


@pytest.mark.parametrize("kind,deriv_mode,atol", [("peg", 1, 1e-9), ("peg", 0, 1e-6), ("cuboid", 1, 1e-9)])
def test_plugin_steps_like_the_stock_force(plugin_built, kind, deriv_mode, atol):
    with mp.get_context("spawn").Pool(1) as pool:
        q_ref, q_gpu = pool.apply(_drive, ((kind, deriv_mode),))
    assert np.abs(np.diff(q_ref, axis=0)).sum() > 1e-2  # the body moves
    np.testing.assert_allclose(q_gpu, q_ref, rtol=0, atol=atol)
