"""GB300-native point-vs-SDF penalty contact for the redmax simulator of Assemble-Them-All.

Import with ``importlib.import_module("assemble-them-all_gb300")`` (the package
directory name is not a Python identifier).  Submodules:
  sdfc       ctypes front end of libsdfcontact.so (include/sdfc.h): contexts, grid and
             point uploads, single and batched force evaluations, batched BDF1 scenes and
             their adjoint, launch tuning, planner distances, disassembly check, SDF files
  autograd   torch.autograd.Function over the batched rollout and its adjoint
  mesh       the planner-side SDFMesh / body-distance / disassembly-check objects
  scenes     planner scenes of procedural assemblies on one batched simulation
  workloads  seeded synthetic inputs (peg-in-hole, procedural assemblies, meshes)
  build      in-tree nvcc build of libsdfcontact.so
  plugin/    ForceGeneralSDFContactGPU, the C++ drop-in for the reference's Force
"""
