"""GB300-native point-vs-SDF penalty contact for the redmax simulator of Assemble-Them-All.

Import with ``importlib.import_module("assemble-them-all_gb300")`` (the package
directory name is not a Python identifier).  Submodules:
  sdfc       ctypes front end of libsdfcontact.so (include/sdfc.h)
  force      ForceGeneralSDFContact-style Force objects over the GPU library
  workloads  synthetic peg-in-hole inputs
  build      in-tree nvcc build of libsdfcontact.so
"""
