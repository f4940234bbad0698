"""The GPU Force plugin builds against the reference's own headers and links
with the reference objects and libsdfcontact (no GPU needed: build and symbol
resolution only).  Skipped where the reference sources are absent."""
import ctypes
import os
import subprocess

import pytest

from conftest import ROOT, submodule
from oracle import refsim

REF_SRC = os.path.join(refsim.REFERENCE_ROOT, "simulation", "redmax")
pytestmark = pytest.mark.skipif(not os.path.isdir(REF_SRC), reason="reference sources not present")


def test_plugin_builds_and_links():
    submodule("build").build()
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), f"REF={refsim.REFERENCE_ROOT}",
                           "-j8", "plugin-check"])
    so = os.path.join(ROOT, "oracle", "_ref", "libredmax_gpu_plugin.so")
    lib = ctypes.CDLL(so)  # every symbol resolves (RTLD_NOW)
    assert lib is not None
