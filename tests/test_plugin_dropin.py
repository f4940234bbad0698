"""The GPU Force plugin builds against the reference's own headers and links
with the reference objects and libsdfcontact (no GPU needed: build and symbol
resolution only).  Skipped where the reference sources are absent."""
import ctypes
import os

import pytest

from conftest import submodule
from oracle import refsim

pytestmark = pytest.mark.skipif(refsim.reference_root() is None, reason="reference sources not present")


def test_plugin_builds_and_links():
    submodule("build").build()
    assert refsim.build_plugin()
    so = refsim.PLUGIN_LIB_PATH
    lib = ctypes.CDLL(so)  # every symbol resolves (RTLD_NOW)
    assert lib is not None
