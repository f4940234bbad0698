"""The C-ABI library builds, loads and exports every symbol include/sdfc.h declares (no GPU needed)."""
import ctypes
import os
import re

from conftest import ROOT, submodule


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "sdfc.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(sdfc_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_header_symbols():
    lib_path = submodule("build").build()
    lib = ctypes.CDLL(lib_path)
    names = declared_symbols()
    assert len(names) >= 10
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(submodule("sdfc").EXPORTS)


def test_create_without_gpu_fails_cleanly():
    """On a machine without a usable device sdfc_create returns an error code, never crashes."""
    sdfc = submodule("sdfc")
    lib = sdfc.lib()
    h = ctypes.c_void_p()
    rc = lib.sdfc_create(ctypes.byref(h), 0)
    if rc == 0:
        lib.sdfc_destroy(h)
    else:
        assert rc == -2 and not h
    assert lib.sdfc_create(ctypes.byref(h), -1) != 0
