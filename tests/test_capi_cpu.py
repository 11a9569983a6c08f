"""The C ABI library builds, loads and exports every entry point that
include/sdl_gpu.h declares (no device calls here)."""
import ctypes
import os
import re

from conftest import ROOT


def declared():
    with open(os.path.join(ROOT, "include", "sdl_gpu.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"\b(sdlg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_header_symbols():
    from sdl_gb300 import build, lib
    build.build()
    L = lib()
    names = declared()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), n


def test_create_without_device_reports_error():
    import sdl_gb300
    L = sdl_gb300.lib()
    h = ctypes.c_void_p()
    rc = L.sdlg_create(ctypes.byref(h), 0)
    if rc == 0:  # a GPU is present: nothing to check here
        L.sdlg_destroy(h)
    else:
        assert rc in (-9, -2)
