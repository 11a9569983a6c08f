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


def build_cpp_demo(tmpdir):
    """Compiles tests/cpp_event_api.cc against include/sdl_event.hpp and the library."""
    import subprocess
    from sdl_gb300 import build
    lib = build.build()
    exe = os.path.join(str(tmpdir), "cpp_event_api")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp_event_api.cc"), "-o", exe, lib,
                    "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    return exe


def test_cpp_event_api_builds_and_reports_missing_device(tmp_path):
    import subprocess
    from sdl_gb300 import synth
    exe = build_cpp_demo(tmp_path)
    det, ev = synth.workload_event("barrel_flat", 0)
    paths = det.write_files(str(tmp_path))
    hb = os.path.join(str(tmp_path), "hits.bin")
    ev.write_bin(hb)
    r = subprocess.run([exe, *paths, hb], capture_output=True, text=True)
    assert r.returncode in (0, 3), r.stderr


def test_null_context_is_an_argument_error():
    """Entry points that read results reject a null context with SDLG_ERR_ARG
    before touching a device (the tracklet debug dump, the decision
    self-check, the pass timers, the pre-filter counters)."""
    import sdl_gb300
    L = sdl_gb300.lib()
    n = ctypes.c_int64()
    buf = (ctypes.c_uint64 * 8)()
    f = (ctypes.c_float * 16)()
    i = (ctypes.c_int64 * 4)()
    assert L.sdlg_get_tracklet_vars(None, ctypes.c_int64(0), f, ctypes.c_int64(0), ctypes.byref(n)) == -1
    assert L.sdlg_tl_phase_a_check(None, buf) == -1
    assert L.sdlg_last_tl_pass_times(None, f) == -1
    assert L.sdlg_mlp_stats(None, i) == -1
