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


def test_module_info_decodes_the_synthetic_detids():
    """sdlg_module_info (SDL::Module's detId decoding, Module.cc:159-358) on
    every sensor of the synthetic detector: layer, side, rod / ring, module,
    lower / upper sensor and partner as the generator laid them out."""
    import numpy as np
    from sdl_gb300 import module_info, synth
    det = synth.detector("full")
    ids = set(int(d) for d in det.detid)
    for d, inner in zip(det.detid[::7], det.is_inner[::7]):
        m = module_info(int(d))
        assert m["valid"]
        assert m["isLower"] == int(bool(inner))
        assert m["partnerDetId"] in ids and module_info(m["partnerDetId"])["partnerDetId"] == int(d)
        if m["subdet"] == 5:
            assert m["layer"] == (int(d) >> 20) & 7 and m["side"] == (int(d) >> 18) & 3
            assert m["moduleType"] == (0 if m["layer"] <= 3 else 1)
        else:
            assert m["subdet"] == 4 and m["ring"] == (int(d) >> 12) & 15
    assert not module_info(0x0123457)["valid"]


def test_hit_derived_quantities():
    """sdlg_hit_derived (Hit.cc:68-83): rt and r3 are float sums of float
    products under a double square root, phi is Phi_mpi_pi(M_PI + ATan2(-y, -x))."""
    import math
    import numpy as np
    from sdl_gb300 import hit_derived
    rng = np.random.default_rng(7)
    x, y, z = (rng.uniform(-120, 120, 1000).astype(np.float32) for _ in range(3))
    x[:3] = 0
    y[:2] = 0
    rt, phi, eta, r3 = hit_derived(x, y, z)
    for i in range(len(x)):
        X, Y, Z = np.float32(x[i]), np.float32(y[i]), np.float32(z[i])
        assert rt[i] == np.float32(math.sqrt(float(X * X + Y * Y)))
        assert r3[i] == np.float32(math.sqrt(float(X * X + Y * Y + Z * Z)))
        if X != 0:
            at = np.float32(math.atan2(float(-Y), float(-X)))
        else:
            at = np.float32(0.0 if Y == 0 else (math.pi / 2 if -Y > 0 else -math.pi / 2))
        p = np.float32(math.pi + float(at))
        while float(p) >= math.pi:
            p = np.float32(float(p) - 2 * math.pi)
        while float(p) < -math.pi:
            p = np.float32(float(p) + 2 * math.pi)
        assert phi[i] == p
        if rt[i] > 0:  # the float acosh of the float quotient r3 / rt
            ratio = float(np.float32(r3[i]) / np.float32(rt[i]))
            want = math.copysign(math.acosh(ratio), float(Z)) * (Z != 0)
            assert abs(float(eta[i]) - want) <= 2e-7 * max(1.0, abs(want))
