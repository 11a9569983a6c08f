"""The allocation-free mini-doublet entry point (sdlg_mini_doublets_static).

It exists for callers that may not allocate device memory while they process
events (frameworks that hand out all device memory from a pool they allocate
at start-up, plugins whose host owns the allocator).  Its output must equal
the regular entry point's (sdlg_set_events + sdlg_run + sdlg_get_objects)
exactly, call after call: the
calls share one fixed array, so a later call must not see the earlier one's
leftovers.  This file is collected last on purpose.
"""
import ctypes
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cudart():
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    return ctypes.CDLL(os.path.join("/usr/local/cuda/lib64", "libcudart.so"))


class DeviceArray:
    """Test-owned device memory (the entry point itself allocates nothing)."""

    def __init__(self, rt, host=None, nbytes=None):
        self.rt = rt
        self.nbytes = int(host.nbytes if host is not None else nbytes)
        self.p = ctypes.c_void_p()
        assert rt.cudaMalloc(ctypes.byref(self.p), ctypes.c_size_t(max(self.nbytes, 4))) == 0
        if host is not None:
            host = np.ascontiguousarray(host)
            assert rt.cudaMemcpy(self.p, host.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(self.nbytes), 1) == 0

    def get(self, dtype, count):
        out = np.empty(count, dtype=dtype)
        if out.nbytes:
            assert self.rt.cudaMemcpy(out.ctypes.data_as(ctypes.c_void_p), self.p, ctypes.c_size_t(out.nbytes), 2) == 0
        return out

    def free(self):
        self.rt.cudaFree(self.p)


def _static_call(ch, rt, ev, cap):
    bufs = [DeviceArray(rt, np.ascontiguousarray(a)) for a in (ev.x, ev.y, ev.z, ev.idx, ev.detid)]
    pairs = DeviceArray(rt, nbytes=cap * 8)
    count = DeviceArray(rt, np.zeros(1, np.int64))
    status = DeviceArray(rt, np.zeros(1, np.uint32))
    ch.mini_doublets_static(len(ev), *[b.p for b in bufs], pairs.p, cap, count.p, status.p, None)
    assert rt.cudaDeviceSynchronize() == 0
    n = int(count.get(np.int64, 1)[0])
    st = int(status.get(np.uint32, 1)[0])
    got = pairs.get(np.int32, 2 * min(n, cap)).reshape(-1, 2)
    for b in bufs + [pairs, count, status]:
        b.free()
    return got, n, st


def test_static_entry_matches_regular_entry_two_calls():
    import oracle
    from sdl_gb300 import Chain, SDLError, build, synth
    build.build()
    rt = _cudart()
    det = synth.detector("full")
    events = [synth.make_event(det, 31, "full", n_pu=700), synth.make_event(det, 32, "full", n_pu=1750),
              synth.make_event(det, 31, "full", n_pu=700)]
    ch = Chain(0)
    ch.upload_detector(det)
    for ev in events:  # consecutive calls share the fixed array
        ch.set_events([ev])
        ch.run(0)
        ref = ch.objects(0, 0)
        got, n, st = _static_call(ch, rt, ev, cap=len(ev) * 2)
        assert st == 0
        assert n == len(ref)
        assert np.array_equal(oracle.canon(got), oracle.canon(ref))
        # an output buffer smaller than the result: the full count, a clean
        # status, and the first pair_cap pairs, all of them mini-doublets
        few, n_few, st_few = _static_call(ch, rt, ev, cap=5)
        assert st_few == 0 and n_few == len(ref) and len(few) == min(5, len(ref))
        ref_rows = set(map(tuple, ref.tolist()))
        assert all(tuple(r) in ref_rows for r in few.tolist())
    # sizes beyond the fixed array are refused before anything is launched
    with pytest.raises(SDLError):
        ch.mini_doublets_static(131073, 1, 1, 1, 1, 1, 1, 0, 1, 1, None)
    ch.close()
