"""The device's std::asin/atan/sin/cos/tan of floats against the host libm's
float functions (glibc's asinf, atanf, sinf, cosf, tanf), which are what the
reference calls: bit for bit on every non-negative float of each function's
domain in the chain (asin on [0, 0.95], atan on all floats, sin and cos on
[0, 6.3], tan on [0, 1.26]) and on the negated floats of a strided sample.
The chain's correctly rounded evaluation alone would differ from the host's
on 0.4-3 % of these floats."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FN = ("asin", "atan", "sin", "cos", "tan")
HI = (0.95, float("inf"), 6.3, 6.3, 1.26)
CHUNK = 1 << 27


@pytest.fixture(scope="module")
def gpu():
    from sdl_gb300 import Chain, build
    build.build()
    ch = Chain(0)
    yield ch
    ch.close()


@pytest.mark.parametrize("fn", range(5))
def test_device_libm_equals_host_libm(fn, gpu, oracle_lib):
    hi = int(np.float32(HI[fn]).view(np.uint32))
    moved = 0
    for start in range(0, hi + 1, CHUNK):
        n = min(CHUNK, hi + 1 - start)
        dev = gpu.libm_eval(fn, start, n)
        host = oracle_lib.libm_values(fn, start, n)
        bad = np.nonzero(dev.view(np.uint32) != host.view(np.uint32))[0]
        assert bad.size == 0, "%s: %d floats differ from the host libm, first x bits 0x%08x: device %r host %r" % (
            FN[fn], bad.size, start + bad[0], dev[bad[0]], host[bad[0]])
    # negative arguments (odd functions, and the even cos), every 97th float
    start = 0x80000000 + 0x39800000
    n = (0x80000000 + hi) - start + 1
    for s0 in range(start, start + n, CHUNK * 97):
        m = min(CHUNK, (start + n - s0))
        dev = gpu.libm_eval(fn, s0, m)[::97]
        host = oracle_lib.libm_values(fn, s0, m)[::97]
        assert np.array_equal(dev.view(np.uint32), host.view(np.uint32)), FN[fn] + " on negative floats"
    st = gpu.libm_stats(fn)
    assert st["tabulated"] > 0 and st["exceptions"] == 0
    moved += st["moved"]
    print("%s: %d tabulated floats, %d not correctly rounded in the host libm" % (FN[fn], st["tabulated"], st["moved"]))
