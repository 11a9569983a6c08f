"""The polynomial atan of the tracklet enumeration's phase-B1 decision
(atan01_approx in sdl_gb300/csrc/sdl_device.cuh), evaluated in float32 with
the header's own coefficients and the device's operation order (one rounded
multiply and one rounded add per step, no fused multiply-add), on every float
q in [0, 1]: within 1.76e-6 of atan(q).  The bound of phi_fast built on it
(2.5e-6) adds the quotient's and the reconstruction's roundings; the GPU
self-check (function 20) samples that on 2^28 points."""
import os
import re

import numpy as np

HEADER = os.path.join(os.path.dirname(__file__), "..", "sdl_gb300", "csrc", "sdl_device.cuh")


def coefficients():
    text = open(HEADER).read()
    m = re.search(r"kAtanP\[6\]\s*=\s*\{([^}]*)\}", text)
    assert m, "kAtanP not found"
    vals = [np.float32(float(v.strip().rstrip("f"))) for v in m.group(1).split(",")]
    assert len(vals) == 6
    return vals


def test_atan01_approx_bound_on_every_float():
    c = coefficients()
    top = int(np.float32(1.0).view(np.uint32))
    worst = 0.0
    chunk = 1 << 24
    for s0 in range(0, top + 1, chunk):
        q = np.arange(s0, min(top + 1, s0 + chunk), dtype=np.uint32).view(np.float32)
        s = q * q
        p = np.full_like(q, c[5])
        for k in (4, 3, 2, 1, 0):
            p = p * s + c[k]
        r = q * p
        worst = max(worst, float(np.max(np.abs(r.astype(np.float64) - np.arctan(q.astype(np.float64))))))
    assert worst <= 1.76e-6, worst
