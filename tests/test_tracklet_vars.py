"""Debug dump of the tracklets' final cut variables (sdlg_get_tracklet_vars)
against the reference's own Tracklet recovars, recorded by the reference
driver into the golden fixtures: -999 for BBEE tracklets as in the
reference; bit-identical otherwise, including the values that go through the
reference's float std::asin (the chain reproduces the host libm's asinf,
which is not always correctly rounded)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_meta, golden_names, regenerate

FULL = [n for n in golden_names() if os.path.exists(os.path.join(GOLDEN, n + ".npz"))]
FLAGS = {"map": 0, "layer": 3, "nav": 32, "tctl": 64, "tctp": 128}


def test_fixtures_hold_the_reference_recovars():
    from sdl_gb300 import TL_VAR_NAMES
    for name in FULL:
        z = np.load(os.path.join(GOLDEN, name + ".npz"))
        assert z["tl_vars"].shape == (z["TL"].shape[0], len(TL_VAR_NAMES)), name
        assert np.all(np.isfinite(z["tl_vars"])), name  # every tracklet reaches the final block


@pytest.mark.gpu
@pytest.mark.parametrize("name", FULL)
def test_tracklet_vars_match_reference(name, oracle_lib):
    from sdl_gb300 import Chain, build
    build.build()
    meta = golden_meta(name)
    det, ev = regenerate(meta)
    ch = Chain(0)
    ch.upload_detector(det)
    ch.set_events([ev])
    ch.run(4, FLAGS[meta["mode"]])
    tl = ch.objects(2, 0)
    v = ch.tracklet_vars(0)[oracle_lib.canon_order(tl)]
    ref = np.load(os.path.join(GOLDEN, name + ".npz"))["tl_vars"]
    assert v.shape == ref.shape
    # BBEE tracklets: -999 in both (the reference records none of these)
    unset = ref[:, 0] == -999.0
    assert np.array_equal(v[unset], ref[unset])
    # the others: bit-identical
    exact_rows = np.all(v.view(np.uint32) == ref.view(np.uint32), axis=1)
    assert exact_rows.all(), (exact_rows.mean(), np.argwhere(~exact_rows)[:5])
    ch.close()
