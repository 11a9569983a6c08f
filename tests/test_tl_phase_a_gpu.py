"""The tracklet enumeration's single-precision decisions (tl_ab1_decide:
phase A, then phase B1 for its survivors) against the exact cuts (tl_phaseA,
tl_phaseB1_sgv) on every tracklet candidate of a batch at PU 100, 200 and
300, for the module-map, layer-pair, Nm1 and navigation candidate sets: they
never settle a candidate differently, and they leave only a small share of
them to the exact cuts.  The object sets of the chain that uses them are
checked against the reference and the oracle elsewhere."""
import pytest

from test_gpu_parity import run_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from sdl_gb300 import Chain, build
    build.build()
    return Chain(0)


@pytest.fixture(scope="module")
def batch():
    from sdl_gb300 import synth
    det = synth.detector("full")
    return det, [synth.make_event(det, 970 + k, "full", n_pu=n) for k, n in enumerate((3500, 7000, 10500))]


@pytest.mark.parametrize("flags", [0, 3, 4, 32])
def test_phase_a_decision_matches_exact_cuts(gpu, batch, flags):
    det, events = batch
    run_gpu(gpu, det, events, flags)
    r = gpu.tl_phase_a_check()
    assert r["candidates"] > 1_000_000, r
    assert r["settled"] + r["exact"] == r["candidates"], r
    assert r["mismatches"] == 0, r
    assert r["exact"] <= 1e-2 * r["candidates"], r
