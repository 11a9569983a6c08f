"""createTrackletsViaNavigation, createTrackCandidatesFromTracklets and
createTrackCandidatesFromTriplets on the GPU against the CPU restatement
(mode bits = chain flag bits), objects and counters, on a batch with barrel,
tilted and endcap hits, an empty event and a PU event; alone and combined
(track candidates from triplets after module-map segments take the
segment-object path, after layer-pair segments the trial-segment path)."""
import numpy as np
import pytest

from test_gpu_parity import describe, run_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from sdl_gb300 import Chain, build
    build.build()
    return Chain(0)


@pytest.mark.parametrize("flags", [32, 64, 128, 32 | 64, 32 | 128, 32 | 4, 3 | 64, 1 | 128])
def test_variants_match_oracle(flags, gpu, oracle_lib):
    from sdl_gb300 import synth
    det = synth.detector("full")
    events = [synth.make_event(det, 950, "full", n_pu=350),
              synth.make_event(det, 951, "full", n_pu=0, n_signal=0, noise_frac=0.0),
              synth.make_event(det, 952, "full", n_pu=1050)]
    run_gpu(gpu, det, events, flags)
    orc = oracle_lib.Oracle(det)
    for e, ev in enumerate(events):
        ref, cnt, _ = orc.run(ev, mode=flags)
        for s in range(5):
            got = gpu.objects(s, e)
            assert oracle_lib.digest(got) == oracle_lib.digest(ref[s]), describe(oracle_lib, got, ref[s], s)
        assert np.array_equal(gpu.counters(e), cnt)
