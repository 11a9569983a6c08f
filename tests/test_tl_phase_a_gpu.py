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


@pytest.mark.parametrize("flags", [0, 3, 32])
def test_b2_filter_rejects_only_what_exact_phase_b2_rejects(gpu, batch, flags):
    """The single-precision phase-B2 filter (tl_b2_quick) against the exact
    phases B1 and B2 on every phase-A survivor: it never rejects a candidate
    the exact phases accept and never accepts one exact phase B2 rejects, its
    bounds on deltaBeta, dBetaCut2 and betaOut hold (largest error / bound
    below 1; the decisions use four times the bounds), it rejects most of
    what the exact phases reject and accepts most of what they accept."""
    det, events = batch
    run_gpu(gpu, det, events, flags)
    r = gpu.tl_b2_filter_check()
    print(r)
    assert r["entries"] > 1_000_000, r
    assert r["violations"] == 0 and r["accept_violations"] == 0, r
    assert all(v < 1.0 for v in r["bound_ratio"].values()), r
    assert r["accepted"] >= 0.8 * r["b2_pass"], r
    failing = r["entries"] - r["b2_pass"]
    assert r["rejected"] >= 0.6 * failing, r
    lists = gpu.tl_list_counts()
    # the exact phases get what the filter neither rejected nor turned into a
    # tracklet (it accepts only entries whose phase B1 is decided already)
    assert lists["listed"] == r["entries"], (lists, r)
    assert r["entries"] - r["rejected"] - r["accepted"] <= lists["filtered"] <= r["entries"] - r["rejected"], (lists, r)


@pytest.mark.parametrize("flags", [0, 3, 32, 64])
def test_b2_filter_changes_no_object(gpu, batch, flags):
    """The chain with and without the phase-B2 filter (SDLG_FLAG_NO_B2_FILTER):
    the same objects and counters in every event, with and without the
    learned pre-filter."""
    import bench
    from sdl_gb300 import FLAG_MLP, FLAG_NO_B2_FILTER, mlp
    import oracle
    det, events = batch
    params, thr, _ = mlp.load(bench.MLP_WEIGHTS)
    gpu.upload_detector(det)
    gpu.mlp_set_params(params, thr)
    gpu.set_events(events)
    for extra in (0, FLAG_MLP):
        got = []
        for off in (0, FLAG_NO_B2_FILTER):
            gpu.run(4, flags | extra | off)
            got.append(([[oracle.digest(gpu.objects(s, e)) for s in range(5)] for e in range(len(events))],
                        [gpu.counters(e).tolist() for e in range(len(events))]))
        assert got[0] == got[1], (flags, extra)
        last = gpu.tl_list_counts()  # the last run had the filter off
        assert last["filtered"] == (last["kept"] if extra else last["listed"])
