"""GPU chain (libsdlgpu.so through its C ABI) against the reference's object
sets: the golden fixtures from the unmodified reference, and the CPU
restatement on the same inputs.  Integer/index work: bit-exact multisets."""
import numpy as np
import pytest

from conftest import golden_meta, golden_names, golden_tuples, regenerate

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from sdl_gb300 import Chain, build
    build.build()
    return Chain(0)


def describe(oracle, a, b, stage):
    extra, missing = oracle.multiset_diff(a, b)
    return "%s: gpu %d vs ref %d; extra %s missing %s" % (oracle.STAGES[stage], len(a), len(b), extra[:4], missing[:4])


def run_gpu(gpu, det, events, flags=0):
    gpu.upload_detector(det)
    gpu.set_events(events)
    gpu.run(4, flags)
    return gpu


# fixture mode -> chain flags: "layer" fixtures were made with the
# reference's createSegments + createTracklets (layer pairs); "nav" with
# createTrackletsViaNavigation; "tctl" / "tctp" with
# createTrackCandidatesFromTracklets / FromTriplets
FLAGS = {"map": 0, "layer": 3, "nav": 32, "tctl": 64, "tctp": 128}


@pytest.mark.parametrize("name", golden_names())
def test_gpu_matches_reference_golden(name, gpu, oracle_lib):
    meta = golden_meta(name)
    det, ev = regenerate(meta)
    run_gpu(gpu, det, [ev], FLAGS[meta["mode"]])
    full = golden_tuples(name)
    for s in range(5):
        got = gpu.objects(s, 0)
        if full is not None:
            ref = full[s]
            assert oracle_lib.canon(got).shape == ref.shape and np.array_equal(oracle_lib.canon(got), ref), \
                describe(oracle_lib, got, ref, s)
        assert oracle_lib.digest(got) == meta["digests"][s], "%s digest (n=%d vs %d)" % (
            oracle_lib.STAGES[s], len(got), meta["counts"][s])
    assert [int(v) for v in gpu.counters(0)] == meta["counters"]


def test_gpu_matches_oracle_batch_uneven(gpu, oracle_lib):
    """One batch of events of uneven size (including an empty one) against
    the CPU restatement event by event."""
    from sdl_gb300 import synth
    det = synth.detector("full")
    events = []
    for k, pu in enumerate((10, 60, 0, 25, 140)):
        if pu == 0:
            e = synth.make_event(det, 900 + k, "full", n_pu=0, n_signal=0, noise_frac=0.0)
        else:
            e = synth.make_event(det, 900 + k, "full", n_pu=int(7000 * pu / 200))
        events.append(e)
    run_gpu(gpu, det, events)
    orc = oracle_lib.Oracle(det)
    for e, ev in enumerate(events):
        ref, cnt, _ = orc.run(ev)
        for s in range(5):
            got = gpu.objects(s, e)
            assert oracle_lib.digest(got) == oracle_lib.digest(ref[s]), describe(oracle_lib, got, ref[s], s)
        assert np.array_equal(gpu.counters(e), cnt)
    tot = gpu.counts(-1)
    assert tot[4] == sum(len(orc.run(ev)[0][4]) for ev in events)


@pytest.mark.parametrize("flags", [1, 2, 3, 3 | 4])
def test_layer_pair_variants_match_oracle(flags, gpu, oracle_lib):
    """createSegments / createTracklets (layer pairs), alone and together, on
    a batch with barrel, tilted and endcap hits and an empty event, against
    the CPU restatement (mode bits = chain flag bits), counters included."""
    from sdl_gb300 import synth
    det = synth.detector("full")
    events = [synth.make_event(det, 940, "full", n_pu=350),
              synth.make_event(det, 941, "full", n_pu=0, n_signal=0, noise_frac=0.0),
              synth.make_event(det, 942, "full", n_pu=1050)]
    run_gpu(gpu, det, events, flags)
    orc = oracle_lib.Oracle(det)
    for e, ev in enumerate(events):
        ref, cnt, _ = orc.run(ev, mode=flags)
        for s in range(5):
            got = gpu.objects(s, e)
            assert oracle_lib.digest(got) == oracle_lib.digest(ref[s]), describe(oracle_lib, got, ref[s], s)
        assert np.array_equal(gpu.counters(e), cnt)


def test_graph_and_direct_launch_agree(gpu, oracle_lib):
    from sdl_gb300 import FLAG_NO_GRAPH, synth
    det, ev = synth.workload_event("pu", 7, pu=40)
    run_gpu(gpu, det, [ev], 0)
    a = [oracle_lib.digest(gpu.objects(s, 0)) for s in range(5)]
    run_gpu(gpu, det, [ev], FLAG_NO_GRAPH)
    b = [oracle_lib.digest(gpu.objects(s, 0)) for s in range(5)]
    gpu.run(4, 0)
    c = [oracle_lib.digest(gpu.objects(s, 0)) for s in range(5)]
    assert a == b == c


def test_objects_into_pinned_memory(gpu, oracle_lib):
    """sdlg_get_objects into pinned host memory, 16-byte aligned and not,
    gives the rows it gives into a fresh array."""
    from sdl_gb300 import synth
    det, ev = synth.workload_event("pu", 8, pu=60)
    run_gpu(gpu, det, [ev, ev], 0)
    width = (2, 4, 8, 8, 16)
    for s in range(5):
        want = gpu.objects(s, -1)
        n = len(want)
        assert n > 0
        raw = gpu.pinned(n * width[s] * 4 + 64)
        for shift in (0, 4, 8):
            out = raw[shift:shift + n * width[s] * 4].view(np.int32).reshape(n, width[s])
            got = gpu.objects(s, -1, out=out)
            assert np.array_equal(got, want), (s, shift)
        one = gpu.objects(s, 1, out=raw[16:16 + n * width[s] * 4].view(np.int32).reshape(n, width[s]))
        assert np.array_equal(one, gpu.objects(s, 1))
    assert oracle_lib.digest(gpu.objects(4, 0)) == oracle_lib.digest(gpu.objects(4, 1))


def test_async_readback_overlaps_the_next_run(gpu, oracle_lib):
    """sdlg_get_objects_async: the tuples of one batch arrive in pinned
    memory while the next batch is set and run; a synchronous readback right
    after an asynchronous one waits for it; both batches' objects are right."""
    from sdl_gb300 import synth
    det, ev_a = synth.workload_event("pu", 9, pu=80)
    _, ev_b = synth.workload_event("pu", 10, pu=120)
    run_gpu(gpu, det, [ev_a, ev_b], 0)
    want_a = [gpu.objects(s, -1) for s in range(5)]
    width = (2, 4, 8, 8, 16)
    bufs = [gpu.pinned(len(w) * width[s] * 4 + 16)[:len(w) * width[s] * 4].view(np.int32).reshape(len(w), width[s])
            for s, w in enumerate(want_a)]
    for s in range(5):
        assert gpu.objects_async(s, -1, bufs[s]) == len(want_a[s])
    gpu.set_events([ev_b])
    gpu.run(4, 0)
    got_b = gpu.objects(4, 0)  # waits for the pending copies first
    gpu.wait_objects()
    for s in range(5):
        assert np.array_equal(bufs[s], want_a[s]), s
    ref, _, _ = oracle_lib.Oracle(det).run(ev_b)
    assert oracle_lib.digest(got_b) == oracle_lib.digest(ref[4])
    gpu.wait_objects()  # nothing pending: returns at once


def test_async_readback_before_a_run_on_the_same_buffers(gpu, oracle_lib):
    """The asynchronous readback's gathering kernel runs on the copy stream:
    a next batch of the same shape (no reallocation) set and run right after
    it must not overwrite the objects before they are gathered."""
    from sdl_gb300 import synth
    det, ev_a = synth.workload_event("pu", 11, pu=100)
    _, ev_b = synth.workload_event("pu", 12, pu=100)
    run_gpu(gpu, det, [ev_a, ev_b], 0)
    want = [gpu.objects(s, -1) for s in range(5)]
    width = (2, 4, 8, 8, 16)
    bufs = [gpu.pinned(len(w) * width[s] * 4 + 16)[:len(w) * width[s] * 4].view(np.int32).reshape(len(w), width[s])
            for s, w in enumerate(want)]
    for s in range(5):
        assert gpu.objects_async(s, -1, bufs[s]) == len(want[s])
    gpu.set_events([ev_b, ev_a])  # the same events and hits: the buffers stay
    gpu.run(4, 0)
    gpu.wait_objects()
    for s in range(5):
        assert np.array_equal(bufs[s], want[s]), s
    ref, _, _ = oracle_lib.Oracle(det).run(ev_b)
    assert oracle_lib.digest(gpu.objects(4, 0)) == oracle_lib.digest(ref[4])


def test_staged_batches(gpu, oracle_lib):
    """sdlg_stage_events: the next batch copied while the current one runs,
    taken by the next run; the current batch's results stay readable until
    then; a batch with another event count waits on the host; set_events
    drops a staged batch.  Every run's objects against the restatement."""
    from sdl_gb300 import synth
    det, e1 = synth.workload_event("pu", 21, pu=60)
    evs = [e1] + [synth.workload_event("pu", 22 + k, pu=60)[1] for k in range(4)]
    orc = oracle_lib.Oracle(det)
    want = [[oracle_lib.digest(o) for o in orc.run(e)[0]] for e in evs]

    def check(batch):
        for k, e in enumerate(batch):
            got = [oracle_lib.digest(gpu.objects(s, k)) for s in range(5)]
            assert got == want[e], (batch, k)

    gpu.upload_detector(det)
    gpu.set_events([evs[0], evs[1]])
    gpu.run_async(4, 0)
    gpu.stage_events([evs[2], evs[3]])  # overlaps the run
    gpu.sync()
    check([0, 1])  # still the current batch
    gpu.run(4, 0)
    check([2, 3])
    gpu.stage_events([evs[4], evs[0], evs[1]])  # three events: through the host
    check([2, 3])
    gpu.run(4, 0)
    check([4, 0, 1])
    gpu.stage_events([evs[3], evs[2], evs[4]])
    gpu.set_events([evs[1], evs[4], evs[0]])  # drops the staged batch
    gpu.run(4, 0)
    check([1, 4, 0])
    gpu.run(4, 0)  # nothing staged: the same batch again
    check([1, 4, 0])


def test_stop_after_stage(gpu, oracle_lib):
    from sdl_gb300 import synth
    det, ev = synth.workload_event("barrel_flat", 5)
    run_gpu(gpu, det, [ev])
    full = [gpu.objects(s, 0) for s in range(5)]
    gpu.run(1, 0)
    assert oracle_lib.digest(gpu.objects(1, 0)) == oracle_lib.digest(full[1])
    assert gpu.counts(0)[2] == 0


def test_edge_events(gpu, oracle_lib):
    """Single-hit, single-module and duplicate-free tiny events."""
    from sdl_gb300 import synth
    det, base = synth.workload_event("barrel_flat", 1)
    lower = np.array(sorted(det.lower_index), dtype=np.uint32)
    one = synth.Event(x=base.x[:1], y=base.y[:1], z=base.z[:1], idx=base.idx[:1], detid=base.detid[:1])
    m = base.detid[0]
    sel = base.detid == m
    same = synth.Event(x=base.x[sel], y=base.y[sel], z=base.z[sel], idx=base.idx[sel], detid=base.detid[sel])
    tiny = synth.Event(x=base.x[:50], y=base.y[:50], z=base.z[:50], idx=base.idx[:50], detid=base.detid[:50])
    evs = [one, same, tiny]
    run_gpu(gpu, det, evs)
    orc = oracle_lib.Oracle(det)
    for e, ev in enumerate(evs):
        ref, cnt, _ = orc.run(ev)
        for s in range(5):
            assert oracle_lib.digest(gpu.objects(s, e)) == oracle_lib.digest(ref[s])
    assert lower.size > 0


def test_unknown_module_extends_table(gpu, oracle_lib):
    """Hits in a module that no geometry table lists: the module is created
    on demand, as Event::getModule does (Event.cc:54-78)."""
    from sdl_gb300 import synth
    det, ev = synth.workload_event("barrel_flat", 2)
    # a valid barrel detId outside the synthetic layout (rod 100)
    d = (5 << 25) | (2 << 20) | (3 << 18) | (100 << 10) | (3 << 2) | 1
    extra = synth.Event(x=np.array([1.0, 1.1], np.float32), y=np.array([34.6, 35.0], np.float32),
                        z=np.array([0.5, 0.5], np.float32), idx=np.array([90000, 90001], np.int32),
                        detid=np.array([d, d + 1], np.uint32))
    cat = synth.Event(*(np.concatenate([getattr(ev, k), getattr(extra, k)]) for k in ("x", "y", "z", "idx", "detid")))
    run_gpu(gpu, det, [cat])
    ref, _, _ = oracle_lib.Oracle(det).run(cat)
    for s in range(5):
        assert oracle_lib.digest(gpu.objects(s, 0)) == oracle_lib.digest(ref[s])


@pytest.mark.parametrize("name", ["flat_s0", "flat_s0_layer", "pu20_s0_nav", "pu20_s0_tctl", "pu20_s0_tctp"])
def test_cpp_event_api_matches_golden(name, tmp_path, oracle_lib):
    """The reference's call sequence through include/sdl_event.hpp."""
    import os
    import subprocess
    from test_capi_cpu import build_cpp_demo
    meta = golden_meta(name)
    det, ev = regenerate(meta)
    exe = build_cpp_demo(tmp_path)
    paths = det.write_files(str(tmp_path))
    hb = os.path.join(str(tmp_path), "hits.bin")
    ev.write_bin(hb)
    r = subprocess.run([exe, *paths, hb, meta["mode"]], capture_output=True, text=True, check=True)
    nums = [int(v) for v in r.stdout.split("\n")[0].split()]
    assert nums[0] == len(ev)
    assert nums[1:] == meta["counts"]
