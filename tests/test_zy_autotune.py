"""The autotuner changes launch shapes only: the objects after tuning are
the ones before it (and the reference's)."""
import pytest

pytestmark = pytest.mark.gpu


def test_autotune_keeps_results():
    import oracle
    from sdl_gb300 import Chain, build, synth
    build.build()
    det = synth.detector("full")
    events = [synth.make_event(det, 970 + k, "full", n_pu=700 * (k + 1)) for k in range(3)]
    ch = Chain(0)
    ch.upload_detector(det)
    ch.set_events(events)
    ch.run(4, 0)
    before = [[oracle.digest(ch.objects(s, e)) for s in range(5)] for e in range(3)]
    shape = ch.autotune(4, 0)
    assert all(t in (128, 256, 512, 1024) for t in shape["task"])
    assert all(g in (4, 8, 16) for g in shape["ctas_per_sm"])
    ch.run(4, 0)
    after = [[oracle.digest(ch.objects(s, e)) for s in range(5)] for e in range(3)]
    assert after == before
    ch.close()
