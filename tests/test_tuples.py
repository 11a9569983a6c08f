"""Object-list digests: the numpy digest (sdl_gb300/tuples.py) used for the
GPU chain's objects equals the CPU restatement's own per-event digest, is
independent of row order, and the multiset intersection counts repeats."""
import numpy as np

from sdl_gb300 import tuples


def test_digest_matches_oracle_per_event(oracle_lib):
    from sdl_gb300 import synth
    det = synth.detector("full")
    events = [synth.make_event(det, 77, "full", n_pu=200), synth.make_event(det, 78, "full", n_pu=0, n_signal=0,
                                                                             noise_frac=0.0),
              synth.make_event(det, 79, "full", n_pu=400)]
    orc = oracle_lib.Oracle(det)
    counts, digests, counters = orc.run_many_digest(events, 2)
    for e, ev in enumerate(events):
        out, cnt, _ = orc.run(ev)
        assert [len(o) for o in out] == counts[e].tolist()
        assert [tuples.multiset_digest(o) for o in out] == [int(v) for v in digests[e]]
        assert np.array_equal(cnt, counters[e])
    assert counts[0, 4] > 0 and counts[1].sum() == 0


def test_digest_is_order_independent_and_multiset_aware():
    rng = np.random.default_rng(5)
    t = rng.integers(-5, 1 << 20, size=(1000, 8)).astype(np.int32)
    assert tuples.multiset_digest(t) == tuples.multiset_digest(t[rng.permutation(len(t))])
    assert tuples.multiset_digest(np.concatenate([t, t[:1]])) != tuples.multiset_digest(t)
    u = t.copy()
    u[3, 7] ^= 1
    assert tuples.multiset_digest(u) != tuples.multiset_digest(t)
    assert tuples.multiset_digest(t[:, ::-1]) != tuples.multiset_digest(t)


def test_multiset_intersection():
    a = np.array([[1, 2], [1, 2], [3, 4], [5, 6]], dtype=np.int32)
    b = np.array([[1, 2], [3, 4], [3, 4], [7, 8]], dtype=np.int32)
    assert tuples.multiset_intersection(a, b) == 2
    assert tuples.multiset_intersection(a, a) == 4
    assert tuples.multiset_intersection(a, b[:0]) == 0
    parts = tuples.split_by_event(a, np.array([1, 0, 3]))
    assert [len(p) for p in parts] == [1, 0, 3]
