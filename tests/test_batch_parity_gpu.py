"""The plain batched chain against the CPU restatement at the full size of
the batched configurations, event by event: every event's five object
multisets (order-independent digests of the hit-index tuples), object counts
and 110 per-layer counters must be identical.

* configuration 3: 64 events of uneven size, PU drawn uniformly in 50-250;
* configuration 5: the benchmark's headline batch, 128 events of PU drawn
  uniformly in 150-300 (the same seeds and PU draws as bench.py);
* the stated density: 128 events of PU drawn uniformly in 227-474, 110k-229k
  hits per event (bench.py's stated_density batch).

Also: the pre-filtered chain's track candidates are a subset of the plain
chain's (exact multiset intersection, not a count ratio) on a batch of
PU200-like events at the shipped threshold.
"""
import multiprocessing as mp
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_events(plan):
    """Events generated in worker processes started with spawn (the test
    process may already hold a CUDA context)."""
    import bench
    procs = max(1, min(16, os.cpu_count() or 1, len(plan)))
    if procs == 1:
        return [bench._gen(a) for a in plan]
    with mp.get_context("spawn").Pool(procs) as pool:
        return pool.map(bench._gen, plan)


def config3_plan(n=64):
    import bench
    return bench.uneven_plan(0, n)


def gpu_digests(ch, n_ev):
    from sdl_gb300 import tuples
    counts = np.array([ch.counts(e) for e in range(n_ev)], dtype=np.int64)
    digests = np.zeros((n_ev, 5), dtype=np.uint64)
    for s in range(5):
        parts = tuples.split_by_event(ch.objects(s, -1), counts[:, s])
        for e, p in enumerate(parts):
            digests[e, s] = tuples.multiset_digest(p)
    counters = np.array([ch.counters(e) for e in range(n_ev)], dtype=np.uint32)
    return counts, digests, counters


def check_batch(plan, oracle_lib):
    from sdl_gb300 import Chain, synth
    events = make_events(plan)
    det = synth.detector("full")
    orc = oracle_lib.Oracle(det)
    oc, od, ok = orc.run_many_digest(events, os.cpu_count() or 1)
    ch = Chain(0)
    try:
        ch.upload_detector(det)
        ch.set_events(events)
        ch.run(4, 0)
        gc, gd, gk = gpu_digests(ch, len(events))
    finally:
        ch.close()
    bad = [(e, oracle_lib.STAGES[s], int(gc[e, s]), int(oc[e, s]))
           for e in range(len(events)) for s in range(5) if gc[e, s] != oc[e, s] or gd[e, s] != od[e, s]]
    assert not bad, "events/stages that differ (event, stage, gpu count, oracle count): %s" % bad[:10]
    bad_cnt = [e for e in range(len(events)) if not np.array_equal(gk[e], ok[e])]
    assert not bad_cnt, "per-layer counters differ on events %s" % bad_cnt[:10]
    hits = sum(len(e) for e in events)
    return len(events), hits, gc.sum(axis=0)


def test_config3_batch_matches_oracle(oracle_lib):
    n, hits, objs = check_batch(config3_plan(), oracle_lib)
    assert n == 64 and hits > 64 * 20000
    print("config 3: %d events, %d hits, objects %s identical" % (n, hits, objs.tolist()))


def test_config5_headline_batch_matches_oracle(oracle_lib):
    import bench
    n, hits, objs = check_batch(bench.headline_plan(0, 128), oracle_lib)
    assert n == 128
    print("config 5: %d events, %d hits, objects %s identical" % (n, hits, objs.tolist()))


def test_stated_density_batch_matches_oracle(oracle_lib):
    import bench
    n, hits, objs = check_batch(bench.dense_plan(0, 128), oracle_lib)
    assert n == 128 and hits > 128 * 150000
    print("stated density: %d events, %d hits, objects %s identical" % (n, hits, objs.tolist()))


def test_prefiltered_track_candidates_are_a_subset():
    """Exact multiset intersection of the pruned and plain track candidates,
    event by event, at the shipped pre-filter and threshold."""
    import bench
    from sdl_gb300 import FLAG_MLP, Chain, mlp, synth, tuples
    events = make_events([(40000 + k, 200.0) for k in range(8)])
    params, thr, _ = mlp.load(bench.MLP_WEIGHTS)
    ch = Chain(0)
    try:
        ch.upload_detector(synth.detector("full"))
        ch.mlp_set_params(params, thr)
        ch.set_events(events)
        ch.run(4, 0)
        plain = [ch.objects(4, e) for e in range(len(events))]
        ch.run(4, FLAG_MLP)
        pruned = [ch.objects(4, e) for e in range(len(events))]
    finally:
        ch.close()
    inter = sum(tuples.multiset_intersection(p, q) for p, q in zip(pruned, plain))
    n_pruned = sum(len(p) for p in pruned)
    n_plain = sum(len(q) for q in plain)
    assert inter == n_pruned, "pruned track candidates outside the plain chain's: %d" % (n_pruned - inter)
    assert n_plain > 0 and inter / n_plain >= 0.99
