"""The reference's object graph through include/sdl_event.hpp: a C++ program
(tests/cpp_object_api.cc) walks Event::getLowerModulePtrs() ->
Module::getMiniDoubletPtrs()/getSegmentPtrs()/getTripletPtrs() -> the
objects' pointer accessors (innerMiniDoubletPtr()->lowerHitPtr()->idx(), ...)
and Event::getLayerPtrs() -> Layer::getTrackletPtrs()/getTrackCandidatePtrs(),
as a caller of the reference does.  The tuples it collects must be the
reference's objects (golden fixtures), the mini-doublets' and segments' kept
floats (getDz, getDeltaPhi, ..., getDeltaPhiMaxChange) the CPU restatement's,
bit for bit, the hits-by-layer counts those of the hits' modules, and the
five create* calls must cost about one chain run (each runs only its
stage)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden_meta, golden_tuples, regenerate

pytestmark = pytest.mark.gpu

W = (2, 4, 8, 8, 16)
NV = (4, 6, 0, 0, 0)


def build_walker(tmpdir):
    from sdl_gb300 import build
    lib = build.build()
    exe = os.path.join(str(tmpdir), "cpp_object_api")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp_object_api.cc"), "-o", exe, lib,
                    "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    return exe


def read_walk(path):
    data = open(path, "rb").read()
    pos = 0
    tup, vals = [], []
    for s in range(5):
        n = int(np.frombuffer(data, np.int64, 1, pos)[0])
        pos += 8
        rec = np.frombuffer(data, np.uint32, n * (W[s] + NV[s]), pos).reshape(n, W[s] + NV[s])
        pos += rec.nbytes
        tup.append(rec[:, :W[s]].view(np.int32).copy())
        vals.append(rec[:, W[s]:].view(np.float32).copy())
    hl = np.frombuffer(data, np.uint32, 24, pos).reshape(4, 6)
    pos += 96
    cnt = np.frombuffer(data, np.uint32, 6, pos)
    pos += 24
    times = np.frombuffer(data, np.float64, 2, pos)
    return tup, vals, hl, cnt, times


def rows(t, v):
    """(tuple, float bits) rows in canonical order"""
    import oracle
    a = np.concatenate([t.view(np.int32), v.view(np.int32)], axis=1)
    return oracle.canon(a)


@pytest.mark.parametrize("name,mode", [("flat_s0", "map"), ("pu20_s0_layer", "layer"), ("pu20_s0_tctl", "tctl"),
                                       ("pu20_s0_tctp", "tctp"), ("pu200_s0", "map")])
def test_object_graph_walk_matches_reference(name, mode, tmp_path, oracle_lib):
    meta = golden_meta(name)
    det, ev = regenerate(meta)
    exe = build_walker(tmp_path)
    paths = det.write_files(str(tmp_path))
    hb = os.path.join(str(tmp_path), "hits.bin")
    ev.write_bin(hb)
    out = os.path.join(str(tmp_path), "walk.bin")
    r = subprocess.run([exe, *paths, hb, out, mode], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    tup, vals, hl, cnt, times = read_walk(out)
    assert cnt[5] == 0, "object-graph inconsistencies"
    assert [int(c) for c in cnt[:5]] == meta["counts"]
    full = golden_tuples(name)
    for s in range(5):
        assert oracle_lib.digest(tup[s]) == meta["digests"][s], "%s from the walk" % oracle_lib.STAGES[s]
        if full is not None:
            assert np.array_equal(oracle_lib.canon(tup[s]), full[s])
    # kept floats of mini-doublets and segments, bit for bit
    flags = {"map": 0, "layer": 3, "tctl": 64, "tctp": 128}[mode]
    ref, _, _, rv = oracle_lib.Oracle(det).run(ev, mode=flags, vals=True)
    for s in (0, 1):
        assert np.array_equal(rows(tup[s], vals[s]), rows(ref[s], rv[s])), "%s floats" % oracle_lib.STAGES[s]
    # hits by layer, lower and upper modules (Event.cc:1170-1190)
    from sdl_gb300 import module_info
    exp = np.zeros((4, 6), np.uint32)
    for d, c in zip(*np.unique(ev.detid, return_counts=True)):
        m = module_info(int(d))
        exp[(0 if m["isLower"] else 2) + (0 if m["subdet"] == 5 else 1), m["layer"] - 1] += c
    assert np.array_equal(hl, exp)
    # the five create* calls against one run of the whole chain (PU200)
    if name.startswith("pu200"):
        print("create* %.3f ms, one chain run %.3f ms" % tuple(times))
        assert times[0] < 2.0 * times[1] + 2.0, times


def test_run_stages_continues_the_last_run(oracle_lib):
    """Stage by stage through sdlg_run_stages gives the objects and counters
    of one run, for the module-map chain and the variants."""
    from sdl_gb300 import Chain, synth
    det, ev = synth.workload_event("pu", 11, pu=60)
    ch = Chain(0)
    try:
        ch.upload_detector(det)
        ch.set_events([ev, ev])
        for flags in (0, 3, 32, 64, 128):
            ch.run(4, flags)
            whole = [oracle_lib.digest(ch.objects(s, -1)) for s in range(5)]
            cnt = [ch.counters(e).copy() for e in range(2)]
            ch.run_stages(0, 0, flags)
            for st in range(1, 5):
                ch.run_stages(st, st, flags)
            assert [oracle_lib.digest(ch.objects(s, -1)) for s in range(5)] == whole, flags
            assert all(np.array_equal(ch.counters(e), cnt[e]) for e in range(2))
    finally:
        ch.close()
