"""Failure paths of the chain, made on the host or by a flag; none of them
faults, traps or hangs the GPU:

* object capacities forced to 1: every stage overflows, the host grows the
  buffers and repeats the run, and the objects are those of a run with the
  default capacities;
* a hit whose detId decodes to no barrel or endcap module: SDLG_ERR_DETID,
  and the context still runs good events;
* a truncated binary geometry file: SDLG_ERR_IO; a missing text file:
  SDLG_ERR_IO; a text map file cut in the middle of a line is read as the
  reference's stream parsing reads it (ModuleConnectionMap.cc:28-45);
* the pre-filter's bounded tensor-core wait made to give up at once
  (SDLG_FLAG_TEST_MLP_GIVE_UP): the run fails with SDLG_ERR_CUDA, the
  counters show the waits that gave up, and the next run on the same
  context gives the right objects.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def digests(ch, oracle_lib, n_ev):
    return [[oracle_lib.digest(ch.objects(s, e)) for s in range(5)] for e in range(n_ev)]


@pytest.fixture(scope="module")
def events():
    from sdl_gb300 import synth
    det = synth.detector("full")
    return det, [synth.make_event(det, 960, "full", n_pu=700), synth.make_event(det, 961, "full", n_pu=1400)]


def test_capacities_of_one_grow_to_the_same_objects(events, oracle_lib):
    from sdl_gb300 import FLAG_MLP, Chain, mlp
    import bench
    det, evs = events
    params, thr, _ = mlp.load(bench.MLP_WEIGHTS)
    ref = Chain(0)
    ref.upload_detector(det)
    ref.mlp_set_params(params, thr)
    ref.set_events(evs)
    want = {}
    for fl in (0, FLAG_MLP):
        ref.run(4, fl)
        want[fl] = (digests(ref, oracle_lib, 2), [ref.counters(e).copy() for e in range(2)])
    default_caps = ref.capacities()
    ref.close()
    ch = Chain(0)
    try:
        ch.upload_detector(det)
        ch.mlp_set_params(params, thr)
        ch.set_capacities([1] * 6)
        assert list(ch.capacities()) == [1] * 6
        ch.set_events(evs)
        for fl in (0, FLAG_MLP):
            ch.run(4, fl)
            assert digests(ch, oracle_lib, 2) == want[fl][0]
            assert all(np.array_equal(ch.counters(e), want[fl][1][e]) for e in range(2))
        caps = ch.capacities()
        counts = ch.counts(-1)
        assert all(caps[s] >= counts[s] > 1 for s in range(5)), (caps, counts)
        assert all(caps[s] < default_caps[s] for s in range(5)), (caps, default_caps)
    finally:
        ch.close()


def test_bad_detid_is_rejected(events, oracle_lib):
    from sdl_gb300 import Chain, SDLError, synth
    det, evs = events
    ev = evs[0]
    bad = synth.Event(x=np.append(ev.x, np.float32(30.0)), y=np.append(ev.y, np.float32(1.0)),
                      z=np.append(ev.z, np.float32(2.0)), idx=np.append(ev.idx, np.int32(len(ev))),
                      detid=np.append(ev.detid, np.uint32(0x0123457)))  # subdet 0
    ch = Chain(0)
    try:
        ch.upload_detector(det)
        ch.set_events([bad])
        with pytest.raises(SDLError) as e:
            ch.run(4, 0)
        assert str(e.value).startswith("-6:") and "not a barrel or endcap module" in str(e.value)
        ch.set_events([ev])
        ch.run(4, 0)
        ref, _, _ = oracle_lib.Oracle(det).run(ev)
        assert [oracle_lib.digest(ch.objects(s, 0)) for s in range(5)] == [oracle_lib.digest(r) for r in ref]
    finally:
        ch.close()


def test_truncated_geometry_files(events, tmp_path, oracle_lib):
    from sdl_gb300 import Chain, SDLError, geometry_convert
    det, evs = events
    paths = det.write_files(str(tmp_path))
    binp = os.path.join(str(tmp_path), "geo.bin")
    geometry_convert(*paths, binp)
    blob = open(binp, "rb").read()
    ch = Chain(0)
    try:
        for cut in (0, 7, 8, 12, 20, len(blob) // 2, len(blob) - 3):
            p = os.path.join(str(tmp_path), "cut%d.bin" % cut)
            with open(p, "wb") as f:
                f.write(blob[:cut])
            with pytest.raises(SDLError) as e:
                ch.load_binary(p)
            assert str(e.value).startswith("-5:")
        with pytest.raises(SDLError) as e:
            ch.load_files(paths[0], paths[1], os.path.join(str(tmp_path), "missing.txt"))
        assert str(e.value).startswith("-5:")
        # the whole file loads and runs
        ch.load_binary(binp)
        ch.set_events([evs[0]])
        ch.run(4, 0)
        ref, _, _ = oracle_lib.Oracle(det).run(evs[0])
        assert oracle_lib.digest(ch.objects(4, 0)) == oracle_lib.digest(ref[4])
        # a map file cut inside its last line: the stream parse reads the
        # missing connections of that key as detId 0 (no module), as the
        # reference's does; the same tables given as arrays give the same
        # module table and objects
        lines = open(paths[2]).read().splitlines()
        cutp = os.path.join(str(tmp_path), "map_cut.txt")
        with open(cutp, "w") as f:
            f.write("\n".join(lines[:-1] + [" ".join(lines[-1].split()[:3])]))
        t_id, t_val, e_id, e_val, keys, off, dst = det.tables()
        dst2 = dst.copy()
        dst2[off[-2] + 1:] = 0
        ch.upload_tables(t_id, t_val, e_id, e_val, keys, off, dst2)
        n_ref = ch.num_modules
        ch.set_events([evs[0]])
        ch.run(4, 0)
        want = [oracle_lib.digest(ch.objects(s, 0)) for s in range(5)]
        ch.load_files(paths[0], paths[1], cutp)
        assert ch.num_modules == n_ref
        ch.set_events([evs[0]])
        ch.run(4, 0)
        assert [oracle_lib.digest(ch.objects(s, 0)) for s in range(5)] == want
    finally:
        ch.close()


def test_prefilter_wait_give_up_is_reported(events, oracle_lib):
    import bench
    from sdl_gb300 import FLAG_MLP, FLAG_TEST_MLP_GIVE_UP, Chain, SDLError, mlp
    det, evs = events
    params, thr, _ = mlp.load(bench.MLP_WEIGHTS)
    ch = Chain(0)
    try:
        ch.upload_detector(det)
        ch.mlp_set_params(params, thr)
        ch.set_events(evs)
        ch.run(4, FLAG_MLP)
        want = digests(ch, oracle_lib, 2)
        assert ch.mlp_stats()["timeouts"] == 0
        with pytest.raises(SDLError) as e:
            ch.run(4, FLAG_MLP | FLAG_TEST_MLP_GIVE_UP)
        assert str(e.value).startswith("-2:") and "gave up" in str(e.value)
        assert ch.mlp_stats()["timeouts"] > 0
        ch.run(4, FLAG_MLP)
        assert ch.mlp_stats()["timeouts"] == 0
        assert digests(ch, oracle_lib, 2) == want
    finally:
        ch.close()
