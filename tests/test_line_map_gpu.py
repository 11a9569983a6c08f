"""The straight-line module connection map built on the GPU
(sdlg_build_line_map) against the synthetic detector's own map
(sdl_gb300/synth.py, numpy): identical for the barrel-only and the full
detector, and the chain on it gives the same objects as on the host map."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["barrel_flat", "full"])
def test_gpu_line_map_equals_host_map(kind):
    from sdl_gb300 import line_map, synth
    det = synth.detector(kind)
    gmap = line_map(det)
    assert gmap.keys() == det.conn.keys()
    diff = [k for k in det.conn if det.conn[k] != gmap[k]]
    assert not diff, "%d keys differ, first %d: %s vs %s" % (len(diff), diff[0], gmap[diff[0]], det.conn[diff[0]])
    assert sum(len(v) for v in gmap.values()) > 10 * len(gmap)


def test_chain_on_gpu_map(oracle_lib):
    import numpy as np
    from sdl_gb300 import Chain, line_map, synth
    det, ev = synth.workload_event("pu", 3, pu=40)
    gmap = line_map(det)
    t_id, t_val, e_id, e_val, _, _, _ = det.tables()
    keys = np.array(sorted(gmap), dtype=np.uint32)
    off = np.zeros(len(keys) + 1, dtype=np.int64)
    off[1:] = np.cumsum([len(gmap[int(k)]) for k in keys])
    dst = np.array([d for k in keys for d in gmap[int(k)]], dtype=np.uint32)
    ch = Chain(0)
    try:
        ch.upload_tables(t_id, t_val, e_id, e_val, keys, off, dst)
        ch.set_events([ev])
        ch.run(4, 0)
        ref, _, _ = oracle_lib.Oracle(det).run(ev)
        for s in range(5):
            assert oracle_lib.digest(ch.objects(s, 0)) == oracle_lib.digest(ref[s])
    finally:
        ch.close()
