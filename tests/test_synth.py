"""Synthetic detector: detId layout, inversion/partner rules and the text
formats the reference's loaders read."""
import os

import numpy as np

from sdl_gb300 import synth


def decode(d):
    # Module.cc:159-358 restated for the checks here
    sub = (d >> 25) & 7
    ec = sub == 4
    side = (d >> 23) & 3 if ec else (d >> 18) & 3
    layer = (d >> 18) & 7 if ec else (d >> 20) & 7
    module = (d >> 2) & 127
    if ec:
        inv = (module % 2 == 1) if side == 1 else (module % 2 == 0)
    elif side == 3:
        inv = (module % 2 == 1) if layer <= 3 else (module % 2 == 0)
    else:
        inv = (module % 2 == 1) if layer <= 2 else (module % 2 == 0)
    lower = (not (d & 1)) if inv else bool(d & 1)
    return sub, side, layer, module, inv, lower


def test_inner_sensor_is_reference_lower():
    for kind in ("barrel_flat", "full"):
        det = synth.detector(kind)
        for d, inner in zip(det.detid[::7], det.is_inner[::7]):
            assert decode(int(d))[5] == bool(inner)


def test_partner_pairs_exist():
    det = synth.detector("full")
    ids = set(int(d) for d in det.detid)
    for d in list(det.lower_index)[::11]:
        inv = decode(d)[4]
        assert (d - 1 if inv else d + 1) in ids


def test_map_connects_next_layer_only():
    det = synth.detector("full")
    for k, v in list(det.conn.items())[::37]:
        sk, _, lk, _, _, _ = decode(k)
        for d in v:
            sd, _, ld, _, _, lower = decode(d)
            assert lower
            if sk == 5 and sd == 5:
                assert ld == lk + 1
            if sk == 4:
                assert sd == 4 and ld == lk + 1


def test_text_files_roundtrip(tmp_path):
    det = synth.detector("full")
    t, e, m = det.write_files(str(tmp_path))
    t_id, t_val, e_id, e_val, keys, off, dst = det.tables()
    rows = np.loadtxt(t, dtype=np.float64)
    assert rows.shape[0] == len(t_id)
    np.testing.assert_array_equal(rows[:, 1:].astype(np.float32), t_val)
    with open(m) as f:
        first = f.readline().split()
    assert int(first[0]) == keys[0] and int(first[1]) == off[1] - off[0]


def test_event_is_deterministic():
    _, a = synth.workload_event("barrel_flat", 3)
    _, b = synth.workload_event("barrel_flat", 3)
    assert a.fingerprint() == b.fingerprint()
    assert len(np.unique(a.idx)) == len(a)
