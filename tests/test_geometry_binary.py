"""Binary geometry files (sdlg_geometry_convert / sdlg_geometry_load_binary):
the file holds exactly the tables the text files give, and the chain run on a
binary geometry gives the same objects as on the text files."""
import struct

import numpy as np
import pytest


def _read_binary(path):
    with open(path, "rb") as f:
        data = f.read()
    assert data[:8] == b"SDLGEO1\0"
    pos = 8
    tables = []
    for _ in range(2):
        (n,) = struct.unpack_from("<Q", data, pos)
        pos += 8
        rows = {}
        for _ in range(n):
            d, a, c = struct.unpack_from("<Iff", data, pos)
            pos += 12
            rows[d] = (a, c)
        tables.append(rows)
    (nk,) = struct.unpack_from("<Q", data, pos)
    pos += 8
    keys = [struct.unpack_from("<II", data, pos + 8 * k) for k in range(nk)]
    pos += 8 * nk
    conn = {}
    for d, n in keys:
        conn[d] = list(struct.unpack_from("<%dI" % n, data, pos))
        pos += 4 * n
    assert pos == len(data)
    return tables[0], tables[1], conn


def test_convert_matches_text_tables(tmp_path):
    from sdl_gb300 import geometry_convert, synth
    det = synth.detector("full")
    paths = det.write_files(str(tmp_path))
    out = str(tmp_path / "geo.bin")
    geometry_convert(*paths, out)
    tilted, endcap, conn = _read_binary(out)
    assert sorted(tilted) == sorted({int(r[0]) for r in det.tilted_rows})
    for r in det.tilted_rows:
        assert tilted[int(r[0])] == (np.float32(r[1]), np.float32(r[2]))
    for r in det.endcap_rows:  # slope lower (column 3) and the 7th column
        assert endcap[int(r[0])] == (np.float32(r[3]), np.float32(r[6]))
    t_id, t_val, e_id, e_val, keys, off, dst = det.tables()
    assert sorted(conn) == sorted(int(k) for k in keys)
    for k, key in enumerate(keys):
        assert conn[int(key)] == [int(v) for v in dst[off[k]:off[k + 1]]]


def test_convert_reports_missing_file(tmp_path):
    from sdl_gb300 import SDLError, geometry_convert
    with pytest.raises(SDLError):
        geometry_convert(str(tmp_path / "absent.txt"), None, None, str(tmp_path / "geo.bin"))


@pytest.mark.gpu
def test_binary_geometry_runs_the_same_chain(tmp_path, oracle_lib):
    from sdl_gb300 import Chain, build, geometry_convert, synth
    build.build()
    det, ev = synth.workload_event("pu", 3, pu=40)
    paths = det.write_files(str(tmp_path))
    out = str(tmp_path / "geo.bin")
    geometry_convert(*paths, out)
    a, b = Chain(0), Chain(0)
    a.load_files(*paths)
    b.load_binary(out)
    for ch in (a, b):
        ch.set_events([ev])
        ch.run(4, 0)
    for s in range(5):
        assert oracle_lib.digest(a.objects(s, 0)) == oracle_lib.digest(b.objects(s, 0))
    assert np.array_equal(a.counters(0), b.counters(0))
