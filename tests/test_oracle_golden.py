"""The CPU restatement (oracle/) against the golden fixtures produced by the
unmodified reference chain (tests/golden/make_golden.py)."""
import numpy as np
import pytest

from conftest import golden_meta, golden_names, golden_tuples, regenerate

# fixture mode -> oracle mode bits (the chain's flag bits)
MODE = {"map": 0, "layer": 3, "nav": 32, "tctl": 64, "tctp": 128}


@pytest.mark.parametrize("name", golden_names())
def test_oracle_matches_reference(name, oracle_lib):
    meta = golden_meta(name)
    det, ev = regenerate(meta)
    out, cnt, _ = oracle_lib.Oracle(det).run(ev, mode=MODE[meta["mode"]])
    assert [int(a.shape[0]) for a in out] == meta["counts"]
    assert [oracle_lib.digest(a) for a in out] == meta["digests"]
    assert [int(v) for v in cnt] == meta["counters"]
    full = golden_tuples(name)
    if full is not None:
        for s in range(5):
            np.testing.assert_array_equal(oracle_lib.canon(out[s]), full[s])


def test_golden_fixtures_present():
    names = golden_names()
    assert any(n.startswith("flat_") for n in names)
    assert any(n.startswith("pu200_") for n in names)
