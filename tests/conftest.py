import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def golden_meta(name):
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        return json.load(f)


def golden_tuples(name):
    path = os.path.join(GOLDEN, name + ".npz")
    if not os.path.exists(path):
        return None
    z = np.load(path)
    return [z[s] for s in ("MD", "SG", "TL", "TP", "TC")]


def golden_names():
    return sorted(f[:-5] for f in os.listdir(GOLDEN) if f.endswith(".json"))


def regenerate(meta):
    """The fixture's event and geometry, regenerated and fingerprint-checked."""
    from sdl_gb300 import synth
    det, ev = synth.workload_event(meta["workload"], meta["seed"], pu=meta["pu"] or 200.0)
    assert det.fingerprint() == meta["geometry_fingerprint"], "geometry generator changed"
    assert ev.fingerprint() == meta["event_fingerprint"], "event generator changed"
    return det, ev


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle
