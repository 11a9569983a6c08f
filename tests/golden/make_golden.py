"""Generates the golden fixtures in this directory by running the UNMODIFIED
reference chain (oracle/_ref/ref_driver, built from the reference sources with
`make -C oracle ref`) on seeded synthetic events.

    python tests/golden/make_golden.py --refdir <reference sources> [--jobs 8]

Each fixture records the event and geometry fingerprints (so a consumer can
confirm it regenerated the same inputs), the per-stage object multisets as
canonical hit-index tuples (or their SHA-256 digests for the large events),
object counts and the reference's per-layer counters.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
from concurrent.futures import ProcessPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from sdl_gb300 import synth  # noqa: E402

# (name, workload, seed, pu, mode, store full tuples)
CASES = [
    *[("flat_s%d" % s, "barrel_flat", s, None, "map", True) for s in range(8)],
    ("flat_s0_layer", "barrel_flat", 0, None, "layer", True),
    ("pu20_s0", "pu", 0, 20, "map", True),
    ("pu20_s0_layer", "pu", 0, 20, "layer", True),
    ("pu50_s1", "pu", 1, 50, "map", False),
    ("pu200_s0", "pu", 0, 200, "map", False),
    ("pu200_s1", "pu", 1, 200, "map", False),
    # createTrackletsViaNavigation, createTrackCandidatesFromTracklets / FromTriplets
    *[("flat_s0_" + m, "barrel_flat", 0, None, m, True) for m in ("nav", "tctl", "tctp")],
    *[("pu20_s0_" + m, "pu", 0, 20, m, True) for m in ("nav", "tctl", "tctp")],
    *[("pu50_s1_" + m, "pu", 1, 50, m, False) for m in ("nav", "tctl", "tctp")],
]


def one(case):
    name, wl, seed, pu, mode, full = case
    det, ev = synth.workload_event(wl, seed, pu=pu or 200.0)
    out, cnt, sec, tlv = oracle.run_reference(det, ev, mode=mode, tl_vars=True)
    meta = {
        "name": name, "workload": wl, "seed": seed, "pu": pu, "mode": mode,
        "n_hits": len(ev), "event_fingerprint": ev.fingerprint(), "geometry_fingerprint": det.fingerprint(),
        "counts": [int(a.shape[0]) for a in out], "digests": [oracle.digest(a) for a in out],
        "counters": [int(v) for v in cnt], "reference_seconds": [float(s) for s in sec],
    }
    if full:
        # the tracklets' final recovars, rows in the canonical tracklet order
        np.savez_compressed(os.path.join(HERE, name + ".npz"),
                            **{oracle.STAGES[s]: oracle.canon(out[s]) for s in range(5)},
                            tl_vars=tlv[oracle.canon_order(out[2])])
    with open(os.path.join(HERE, name + ".json"), "w") as f:
        json.dump(meta, f, indent=1)
    return name, meta["counts"], sum(sec)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=os.cpu_count())
    ap.add_argument("--only", default=None)
    ap.add_argument("--refdir", default=os.environ.get("SDL_REFDIR"),
                    help="the reference's source directory (default: $SDL_REFDIR)")
    a = ap.parse_args()
    if not a.refdir:
        raise SystemExit("give the reference's source directory: --refdir DIR or SDL_REFDIR")
    oracle.build(ref_dir=a.refdir)
    cases = [c for c in CASES if a.only is None or c[0] == a.only]
    with ProcessPoolExecutor(a.jobs) as ex:
        for name, counts, secs in ex.map(one, cases):
            print("%-16s %s  reference %.1fs" % (name, counts, secs), flush=True)


if __name__ == "__main__":
    main()
