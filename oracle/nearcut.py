"""Near-cut report -- TEST INFRASTRUCTURE ONLY.

The reference's float std::asin/atan/sin/cos/tan are the host libm's float
functions, which are not correctly rounded; this report lists, for a set of
events, every object whose existence depends on that: the CPU restatement
runs each event with the reference's libm and with correctly rounded floats
(``Oracle.audit``), and each object only one of the two runs makes is listed
with the cut that rejects it in the other run and that cut's distance to its
bound in both runs (in float steps of the bound).  The GPU chain reproduces
the host libm (``sdlg_libm_eval``), so these are the decisions on which a
correctly rounded evaluation would disagree with the reference.

    python -m oracle.nearcut --batch headline|config3 [--events N] [--threads T] [--out report.json]

The committed reports, tests/golden/nearcut/headline.json and config3.json, were made with
--threads 8 and --out set to those paths.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

STAGES = ("MD", "SG", "TL", "TP", "TC")
WIDTH = (2, 4, 8, 8, 16)


def ordered(f: float) -> int:
    """float32 -> an integer whose order is the floats' order (adjacent floats differ by 1)"""
    u = int(np.float32(f).view(np.uint32))
    return u if u < 0x80000000 else 0x80000000 - u


def steps(value: float, lo: float, hi: float) -> int:
    """signed distance of value to the nearer finite bound of [lo, hi] in
    float steps: > 0 inside, <= 0 outside"""
    cands = []
    if np.isfinite(lo):
        cands.append(ordered(value) - ordered(lo))
    if np.isfinite(hi):
        cands.append(ordered(hi) - ordered(value))
    return int(min(cands)) if cands else 0


def describe(rec) -> dict:
    s = int(rec["stage"])
    d = {"stage": STAGES[s], "tuple": [int(v) for v in rec["tuple"][:WIDTH[s]]],
         "made_with": "glibc" if rec["accept_glibc"] else "correctly rounded",
         "algorithm": rec["where"].decode(), "cut": rec["cut"].decode()}
    for tag, k in (("glibc", "g"), ("rounded", "r")):
        v, lo, hi = float(rec[k + "_value"]), float(rec[k + "_lo"]), float(rec[k + "_hi"])
        d[tag] = {"value": v, "lo": lo if np.isfinite(lo) else None, "hi": hi if np.isfinite(hi) else None,
                  "steps_inside": steps(v, lo, hi)}
    return d


def audit_events(events, threads: int, mode: int = 0):
    import oracle
    from sdl_gb300 import synth
    orc = oracle.Oracle(synth.detector("full"))
    with ThreadPoolExecutor(max(1, threads)) as ex:
        return list(ex.map(lambda ev: orc.audit(ev, mode), events))


def report(plan, threads: int, label: str) -> dict:
    import bench
    events = [bench._gen(a) for a in plan]
    res = audit_events(events, threads)
    out = {"batch": label, "events": len(events), "hits": int(sum(len(e) for e in events)),
           "per_stage": {}, "flips": []}
    tot = np.zeros((5, 4), dtype=np.int64)
    for k, (recs, summ) in enumerate(res):
        tot += summ
        for r in recs:
            d = describe(r)
            d["event"] = k
            d["seed"], d["pu"] = int(plan[k][0]), float(plan[k][1])
            out["flips"].append(d)
    for s in range(5):
        out["per_stage"][STAGES[s]] = {"objects_glibc": int(tot[s, 0]), "objects_rounded": int(tot[s, 1]),
                                       "primary_flips": int(tot[s, 2]), "secondary_flips": int(tot[s, 3])}
    return out


def main():
    import bench
    ap = argparse.ArgumentParser()
    ap.add_argument("--batch", choices=("headline", "config3"), default="headline")
    ap.add_argument("--events", type=int, default=0)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    if a.batch == "headline":
        plan = bench.headline_plan(0, 128)
        label = "128 events, PU uniform in 150-300 (the benchmark's headline batch)"
    else:
        rng = np.random.default_rng(3303)
        plan = [(30000 + k, float(p)) for k, p in enumerate(rng.uniform(50.0, 250.0, size=64))]
        label = "64 events, PU uniform in 50-250"
    if a.events:
        plan = plan[:a.events]
    out = report(plan, a.threads, label)
    text = json.dumps(out, indent=1)
    if a.out:
        with open(a.out, "w") as f:
            f.write(text + "\n")
    print(json.dumps(out["per_stage"], indent=1))
    for d in out["flips"]:
        print("event %d %s %s made with %s only; %s: %s (%d / %d float steps inside with glibc / rounded)" % (
            d["event"], d["stage"], d["tuple"], d["made_with"], d["algorithm"], d["cut"],
            d["glibc"]["steps_inside"], d["rounded"]["steps_inside"]))


if __name__ == "__main__":
    main()
