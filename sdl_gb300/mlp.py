"""Training, calibration and evaluation of the learned tracklet pre-filter
(no counterpart in the reference), on top of :class:`sdl_gb300.Chain`.

The pre-filter is a 12-64-64-1 perceptron that scores each tracklet
candidate before the reference's tracklet cuts; candidates below a logit
threshold are dropped, all others are judged by the exact cuts.  Training
data are the plain chain's own candidates and accept/reject decisions
(``Chain.mlp_collect``); training runs on the GPU with the library's kernels
(``Chain.mlp_train``).  The threshold is chosen on held-out events as the
largest one whose track-candidate recall against the plain chain meets a
target: the pruned chain's track candidates are a subset of the plain
chain's, and shrink monotonically as the threshold rises, so recall is
count(pruned) / count(plain) and a bisection finds the threshold.

Run as a script to train the shipped parameter files::

    python -m sdl_gb300.mlp flat [out_dir]   # 500 barrel-only events -> tl_mlp_flat.npz
    python -m sdl_gb300.mlp pu [out_dir]     # PU 100-300 full-geometry events -> tl_mlp_pu.npz

(out_dir defaults to sdl_gb300/weights/, where the shipped files live).
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

from . import FLAG_MLP, Chain, synth

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "weights")


def chunks(seq, n):
    for k in range(0, len(seq), n):
        yield seq[k:k + n]


def collect(chain: Chain, det, events, neg_keep: float, seed: int, per_run: int = 16, flags: int = 0) -> int:
    """Run the plain chain through the tracklet step on `events` and append
    their candidates (features, accept/reject) to the training set."""
    chain.upload_detector(det)
    n = chain.mlp_num_samples()
    for k, part in enumerate(chunks(events, per_run)):
        chain.set_events(part)
        chain.run(2, flags)
        n = chain.mlp_collect(neg_keep, seed + k)
    return n


def plain_counts(chain: Chain, det, events, per_run: int = 16, flags: int = 0):
    """(tracklets, track candidates) of the plain chain, summed over events"""
    chain.upload_detector(det)
    tl = tc = 0
    for part in chunks(events, per_run):
        chain.set_events(part)
        chain.run(4, flags)
        c = chain.counts(-1)
        tl += int(c[2])
        tc += int(c[4])
    return tl, tc


def pruned_counts(chain: Chain, det, events, thr: float, per_run: int = 16, flags: int = 0):
    """(tracklets, track candidates, stats) of the chain with the pre-filter
    at threshold `thr`, summed over events"""
    chain.upload_detector(det)
    chain.mlp_set_threshold(thr)
    tl = tc = 0
    st = {"candidates": 0, "scored": 0, "kept": 0, "timeouts": 0}
    for part in chunks(events, per_run):
        chain.set_events(part)
        chain.run(4, flags | FLAG_MLP)
        c = chain.counts(-1)
        tl += int(c[2])
        tc += int(c[4])
        for k, v in chain.mlp_stats().items():
            st[k] += v
    return tl, tc, st


def calibrate(chain: Chain, det, events, target: float, per_run: int = 16, iters: int = 22, flags: int = 0):
    """Largest logit threshold whose track-candidate recall on `events`
    reaches `target`; returns (threshold, recall, tracklet recall, stats)."""
    _, tc0 = plain_counts(chain, det, events, per_run, flags)
    lo, hi = -30.0, 30.0
    best = None
    for _ in range(iters):
        mid = 0.5 * (lo + hi)
        tl, tc, st = pruned_counts(chain, det, events, mid, per_run, flags)
        rec = tc / tc0 if tc0 else 1.0
        if rec >= target:
            lo = mid
            best = (mid, rec, tl, st)
        else:
            hi = mid
    if best is None:
        tl, tc, st = pruned_counts(chain, det, events, lo, per_run, flags)
        best = (lo, tc / tc0 if tc0 else 1.0, tl, st)
    tl0, _ = plain_counts(chain, det, events, per_run, flags)
    thr, rec, tl, st = best
    chain.mlp_set_threshold(thr)
    return thr, rec, (tl / tl0 if tl0 else 1.0), st


def baseline_load(chain: Chain, det, events, per_run: int = 16, flags: int = 0) -> dict:
    """Pre-filter counts with every candidate kept (the plain chain's load)."""
    p, thr = chain.mlp_params()
    _, _, st = pruned_counts(chain, det, events, -1e30, per_run, flags)
    chain.mlp_set_threshold(thr)
    return st


def save(path: str, params, thr: float, meta: dict):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    np.savez(path, params=np.asarray(params, np.float32), threshold=np.float32(thr), meta=json.dumps(meta, sort_keys=True))


def load(path: str):
    """(parameters, threshold, meta)"""
    with np.load(path) as f:
        return f["params"].astype(np.float32), float(f["threshold"]), json.loads(str(f["meta"]))


# ---------------------------------------------------------------- workloads
def flat_events(seeds):
    det = synth.detector("barrel_flat")
    return det, [synth.make_event(det, s, "barrel_flat") for s in seeds]


def pu_events(seeds, pu_lo: float, pu_hi: float, salt: int = 0):
    """Full-geometry events with PU drawn uniformly in [pu_lo, pu_hi] (from
    the seed), as the batched workloads make them"""
    det = synth.detector("full")
    out = []
    for s in seeds:
        pu = np.random.default_rng(s + 7919 * salt).uniform(pu_lo, pu_hi)
        out.append(synth.make_event(det, s, "full", n_pu=int(round(7000 * pu / 200.0))))
    return det, out


def evaluate(chain: Chain, det, events, per_run: int = 16, flags: int = 0) -> dict:
    """Recall against the plain chain and pruning of the loaded pre-filter
    (parameters and threshold as set) on `events`."""
    tl0, tc0 = plain_counts(chain, det, events, per_run, flags)
    base = baseline_load(chain, det, events, per_run, flags)
    _, thr = chain.mlp_params()
    tl, tc, st = pruned_counts(chain, det, events, thr, per_run, flags)
    return {
        "events": len(events), "tc_plain": tc0, "tc_pruned": tc, "tc_recall": tc / tc0 if tc0 else 1.0,
        "tl_plain": tl0, "tl_pruned": tl, "tl_recall": tl / tl0 if tl0 else 1.0,
        "candidates": st["candidates"], "scored": st["scored"], "kept": st["kept"],
        "pruned_fraction": 1.0 - st["kept"] / max(1, st["scored"]),
        "exact_cut_load_reduction": 1.0 - st["kept"] / max(1, base["kept"]),
    }


def fit(chain: Chain, det, train, held, *, neg_keep: float, epochs: int, batch: int, lr: float, pos_weight: float,
        target: float, seed: int = 1, per_run: int = 16, log=print) -> dict:
    """Collect on `train`, train, and calibrate the threshold on `held`;
    returns the parameters and a report."""
    t0 = time.time()
    chain.mlp_clear_samples()
    chain.mlp_init(seed)
    n = collect(chain, det, train, neg_keep, seed * 1000, per_run)
    pos = int(chain.mlp_labels().sum())
    log("samples %d (accepted %d) from %d events in %.1f s" % (n, pos, len(train), time.time() - t0))
    t1 = time.time()
    losses = chain.mlp_train(epochs, batch, lr, pos_weight, seed)
    log("trained %d epochs in %.1f s, loss %.4f -> %.4f" % (epochs, time.time() - t1, losses[0], losses[-1]))
    chain.mlp_clear_samples()
    base = baseline_load(chain, det, held, per_run)
    thr, rec, tl_rec, st = calibrate(chain, det, held, target, per_run)
    params, _ = chain.mlp_params()
    report = {
        "train_events": len(train), "held_out_events": len(held), "samples": n, "accepted_samples": pos,
        "neg_keep": neg_keep, "epochs": epochs, "batch": batch, "lr": lr, "pos_weight": pos_weight,
        "loss_first": float(losses[0]), "loss_last": float(losses[-1]), "threshold": thr,
        "tc_recall": rec, "tl_recall": tl_rec, "target": target,
        "candidates": base["candidates"], "scored": base["scored"], "kept": st["kept"],
        "pruned_fraction": 1.0 - st["kept"] / max(1, st["scored"]),
        "exact_cut_load_reduction": 1.0 - st["kept"] / max(1, base["kept"]),
    }
    log(json.dumps(report, sort_keys=True))
    return {"params": params, "threshold": thr, "report": report}


def main(argv):
    which = argv[1] if len(argv) > 1 else "flat"
    out_dir = argv[2] if len(argv) > 2 else WEIGHTS
    chain = Chain(0)
    if which == "flat":
        # barrel-only events of 100 helices + 1,000 noise hits: training seeds
        # 0-499, threshold chosen on seeds 600-699, evaluated on the 100
        # held-out seeds 500-599
        det, train = flat_events(range(0, 500))
        _, val = flat_events(range(600, 700))
        _, held = flat_events(range(500, 600))
        out = fit(chain, det, train, val, neg_keep=1.0, epochs=60, batch=4096, lr=3e-3, pos_weight=4.0,
                  target=0.997, per_run=100)
        out["report"]["held_out"] = evaluate(chain, det, held, per_run=100)
        print(json.dumps(out["report"]["held_out"], sort_keys=True))
        save(os.path.join(out_dir, "tl_mlp_flat.npz"), out["params"], out["threshold"], out["report"])
    elif which == "pu":
        # full-geometry events, PU uniform in 100-300: training seeds
        # 100000-100023, threshold chosen on seeds 100100-100111 (PU 150-300);
        # all disjoint from the benchmark's and the tests' seeds
        det, train = pu_events(range(100000, 100024), 100.0, 300.0)
        _, val = pu_events(range(100100, 100112), 150.0, 300.0)
        out = fit(chain, det, train, val, neg_keep=0.15, epochs=15, batch=16384, lr=2e-3, pos_weight=4.0,
                  target=0.997, per_run=4)
        save(os.path.join(out_dir, "tl_mlp_pu.npz"), out["params"], out["threshold"], out["report"])
    else:
        raise SystemExit("usage: python -m sdl_gb300.mlp flat|pu [out_dir]")
    chain.close()


if __name__ == "__main__":
    main(sys.argv)
