#!/usr/bin/env python
"""Benchmark of the GB300 segment-linking chain.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Headline workload (events/s): the batched chain with the learned tracklet
pre-filter on 128 events of uneven size, PU drawn uniformly in 150-300, full
synthetic geometry (barrel with tilted layers 1-3, 5 endcap disks per side;
per PU unit 35 helices pT = 0.6 + Exp(0.7) GeV, plus 20 signal helices,
|eta| < 2.5, 2 % noise hits), all events in one launch sequence per stage
replayed from a CUDA graph: createMiniDoublets -> createSegmentsWithModuleMap
-> createTrackletsWithModuleMap (pre-filter + exact cuts) -> createTriplets
-> createTrackCandidates.  In the same line: the plain batched chain on the
same events (no pre-filter) and the track-candidate recall of the pruned
chain against it, and the plain chain on one PU200-like event per step (the
configuration whose object sets are checked bit for bit against the
reference).

One JSON line is printed by rank 0.  Under torchrun every rank runs its own
events (weak scaling, no collective on the data path); the barrier and the
max over ranks use gloo on the host.

--impl reference times the reference algorithm on the host cores: the CPU
restatement in oracle/ (the reference's own sources cannot be built on the
GPU host), run on all host threads, one bounded sample of events of the
headline workload per step.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "events/s at PU200-like density, plain vs batched+MLP-pruned at ≥99.5% TC recall"
WORKLOAD = ("batched + MLP-pruned chain: 128 events of PU uniform in 150-300 (full synthetic geometry: tilted "
            "barrel L1-3, 5 endcap disks/side; 35 helices per PU unit pT=0.6+Exp(0.7) GeV + 20 signal, |eta|<2.5, "
            "2% noise), one launch sequence per stage from a CUDA graph, learned pre-filter ahead of the tracklet cuts")
SINGLE_WORKLOAD = ("plain chain, 1 PU200-like event per step (7,000 helices + 20 signal, 2% noise), "
                   "object sets identical to the reference")
MLP_WEIGHTS = os.path.join(ROOT, "sdl_gb300", "weights", "tl_mlp_pu.npz")
FALLBACK_HBM_GBS = 6800.0
FALLBACK_BF16_TFLOPS = 1900.0
MLP_FLOPS_PER_CANDIDATE = 2 * (16 * 64 + 64 * 64 + 64)  # the two MMAs (K padded to 16) and the output layer


def dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as td
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        td.init_process_group("gloo", rank=rank, world_size=world)
        pg = td
    return rank, world, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def allmax(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def allsum(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


def _gen(args):
    from sdl_gb300 import synth
    seed, pu = args
    det = synth.detector("full")
    return synth.make_event(det, seed, "full", n_pu=int(round(7000 * pu / 200.0)))


def make_events(seeds_pus, procs):
    """Events are generated in worker processes started before any CUDA call."""
    from sdl_gb300 import synth
    synth.detector("full")  # built once here, inherited by the workers
    if procs <= 1 or len(seeds_pus) <= 1:
        return [_gen(a) for a in seeds_pus]
    import multiprocessing as mp
    with mp.get_context("fork").Pool(min(procs, len(seeds_pus))) as pool:
        return pool.map(_gen, seeds_pus)


class Clocks:
    """nvidia-smi samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.path = tempfile.mktemp(suffix=".csv")
        self.p = None
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(device), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, mx, reasons = [], 0.0, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        with open(self.path) as f:
            for line in f:
                c = [x.strip() for x in line.split(",")]
                if len(c) < 9:
                    continue
                try:
                    sm.append(float(c[1]))
                    mx = max(mx, float(c[2]))
                except ValueError:
                    continue
                for k, n in enumerate(names):
                    if c[5 + k].lower().startswith("active"):
                        reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


class L2Flush:
    """Writes a 512 MiB device buffer (4x the 129 MB L2) between timed steps."""

    def __init__(self, device):
        self.rt = ctypes.CDLL("libcudart.so.13") if os.path.exists("/usr/local/cuda/lib64/libcudart.so.13") else ctypes.CDLL("libcudart.so")
        self.rt.cudaSetDevice(device)
        self.n = 512 << 20
        self.p = ctypes.c_void_p()
        if self.rt.cudaMalloc(ctypes.byref(self.p), ctypes.c_size_t(self.n)) != 0:
            raise RuntimeError("cudaMalloc for the L2 flush buffer failed")
        self.k = 0

    def __call__(self):
        self.k = (self.k + 1) & 0xff
        self.rt.cudaMemset(self.p, self.k, ctypes.c_size_t(self.n))
        self.rt.cudaDeviceSynchronize()


def peaks():
    """(HBM GB/s, bf16 TFLOP/s sustained, source)"""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        tf = float(d.get("bf16_tflops_sustained") or d.get("bf16_tflops") or FALLBACK_BF16_TFLOPS)
        return float(d["hbm_gbs"]), tf, "measured"
    except Exception:
        return FALLBACK_HBM_GBS, FALLBACK_BF16_TFLOPS, "fallback"


def ncu_traffic(name):
    """DRAM bytes per algorithmic byte of a kernel from a committed ncu summary."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return None


def headline_pus(rank, n):
    import numpy as np
    return np.random.default_rng(4242 + rank).uniform(150.0, 300.0, size=n)


def headline_plan(rank, n):
    """(seed, PU) of the n headline events of a rank: every rank runs its own
    events (weak scaling); seeds of different ranks never coincide for n < 497"""
    base = 1000 + 997 * rank
    return [(base + 500 + k, float(p)) for k, p in enumerate(headline_pus(rank, n))]


def dense_plan(rank, n):
    """(seed, PU) of the stated-density batch of a rank: PU uniform in
    227-474, which gives 110k-230k hits per event with this generator (about
    485 hits per PU unit), the hit counts the 128-event configuration states"""
    import numpy as np
    base = 1000 + 997 * rank
    pus = np.random.default_rng(4343 + rank).uniform(227.0, 474.0, size=n)
    return [(base + 300 + k, float(p)) for k, p in enumerate(pus)]


def uneven_plan(rank, n):
    """(seed, PU) of the batch of uneven events of a rank: PU uniform in
    50-250 (the 64-event plain batched configuration: 30k-121k hits per event
    with this generator, 4.79M in all)"""
    import numpy as np
    pus = np.random.default_rng(3303 + rank).uniform(50.0, 250.0, size=n)
    return [(30000 + 997 * rank + k, float(p)) for k, p in enumerate(pus)]


def single_plan(rank, n):
    """(seed, PU) of the single-event workload of a rank"""
    base = 1000 + 997 * rank
    return [(base + k, 200.0) for k in range(n)]


def cpu_sample(events, threads, digests=False):
    """events/s of the CPU restatement on `threads` host threads; with
    digests, also each event's object counts, multiset digests and counters
    (the parity check of the GPU chain on the same events)"""
    import oracle
    from sdl_gb300 import synth
    orc = oracle.Oracle(synth.detector("full"))
    t0 = time.perf_counter()
    if digests:
        res = orc.run_many_digest(events, threads)
    else:
        res = orc.run_many(events, threads)
    dt = time.perf_counter() - t0
    return len(events) / dt, dt, res


# Algorithmic bytes per unit of each stage (the roofline numerator): inputs
# read once + outputs written once, with the record widths of the reference's
# objects as device SoA (hit 20 B as input / 28 B prepared, MD 36 B, SG 28 B,
# TL / TP / TC 8 B)
STAGE_BYTES = {
    "ingest": lambda n: 20 * n["hits"] + 28 * n["hits"],
    "MD": lambda n: 28 * n["hits"] + 36 * n["MD"],
    "SG": lambda n: 36 * n["MD"] + 28 * n["SG"],
    "TL": lambda n: 28 * n["SG"] + 8 * n["TL"],
    "TP": lambda n: 8 * n["SG"] + 8 * n["TP"],
    "TC": lambda n: 8 * n["TL"] + 8 * n["TC"],
}
STAGE_NAMES = ("ingest", "MD", "SG", "TL", "TP", "TC")


def stage_roofline(n_hits, objs, stage_ms, hbm):
    """Per stage: algorithmic bytes, device ms, achieved GB/s and the fraction
    of the measured HBM bandwidth."""
    n = {"hits": int(n_hits), "MD": int(objs[0]), "SG": int(objs[1]), "TL": int(objs[2]), "TP": int(objs[3]),
         "TC": int(objs[4])}
    out = {}
    for k, ms in zip(STAGE_NAMES, stage_ms):
        b = STAGE_BYTES[k](n)
        gbs = b / (float(ms) * 1e-3) / 1e9 if ms > 0 else 0.0
        out[k] = {"bytes": int(b), "ms": round(float(ms), 3), "achieved_gbs": round(gbs, 2),
                  "frac": round(gbs / hbm, 6)}
    return out


def event_digests(ch, n_ev, keep_tc=False):
    """Per event of the last run: object counts, multiset digests (the CPU
    checker's digest) and the per-layer counters; with keep_tc also the track
    candidates of every event"""
    import numpy as np
    from sdl_gb300 import tuples
    counts = np.array([ch.counts(e) for e in range(n_ev)], dtype=np.int64)
    digests = np.zeros((n_ev, 5), dtype=np.uint64)
    tc = None
    for s in range(5):
        parts = tuples.split_by_event(ch.objects(s, -1), counts[:, s])
        for e, p in enumerate(parts):
            digests[e, s] = tuples.multiset_digest(p)
        if s == 4 and keep_tc:
            tc = parts
        del parts
    counters = np.array([ch.counters(e) for e in range(n_ev)], dtype=np.uint32)
    return (counts, digests, counters, tc) if keep_tc else (counts, digests, counters)


def run_reference_arm(a, rank, world, pg):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    import oracle
    oracle.build()
    n_ev = max(1, threads)
    # events spread evenly over the headline batch (same seeds and PU draws);
    # the whole batch is generated to state how the sample compares with it
    batch = make_events(headline_plan(0, 128), threads)
    events = batch[::max(1, len(batch) // n_ev)][:n_ev]
    batch_mean = sum(len(e) for e in batch) / len(batch)
    for _ in range(a.warmup):
        cpu_sample(events[: max(1, threads // 4)], threads)
    rates, secs = [], []
    for s in range(a.steps):
        r, dt, _ = cpu_sample(events, threads)
        rates.append(r)
        secs.append(dt)
    total = sum(secs)
    value = a.steps * n_ev / total
    hits = int(sum(len(e) for e in events))
    sample = ("%d events spread evenly over the headline batch per step (PU 150-300; %d hits, %.0f per event against "
              "%.0f per event in the whole 128-event batch), plain chain per event (the reference has no "
              "pre-filter), %d host threads" % (n_ev, hits, hits / n_ev, batch_mean, threads))
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "events/s", "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(1e3 * total / a.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "events_per_step": n_ev, "hits_per_step": hits,
                   "hits_per_s": round(a.steps * hits / total, 1),
                   "implementation": "CPU restatement of the reference chain (oracle/), multi-threaded"},
        "cpu_baseline": {"value": round(value, 4), "unit": "events/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 4), "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def timed_runs(ch, flags, steps, flush):
    """device ms per run (CUDA events around the chain on its stream), per
    stage, of the tracklet kernels, and of the tracklet passes (enumeration +
    float cuts, pre-filter, double-precision cuts)"""
    out, stage, tl, pf = [], [], [], []
    for _ in range(steps):
        flush()
        ch.run(4, flags)
        t = ch.times()
        out.append(float(t[6]))
        stage.append(t[:6].copy())
        tl.append(float(ch.kernel_times()[2]))
        pf.append(ch.tl_pass_times().copy())
    return out, stage, tl, pf


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=("gb300", "reference"))
    ap.add_argument("--batch-events", type=int, default=128)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-dense", action="store_true", help="skip the stated-density batch")
    ap.add_argument("--plain-only", action="store_true",
                    help="time only the plain batched chain (a short run to profile its kernels)")
    ap.add_argument("--mlp-only", action="store_true",
                    help="time only the pre-filtered batched chain (a short run to profile its kernels)")
    a = ap.parse_args()
    a.warmup = max(a.warmup, 3)
    rank, world, local, pg = dist()
    if a.impl == "reference":
        run_reference_arm(a, rank, world, pg)
        return

    import numpy as np
    from sdl_gb300 import synth, tuples
    threads = os.cpu_count() or 1
    # ---- inputs (generated before any CUDA call) ----------------------------
    batch = make_events(headline_plan(rank, a.batch_events), threads)
    single = make_events(single_plan(rank, 4), threads)
    dense_batch = [] if (a.no_dense or a.plain_only or a.mlp_only) else make_events(dense_plan(rank, a.batch_events), threads)
    uneven_batch = [] if (a.plain_only or a.mlp_only) else make_events(uneven_plan(rank, 64), threads)
    # the CPU baseline runs the restatement on the whole batch (about 30 s on
    # 16 cores) and doubles as the parity check of the plain batched chain on
    # every event; with fewer than 8 host threads, on every 8th event
    cpu_pick = []
    if rank == 0 and not a.no_cpu_baseline:
        cpu_pick = list(range(len(batch))) if threads >= 8 else list(range(0, len(batch), 8))

    from __graft_entry__ import build
    build()
    from sdl_gb300 import FLAG_MLP, Chain, mlp
    if not os.path.exists(MLP_WEIGHTS):
        raise SystemExit("missing pre-filter parameters: %s" % MLP_WEIGHTS)
    params, thr, meta = mlp.load(MLP_WEIGHTS)
    det = synth.detector("full")
    ch = Chain(local)
    ch.upload_detector(det)
    ch.mlp_set_params(params, thr)
    flush = L2Flush(local)

    if a.plain_only or a.mlp_only:
        fl = FLAG_MLP if a.mlp_only else 0
        ch.set_events(batch)
        tuned_plain = ch.autotune(4, fl)
        for _ in range(a.warmup):
            ch.run(4, fl)
        p_ms, p_stage, _, p_pass = timed_runs(ch, fl, a.steps, flush)
        if rank == 0:
            out = {"workload": "%s batched chain, %d events of PU uniform in 150-300"
                               % ("pre-filtered" if fl else "plain", len(batch)),
                   "ms_per_step": round(statistics.fmean(p_ms), 3), "tuned": tuned_plain,
                   "stage_ms": [round(float(v), 3) for v in np.mean(np.array(p_stage), axis=0)],
                   "tl_passes_ms": [round(float(v), 3) for v in np.mean(np.array(p_pass), axis=0)],
                   "objects": [int(v) for v in ch.counts(-1)], "global_modules": len(batch) * ch.num_modules}
            if fl:
                out["prefilter"] = ch.mlp_stats()
            print(json.dumps(out))
        ch.close()
        return

    # ---- headline: batched + pre-filter, device-resident inputs --------------
    ch.set_events(batch)
    ch.run(4, FLAG_MLP)
    tuned = ch.autotune(4, FLAG_MLP)  # launch shapes per stage for this workload (untimed)
    for _ in range(a.warmup):
        ch.run(4, FLAG_MLP)
    n_pruned = ch.counts(-1)
    mstats = ch.mlp_stats()
    lists = ch.tl_list_counts()
    # the pruned chain's track candidates per event (for the exact recall)
    pruned_ev = [int(ch.counts(e)[4]) for e in range(len(batch))]
    pruned_tc = tuples.split_by_event(ch.objects(4, -1), pruned_ev)
    clocks = Clocks(local)
    barrier(pg)
    t_wall0 = time.perf_counter()
    step_ms, stage_ms, tl_ms, pf_ms = timed_runs(ch, FLAG_MLP, a.steps, flush)
    wall = time.perf_counter() - t_wall0
    barrier(pg)
    clk = clocks.stop()
    launches = ch.launches
    mean_ms = allmax(pg, statistics.fmean(step_ms))
    value = allsum(pg, len(batch)) * 1e3 / mean_ms
    hl_stage = np.mean(np.array(stage_ms), axis=0)

    # ---- end to end through the C ABI: pinned host buffers in, track
    # candidates out, for the whole batch each step (the launch shapes tuned
    # above for this chain) -----------------------------------------------------
    n_hit = int(sum(len(e) for e in batch))
    pin = ch.pinned(n_hit * 20 + 64)
    evoff = np.zeros(len(batch) + 1, dtype=np.int64)
    evoff[1:] = np.cumsum([len(e) for e in batch])
    views = []
    for k, (attr, dt) in enumerate((("x", np.float32), ("y", np.float32), ("z", np.float32), ("idx", np.int32),
                                    ("detid", np.uint32))):
        v = pin[k * n_hit * 4:(k + 1) * n_hit * 4].view(dt)
        v[:] = np.concatenate([getattr(e, attr) for e in batch])
        views.append(v)
    # the result buffers are pinned too (two, used in turn), each sized for
    # twice the headline run's track candidates
    n_tc_cap = 2 * int(n_pruned[4]) + 1024
    tc_outs = [ch.pinned(n_tc_cap * 16 * 4).view(np.int32).reshape(n_tc_cap, 16) for _ in range(2)]

    in_ptrs = (len(batch), evoff.ctypes.data, *[v.ctypes.data for v in views])

    def e2e_step(k):
        ch.set_events_raw(*in_ptrs)
        ch.run(4, FLAG_MLP)
        return ch.objects(4, -1, out=tc_outs[k & 1]).nbytes + 8 * 2

    def e2e_stream(n):
        """n steps streamed: the first step's inputs by sdlg_set_events, every
        later step's staged during the step before it (sdlg_stage_events);
        each step's candidates gathered and copied out while the next step
        runs (sdlg_get_objects_async); returns the bytes read per step"""
        ch.set_events_raw(*in_ptrs)
        out = []
        for k in range(n):
            ch.run_async(4, FLAG_MLP)
            if k + 1 < n:
                ch.stage_events_raw(*in_ptrs)
            ch.sync()
            out.append(ch.objects_async(4, -1, tc_outs[k & 1]) * 64 + 8 * 2)
        ch.wait_objects()
        return out

    # (1) one step after another, each ending when its candidates are in host
    # memory; L2 flushed before each step
    e2e_ms, d2h = [], []
    for k in range(a.warmup + a.steps):
        flush()
        t0 = time.perf_counter()
        nb = e2e_step(k)
        t1 = time.perf_counter()
        if k >= a.warmup:
            e2e_ms.append((t1 - t0) * 1e3)
            d2h.append(nb)
    e2e_sync_mean = allmax(pg, statistics.fmean(e2e_ms))
    # (2) the same steps streamed: each step's inputs copied in during the
    # step before it and its candidates copied out during the step after it;
    # timed from the first step's inputs to the last step's candidates in
    # host memory (inputs of 280 MB, above the L2's 129 MB)
    e2e_stream(a.warmup)
    flush()
    barrier(pg)
    t0 = time.perf_counter()
    d2h_p = e2e_stream(a.steps)
    t1 = time.perf_counter()
    e2e_mean = allmax(pg, (t1 - t0) * 1e3 / a.steps)
    e2e_value = allsum(pg, len(batch)) * 1e3 / e2e_mean
    e2e_sync_value = allsum(pg, len(batch)) * 1e3 / e2e_sync_mean

    # ---- the plain batched chain on the same events --------------------------
    tuned_plain = ch.autotune(4, 0)
    for _ in range(2):
        ch.run(4, 0)
    n_plain = ch.counts(-1)
    p_ms, p_stage, p_tl, p_pass = timed_runs(ch, 0, max(3, a.steps // 4), flush)
    p_mean = allmax(pg, statistics.fmean(p_ms))
    # recall of the pruned chain: |pruned & plain| / |plain| over the track
    # candidate multisets, event by event (the pruned sets must be subsets)
    g_counts, g_digests, g_counters, plain_tc = event_digests(ch, len(batch), keep_tc=True)
    tc_common = sum(tuples.multiset_intersection(p, q) for p, q in zip(pruned_tc, plain_tc))
    tc_rec = tc_common / max(1.0, float(n_plain[4]))
    tc_outside = int(n_pruned[4]) - tc_common
    del pruned_tc, plain_tc
    tl_rec = float(n_pruned[2]) / max(1.0, float(n_plain[2]))
    plain_batched = {"value": round(allsum(pg, len(batch)) * 1e3 / p_mean, 3), "unit": "events/s", "tuned": tuned_plain,
                     "ms_per_step": round(p_mean, 3), "objects_per_step": [int(v) for v in n_plain],
                     "stage_ms": [round(float(v), 3) for v in np.mean(np.array(p_stage), axis=0)],
                     "tl_kernel_ms": round(statistics.fmean(p_tl), 3),
                     "tl_passes_ms": {"enumeration_and_float_cuts": round(float(np.mean([v[0] for v in p_pass])), 3),
                                      "b2_filter": round(float(np.mean([v[2] for v in p_pass])), 3),
                                      "double_cuts": round(float(np.mean([v[3] for v in p_pass])), 3)}}

    # ---- the chain's other variants on the same events (plain chain, shapes
    # tuned for the module-map chain) ---------------------------------------------
    from sdl_gb300 import FLAG_TC_FROM_TL, FLAG_TC_FROM_TP, FLAG_TL_NAV
    variants = {}
    for vname, vflags in (("tracklets_via_navigation", FLAG_TL_NAV),
                          ("track_candidates_from_tracklets", FLAG_TC_FROM_TL),
                          ("track_candidates_from_triplets", FLAG_TC_FROM_TP)):
        for _ in range(2):
            ch.run(4, vflags)
        v_ms, v_stage, _, _ = timed_runs(ch, vflags, 3, flush)
        v_mean = allmax(pg, statistics.fmean(v_ms))
        variants[vname] = {"flags": vflags, "value": round(allsum(pg, len(batch)) * 1e3 / v_mean, 3),
                           "unit": "events/s", "ms_per_step": round(v_mean, 3),
                           "objects_per_step": [int(v) for v in ch.counts(-1)],
                           "stage_ms": [round(float(v), 3) for v in np.mean(np.array(v_stage), axis=0)]}

    # ---- the stated density: 110k-230k hits per event --------------------------
    # (the headline batch's PU 150-300 gives 73k-146k with this generator);
    # pre-filtered and plain chain on the same events, exact recall
    dense = None
    if dense_batch:
        nd = len(dense_batch)
        ch.set_events(dense_batch)
        for _ in range(2):
            ch.run(4, FLAG_MLP)
        dm_ms, dm_stage, _, _ = timed_runs(ch, FLAG_MLP, max(3, a.steps // 4), flush)
        d_pruned = ch.counts(-1)
        d_mstats = ch.mlp_stats()
        d_pr = tuples.split_by_event(ch.objects(4, -1), [int(ch.counts(e)[4]) for e in range(nd)])
        for _ in range(2):
            ch.run(4, 0)
        dp_ms, dp_stage, _, _ = timed_runs(ch, 0, max(3, a.steps // 4), flush)
        d_plain = ch.counts(-1)
        d_pl = tuples.split_by_event(ch.objects(4, -1), [int(ch.counts(e)[4]) for e in range(nd)])
        d_common = sum(tuples.multiset_intersection(p, q) for p, q in zip(d_pr, d_pl))
        del d_pr, d_pl
        hits = [len(e) for e in dense_batch]
        dm_mean = allmax(pg, statistics.fmean(dm_ms))
        dp_mean = allmax(pg, statistics.fmean(dp_ms))
        dense = {"workload": "%d events, PU uniform in 227-474 (%d-%d hits per event, mean %.0f)"
                             % (nd, min(hits), max(hits), statistics.fmean(hits)),
                 "hits_per_step": int(sum(hits)),
                 "value": round(allsum(pg, nd) * 1e3 / dm_mean, 3), "unit": "events/s", "ms_per_step": round(dm_mean, 3),
                 "plain_value": round(allsum(pg, nd) * 1e3 / dp_mean, 3), "plain_ms_per_step": round(dp_mean, 3),
                 "tc_recall": round(d_common / max(1.0, float(d_plain[4])), 5),
                 "tl_recall": round(float(d_pruned[2]) / max(1.0, float(d_plain[2])), 5),
                 "tc_outside_plain": int(d_pruned[4]) - d_common,
                 "objects_per_step": [int(v) for v in d_pruned], "plain_objects_per_step": [int(v) for v in d_plain],
                 "prefilter": {k: d_mstats[k] for k in ("candidates", "scored", "kept")},
                 "stage_ms": {k: round(float(v), 3) for k, v in zip(STAGE_NAMES, np.mean(np.array(dm_stage), axis=0))},
                 "plain_stage_ms": {k: round(float(v), 3) for k, v in zip(STAGE_NAMES, np.mean(np.array(dp_stage), axis=0))}}

    # ---- the plain batched chain on 64 events of uneven size (PU 50-250) ------
    uneven = None
    if uneven_batch:
        nu = len(uneven_batch)
        ch.set_events(uneven_batch)
        ch.run(4, 0)
        tuned_uneven = ch.autotune(4, 0)
        for _ in range(2):
            ch.run(4, 0)
        u_ms, u_stage, _, _ = timed_runs(ch, 0, max(3, a.steps // 4), flush)
        u_mean = allmax(pg, statistics.fmean(u_ms))
        hits_u = [len(e) for e in uneven_batch]
        uneven = {"workload": "plain batched chain, %d events of uneven size, PU uniform in 50-250 (%d-%d hits per "
                              "event)" % (nu, min(hits_u), max(hits_u)),
                  "value": round(allsum(pg, nu) * 1e3 / u_mean, 3), "unit": "events/s", "ms_per_step": round(u_mean, 3),
                  "hits_per_step": int(sum(hits_u)), "hits_per_s": round(sum(hits_u) * 1e3 / u_mean, 1),
                  "objects_per_step": [int(v) for v in ch.counts(-1)], "tuned": tuned_uneven,
                  "stage_ms": {k: round(float(v), 3) for k, v in zip(STAGE_NAMES, np.mean(np.array(u_stage), axis=0))},
                  "parity": "tests/test_batch_parity_gpu.py: every event against the CPU restatement"}

    # ---- plain chain, one PU200-like event per step --------------------------
    ev = single[0]
    ch.set_events([ev])
    ch.run(4, 0)
    tuned_single = ch.autotune(4, 0)
    for _ in range(a.warmup):
        ch.run(4, 0)
    s_counts = ch.counts(0)
    s_ms, s_stage, s_tl, _ = timed_runs(ch, 0, a.steps, flush)
    s_mean = allmax(pg, statistics.fmean(s_ms))
    s_st = np.mean(np.array(s_stage), axis=0)
    plain_single = {"value": round(allsum(pg, 1.0) * 1e3 / s_mean, 3), "unit": "events/s", "ms_per_step": round(s_mean, 4),
                    "workload": SINGLE_WORKLOAD, "hits_per_event": len(ev),
                    "objects_per_event": [int(v) for v in s_counts],
                    "stage_ms": {k: round(float(v), 4) for k, v in zip(("ingest", "MD", "SG", "TL", "TP", "TC"), s_st)},
                    "tuned": tuned_single,
                    "tl_kernel_ms": round(statistics.fmean(s_tl), 4)}

    # ---- roofline of the dominant kernel of the headline run -----------------
    # k_tl_enum_tiles (tracklet enumeration in module-pair tiles, the float
    # cuts and the single-precision decision of the first tracklet cuts).
    # Algorithmic bytes = the tracklet stage's input, 28 B per segment read
    # once (the tracklets, 8 B each, are written by k_tl_b2).  layout_bytes =
    # what this kernel's own data layout reads and writes once: each
    # segment's record as inner segment (112 B), its eleven outer-role fields
    # (44 B) and its entry in the index of segments by outer module (4 B),
    # each global module's tile offset, segment offset and connection sum
    # (24 B), each surviving candidate's list entry (16 B).  traffic = DRAM
    # bytes per layout byte of an ncu capture of the kernel, times this
    # launch's layout bytes.
    hbm, tflops, src = peaks()
    pf = np.mean(np.array(pf_ms), axis=0)
    fc_mean, pf_mean, bf_mean, ex_mean = float(pf[0]), float(pf[1]), float(pf[2]), float(pf[3])
    n_sg = int(n_pruned[1])
    n_gm = len(batch) * ch.num_modules
    en_alg = 28 * n_sg
    en_layout = (112 + 44 + 4) * n_sg + 24 * n_gm + 16 * lists["listed"]
    # k_tl_b2f (phase B2's single-precision filter over the pre-filter's kept
    # list): each entry read once (16 B), each segment's 128-byte record read
    # once, each entry it leaves written once (16 B)
    bf_alg = 16 * lists["kept"] + 128 * n_sg + 16 * lists["filtered"]
    bf_achieved = bf_alg / (bf_mean * 1e-3) / 1e9
    en_achieved = en_alg / (fc_mean * 1e-3) / 1e9
    tr = ncu_traffic("tl_enum_traffic.json")
    en_traffic = None
    if tr and tr.get("traffic_per_layout_byte"):
        en_traffic = int(en_layout * float(tr["traffic_per_layout_byte"]))
    # k_tl_prefilter (the network over the enumeration's survivor list):
    # algorithmic bytes = each scored entry read once (16 B) + each segment's
    # feature record read once (64 B) + each kept entry written once (16 B);
    # tensor work = the network's MMAs per scored candidate
    alg_bytes = 16 * mstats["scored"] + 64 * n_sg + 16 * mstats["kept"]
    achieved = alg_bytes / (pf_mean * 1e-3) / 1e9
    tr = ncu_traffic("tl_prefilter_traffic.json")
    traffic = None
    if tr and tr.get("traffic_per_layout_byte"):
        traffic = int(alg_bytes * float(tr["traffic_per_layout_byte"]))
    mma_tflops = mstats["scored"] * MLP_FLOPS_PER_CANDIDATE / (pf_mean * 1e-3) / 1e12
    roofline = {"bound": "hbm", "achieved": round(en_achieved, 3), "peak": hbm, "unit": "GB/s",
                "frac": round(en_achieved / hbm, 6), "traffic": en_traffic, "peak_source": src,
                "kernel": "k_tl_enum_tiles (tracklet candidate enumeration in module-pair tiles, the float cuts and "
                          "the single-precision phase-B1 decision)",
                "kernel_ms": round(fc_mean, 3), "algorithmic_bytes": en_alg,
                "algorithmic_bytes_rule": "28 B per segment (the tracklet stage's input, read once)",
                "layout_bytes": en_layout,
                "layout_achieved_gbs": round(en_layout / (fc_mean * 1e-3) / 1e9, 3),
                "candidates": mstats["candidates"],
                "candidates_per_s": round(mstats["candidates"] / (fc_mean * 1e-3), 1),
                "note": "issue-bound candidate evaluation (the ncu capture of this kernel shows issue slots, not DRAM, "
                        "saturated); the algorithmic bytes are small by construction",
                "b2_filter": {"kernel": "k_tl_b2f (phase B2's single-precision decision on the pre-filter's kept "
                                        "list; rejects only what the exact phase B2 rejects)",
                              "kernel_ms": round(bf_mean, 3), "algorithmic_bytes": bf_alg,
                              "achieved": round(bf_achieved, 3), "peak": hbm, "unit": "GB/s",
                              "frac": round(bf_achieved / hbm, 6), "entries": lists["kept"],
                              "left": lists["filtered"],
                              "entries_per_s": round(lists["kept"] / (bf_mean * 1e-3), 1)},
                "prefilter": {"kernel": "k_tl_prefilter (tensor-core pre-filter of the candidates through the float cuts "
                                        "and phase B1's decision)",
                              "kernel_ms": round(pf_mean, 3), "algorithmic_bytes": alg_bytes,
                              "achieved": round(achieved, 3), "peak": hbm, "unit": "GB/s",
                              "frac": round(achieved / hbm, 6), "traffic": traffic,
                              "tensor": {"achieved": round(mma_tflops, 2), "peak": tflops, "unit": "TFLOP/s",
                                         "frac": round(mma_tflops / tflops, 5),
                                         "flops_per_candidate": MLP_FLOPS_PER_CANDIDATE,
                                         "candidates": mstats["scored"]}},
                "double_cuts_ms": round(ex_mean, 3),
                "stages": stage_roofline(n_hit, n_pruned, hl_stage, hbm)}
    plain_batched["stage_roofline"] = stage_roofline(n_hit, n_plain, np.mean(np.array(p_stage), axis=0), hbm)
    plain_batched["hits_per_s"] = round(n_hit * 1e3 / p_mean, 1)
    plain_single["stage_roofline"] = stage_roofline(len(ev), s_counts, s_st, hbm)

    # ---- CPU baseline (rank 0) -----------------------------------------------
    cpu = None
    parity = None
    if rank == 0 and cpu_pick:
        cpu_events = [batch[e] for e in cpu_pick]
        r, dt, (o_counts, o_digests, o_counters) = cpu_sample(cpu_events, threads, digests=True)
        cpu_hits = sum(len(e) for e in cpu_events)
        cpu = {"value": round(r, 4), "unit": "events/s", "cores": threads, "kind": "port",
               "hits_per_s": round(cpu_hits / dt, 1),
               "sample": "%d events of the headline workload (PU 150-300, %d hits) through the CPU restatement of "
                         "the reference chain on %d threads (%.1f s)" % (len(cpu_events), cpu_hits, threads, dt)}
        bad = [(e, s) for k, e in enumerate(cpu_pick) for s in range(5)
               if g_counts[e, s] != o_counts[k, s] or g_digests[e, s] != o_digests[k, s]]
        bad_cnt = [e for k, e in enumerate(cpu_pick) if not np.array_equal(g_counters[e], o_counters[k])]
        parity = {"events_checked": len(cpu_pick), "stages": 5, "mismatches": len(bad),
                  "counter_mismatches": len(bad_cnt), "first": bad[:4],
                  "check": "plain batched chain vs the CPU restatement: per event, the five object multisets "
                           "(digests of the hit-index tuples), counts and the 110 per-layer counters"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "events/s", "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": round(mean_ms, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64 cuts, bf16 pre-filter", "data": "synthetic",
            "config": {"workload": WORKLOAD, "events_per_step": len(batch), "hits_per_step": n_hit,
                       "objects_per_step": [int(v) for v in n_pruned],
                       "l2": "flushed between steps (512 MiB memset); inputs > L2",
                       "tuned": {"note": "sdlg_autotune on this batch before timing", **tuned},
                       "stage_ms": {k: round(float(v), 3) for k, v in zip(("ingest", "MD", "SG", "TL", "TP", "TC"), hl_stage)},
                       "prefilter": {"weights": "sdl_gb300/weights/tl_mlp_pu.npz", "threshold": thr,
                                     "trained_on": "%d events, PU 100-300 (seeds 100000+)" % meta.get("train_events", 0),
                                     "candidates": mstats["candidates"],
                                     "scored_after_float_cuts_and_b1": mstats["scored"],
                                     "kept": mstats["kept"],
                                     "pruned_fraction": round(1.0 - mstats["kept"] / max(1, mstats["scored"]), 4),
                                     "left_by_b2_filter": lists["filtered"]},
                       "wall_s": round(wall, 3)},
            "tc_recall": round(tc_rec, 5), "tl_recall": round(tl_rec, 5),
            "recall_method": "track candidates: |pruned & plain| / |plain| over the hit-index tuple multisets, event "
                             "by event; tracklets: count ratio (pruned tracklets are a subset by construction)",
            "plain_batched": plain_batched, "plain_single": plain_single, "variants": variants,
            "stated_density": dense, "batched_uneven": uneven,
            "e2e": {"value": round(e2e_value, 3), "unit": "events/s", "ms_per_step": round(e2e_mean, 3),
                    "h2d_bytes_per_step": n_hit * 20 + 8 * (len(batch) + 1), "d2h_bytes_per_step": int(statistics.fmean(d2h_p)),
                    "path": "streamed steps from pinned host memory: the first step's inputs by sdlg_set_events, each "
                            "later step's by sdlg_stage_events during the step before it; per step sdlg_run_async("
                            "SDLG_FLAG_MLP) + sdlg_sync + sdlg_get_objects_async(TC, into pinned host memory), the "
                            "readback overlapping the next step's run; timed from the first inputs until "
                            "sdlg_wait_objects returns after the last step",
                    "unpipelined": {"value": round(e2e_sync_value, 3), "ms_per_step": round(e2e_sync_mean, 3),
                                    "d2h_bytes_per_step": int(statistics.fmean(d2h)),
                                    "path": "sdlg_set_events + sdlg_run + sdlg_get_objects (synchronous), "
                                            "each step timed alone, L2 flushed before it"}},
            "roofline": roofline, "cpu_baseline": cpu, "parity": parity, "tc_outside_plain": tc_outside,
            "ratios_vs_cpu_baseline": None if not cpu else {
                "headline_events": round(value / cpu["value"], 2),
                "plain_batched_events": round(plain_batched["value"] / cpu["value"], 2),
                "plain_batched_hits": round(plain_batched["hits_per_s"] / cpu["hits_per_s"], 2),
                "note": "the CPU restatement runs the plain chain; plain against plain is the like-for-like ratio"},
            "clocks": clk,
            "gpu_launches": int(launches * a.steps),
        }
        print(json.dumps(line), flush=True)
    ch.close()
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
