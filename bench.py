#!/usr/bin/env python
"""Benchmark of the GB300 segment-linking chain.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload (the configuration the events/s metric is quoted on): the plain
chain createMiniDoublets -> createSegmentsWithModuleMap ->
createTrackletsWithModuleMap -> createTriplets -> createTrackCandidates on
one PU200-like event per step (full synthetic geometry: barrel with tilted
layers 1-3 and 5 endcap disks per side; 7,000 helices pT = 0.6 + Exp(0.7) GeV
plus 20 signal helices, |eta| < 2.5, 2 % noise hits).  The batched form
(64 events of PU 50-250 in one launch sequence) is reported beside it.

One JSON line is printed by rank 0.  Under torchrun every rank runs its own
events (weak scaling, no collective on the data path); the barrier and the
max over ranks use gloo on the host.

--impl reference times the reference algorithm on the host cores: the CPU
restatement in oracle/ (the reference's own sources cannot be built on the
GPU host), run on all host threads, one bounded sample of events per step.
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
WORKLOAD = ("plain chain, 1 PU200-like event per step: full synthetic geometry (tilted barrel L1-3, "
            "5 endcap disks/side), 7,000 helices pT=0.6+Exp(0.7) GeV + 20 signal, |eta|<2.5, 2% noise")
BATCH_WORKLOAD = "batched plain chain: 64 events of PU uniform in 50-250, one launch sequence per stage"
FALLBACK_HBM_GBS = 6800.0


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
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic():
    """DRAM bytes per event of the tracklet kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "tl_kernel_traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return None


def cpu_sample(events, threads):
    import oracle
    from sdl_gb300 import synth
    orc = oracle.Oracle(synth.detector("full"))
    t0 = time.perf_counter()
    n_tc = orc.run_many(events, threads)
    dt = time.perf_counter() - t0
    return len(events) / dt, dt, n_tc


def run_reference_arm(a, rank, world, pg):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    import oracle
    oracle.build()
    n_ev = max(1, threads)
    events = make_events([(5000 + k, 200.0) for k in range(n_ev)], threads)
    for _ in range(a.warmup):
        cpu_sample(events[: max(1, threads // 4)], threads)
    rates, secs = [], []
    for s in range(a.steps):
        r, dt, _ = cpu_sample(events, threads)
        rates.append(r)
        secs.append(dt)
    total = sum(secs)
    value = a.steps * n_ev / total
    sample = "%d PU200-like events per step (seeds 5000-%d), whole chain per event, %d host threads" % (n_ev, 5000 + n_ev - 1, threads)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "events/s", "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(1e3 * total / a.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "events_per_step": n_ev, "implementation": "CPU restatement of the reference chain (oracle/), multi-threaded"},
        "cpu_baseline": {"value": round(value, 4), "unit": "events/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 4), "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=("gb300", "reference"))
    ap.add_argument("--batch-events", type=int, default=64)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    a = ap.parse_args()
    a.warmup = max(a.warmup, 3)
    rank, world, local, pg = dist()
    if a.impl == "reference":
        run_reference_arm(a, rank, world, pg)
        return

    import numpy as np
    from sdl_gb300 import synth
    threads = os.cpu_count() or 1
    # ---- inputs (generated before any CUDA call) ----------------------------
    base = 1000 + 997 * rank
    n_e2e = 8
    single = make_events([(base + k, 200.0) for k in range(n_e2e)], threads)
    rng = np.random.default_rng(4242 + rank)
    batch_pus = rng.uniform(50.0, 250.0, size=a.batch_events) if a.batch_events > 0 else []
    batch = make_events([(base + 500 + k, float(p)) for k, p in enumerate(batch_pus)], threads)
    cpu_events = []
    if rank == 0 and not a.no_cpu_baseline:
        cpu_events = make_events([(7000 + k, 200.0) for k in range(max(1, threads))], threads)

    from __graft_entry__ import build
    build()
    from sdl_gb300 import Chain
    det = synth.detector("full")
    ch = Chain(local)
    ch.upload_detector(det)
    flush = L2Flush(local)

    # ---- device-resident plain chain: 1 event per step ----------------------
    ev = single[0]
    ch.set_events([ev])
    for _ in range(a.warmup):
        ch.run(4)
    counts = ch.counts(0)
    clocks = Clocks(local)
    barrier(pg)
    step_ms, tl_ms, stage_ms = [], [], []
    t_wall0 = time.perf_counter()
    for _ in range(a.steps):
        flush()
        ch.run(4)
        t = ch.times()
        step_ms.append(float(t[6]))
        stage_ms.append(t[:6].copy())
        tl_ms.append(float(ch.kernel_times()[2]))
    wall = time.perf_counter() - t_wall0
    barrier(pg)
    clk = clocks.stop()
    launches = ch.launches
    mean_ms = allmax(pg, statistics.fmean(step_ms))
    value = allsum(pg, 1.0) * 1e3 / mean_ms  # every rank processes one event per step

    # ---- end to end through the C ABI: host buffers in, track candidates out --
    n_max = max(len(e) for e in single)
    pin = ch.pinned(n_max * 20 + 64)
    evoff = np.zeros(2, dtype=np.int64)

    def stage_host(e):
        n = len(e)
        views = []
        for k, (arr, dt) in enumerate(((e.x, np.float32), (e.y, np.float32), (e.z, np.float32), (e.idx, np.int32),
                                       (e.detid, np.uint32))):
            v = pin[k * n * 4:(k + 1) * n * 4].view(dt)
            v[:] = arr
            views.append(v)
        return views

    e2e_ms, h2d, d2h = [], [], []
    for k in range(a.warmup + a.steps):
        e = single[k % n_e2e]
        views = stage_host(e)  # host-side preparation of the caller's pinned buffers (not timed)
        evoff[1] = len(e)
        flush()
        t0 = time.perf_counter()
        ch.set_events_raw(1, evoff.ctypes.data, *[v.ctypes.data for v in views])
        ch.run(4)
        tc = ch.objects(4, 0)
        t1 = time.perf_counter()
        if k >= a.warmup:
            e2e_ms.append((t1 - t0) * 1e3)
            h2d.append(len(e) * 20 + 16)
            d2h.append(tc.nbytes + 8 * 2)
    e2e_mean = allmax(pg, statistics.fmean(e2e_ms))
    e2e_value = allsum(pg, 1.0) * 1e3 / e2e_mean

    # ---- batched chain ---------------------------------------------------------
    batched = None
    if batch:
        ch.set_events(batch)
        for _ in range(a.warmup):
            ch.run(4)
        bms = []
        for _ in range(max(3, a.steps // 2)):
            flush()
            ch.run(4)
            bms.append(float(ch.times()[6]))
        bmean = allmax(pg, statistics.fmean(bms))
        btot = ch.counts(-1)
        batched = {"value": round(allsum(pg, len(batch)) * 1e3 / bmean, 2), "unit": "events/s",
                   "ms_per_step": round(bmean, 3), "events_per_step": len(batch), "workload": BATCH_WORKLOAD,
                   "hits_per_step": int(sum(len(e) for e in batch)), "objects_per_step": [int(v) for v in btot],
                   "stage_ms": [round(float(v), 3) for v in ch.times()[:6]]}

    # ---- roofline of the dominant kernel (tracklet candidate evaluation) -----
    hbm, src = peaks()
    tl_mean = statistics.fmean(tl_ms)
    n_sg, n_tl = int(counts[1]), int(counts[2])
    alg_bytes = 28 * n_sg + 8 * n_tl  # segments read once (28 B) + tracklets written once (8 B)
    achieved = alg_bytes / (tl_mean * 1e-3) / 1e9
    tr = ncu_traffic()
    traffic = None
    if tr and tr.get("traffic_per_algorithmic_byte"):
        # DRAM bytes of one ncu capture of this kernel, scaled to this launch
        # by the algorithmic bytes (segments read, tracklets written)
        traffic = int(alg_bytes * float(tr["traffic_per_algorithmic_byte"]))
    roofline = {"bound": "hbm", "achieved": round(achieved, 3), "peak": hbm, "unit": "GB/s",
                "frac": round(achieved / hbm, 6), "traffic": traffic, "peak_source": src,
                "kernel": "k_tl_enum (tracklet cuts)", "kernel_ms": round(tl_mean, 4),
                "algorithmic_bytes": alg_bytes,
                "note": "latency/FP64-bound candidate evaluation; HBM bytes are small by construction"}

    # ---- CPU baseline (rank 0) -----------------------------------------------
    cpu = None
    if rank == 0 and cpu_events:
        r, dt, _ = cpu_sample(cpu_events, threads)
        cpu = {"value": round(r, 4), "unit": "events/s", "cores": threads, "kind": "port",
               "sample": "%d PU200-like events through the CPU restatement of the reference chain on %d threads (%.1f s)"
                         % (len(cpu_events), threads, dt)}

    if rank == 0:
        stage = np.mean(np.array(stage_ms), axis=0)
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "events/s", "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": round(mean_ms, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "events_per_step": 1, "hits_per_event": len(ev),
                       "objects_per_event": [int(v) for v in counts], "l2": "flushed between steps (512 MiB memset)",
                       "stage_ms": {"ingest": round(float(stage[0]), 4), "MD": round(float(stage[1]), 4),
                                    "SG": round(float(stage[2]), 4), "TL": round(float(stage[3]), 4),
                                    "TP": round(float(stage[4]), 4), "TC": round(float(stage[5]), 4)},
                       "wall_s": round(wall, 3)},
            "e2e": {"value": round(e2e_value, 3), "unit": "events/s", "ms_per_step": round(e2e_mean, 4),
                    "h2d_bytes_per_step": int(statistics.fmean(h2d)), "d2h_bytes_per_step": int(statistics.fmean(d2h)),
                    "path": "sdlg_set_events (pinned host) + sdlg_run + sdlg_get_objects(TC)"},
            "roofline": roofline, "cpu_baseline": cpu, "clocks": clk,
            "gpu_launches": int(launches * a.steps), "batched": batched,
        }
        print(json.dumps(line), flush=True)
    ch.close()
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
