"""Near-cut audit (oracle/nearcut.py) on the event of the benchmark's
headline batch where the host libm decides a cut: the CPU restatement with
correctly rounded floats loses exactly one segment there (the dAlpha cut of
Segment.cc:886-994, 732 float steps inside its bound with glibc, 804 outside
with correctly rounded floats, after the shifted strip hits moved), and the
tracklets, triplets and track candidates built on it.  The GPU chain
reproduces glibc's float functions and makes the segment (test_libm_gpu,
test_batch_parity_gpu)."""
import numpy as np


def test_headline_event_16_flip_is_listed_with_its_distance(oracle_lib):
    import bench
    from oracle import nearcut
    plan = bench.headline_plan(0, 128)[16:17]
    out = nearcut.report(plan, 2, "headline event 16")
    ps = out["per_stage"]
    assert ps["SG"]["primary_flips"] == 1 and ps["SG"]["objects_glibc"] - ps["SG"]["objects_rounded"] == 1
    assert ps["MD"]["primary_flips"] == 0 and ps["MD"]["secondary_flips"] == 0
    for s in ("TL", "TP", "TC"):
        assert ps[s]["primary_flips"] == 0
        assert ps[s]["secondary_flips"] == ps[s]["objects_glibc"] - ps[s]["objects_rounded"] > 0
    (f,) = out["flips"]
    assert f["stage"] == "SG" and f["made_with"] == "glibc" and f["algorithm"] == "dalpha_cuts"
    assert f["tuple"] == [99737, 87072, 113038, 93486]
    assert f["glibc"]["steps_inside"] > 0 >= f["rounded"]["steps_inside"]


def test_steps_measure_float_distance():
    from oracle.nearcut import steps
    one = np.float32(1.0)
    up = np.nextafter(one, np.float32(2.0))
    assert steps(float(one), float("-inf"), float(up)) == 1
    assert steps(float(up), float("-inf"), float(one)) == -1
    # across zero and between negative floats the steps stay adjacent-float counts
    assert steps(-1.0, float(np.nextafter(np.float32(-1.0), np.float32(-2.0))), float("inf")) == 1
    assert steps(0.0, -1e-45, 1e-45) == 1
