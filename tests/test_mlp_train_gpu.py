"""Training the learned tracklet pre-filter on the GPU and what it gains.

Barrel-only events (100 helices + 1,000 noise hits): the network is trained
with the library's kernels on the plain chain's own accept/reject decisions
(seeds 0-199), its threshold is set on validation seeds 600-699 for 99.8 %
track-candidate recall, and it is judged on held-out seeds 500-599.  The
same network untrained, calibrated the same way, is the method without
training; the plain chain (no pre-filter) prunes nothing."""
import pytest

pytestmark = pytest.mark.gpu


def test_trained_prefilter_recall_and_gain():
    from sdl_gb300 import Chain, build, mlp
    build.build()
    ch = Chain(0)
    det, train = mlp.flat_events(range(0, 200))
    _, val = mlp.flat_events(range(600, 700))
    _, held = mlp.flat_events(range(500, 600))
    # untrained network: same initialisation, same calibration
    ch.mlp_init(1)
    mlp.calibrate(ch, det, val, 0.998, per_run=100)
    untrained = mlp.evaluate(ch, det, held, per_run=100)
    out = mlp.fit(ch, det, train, val, neg_keep=1.0, epochs=40, batch=4096, lr=3e-3, pos_weight=4.0, target=0.998,
                  per_run=100, log=lambda *a: None)
    assert out["report"]["loss_last"] < 0.5 * out["report"]["loss_first"]
    trained = mlp.evaluate(ch, det, held, per_run=100)
    print("untrained", untrained)
    print("trained", trained)
    # the pruned chain only ever loses objects, and keeps >= 99.5 % of the track candidates
    assert trained["tc_pruned"] <= trained["tc_plain"] and trained["tl_pruned"] <= trained["tl_plain"]
    assert trained["tc_recall"] >= 0.995
    # the trained network drops most of the candidates it scores (those through
    # the float cuts and the enumeration's direction and betaIn decision) and
    # most of the exact-cut work ...
    assert trained["pruned_fraction"] >= 0.5
    assert trained["exact_cut_load_reduction"] >= 0.5
    # ... where the untrained one, at the same recall target, drops little
    assert trained["pruned_fraction"] >= untrained["pruned_fraction"] + 0.3
    assert trained["exact_cut_load_reduction"] >= untrained["exact_cut_load_reduction"] + 0.3
    ch.close()
