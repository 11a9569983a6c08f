"""Learned tracklet pre-filter on the GPU: the tensor-core inference kernel
and the training kernels against the CPU oracle (oracle/mlp.py), and the
pruned chain against the plain chain."""
import numpy as np
import pytest

from oracle import mlp as omlp

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from sdl_gb300 import Chain, build
    build.build()
    return Chain(0)


def _features(n, seed):
    r = np.random.default_rng(seed)
    x = r.normal(0.0, 1.5, size=(n, omlp.N_IN)).astype(np.float32)
    x[:, 11] = r.choice([0.0, 0.25, 1.0, 1.5], n)
    return x


@pytest.mark.parametrize("n", [1, 127, 128, 1283, 40000])
def test_tensor_core_logits_match_oracle(gpu, n):
    """tcgen05 BF16 x BF16 -> FP32 tiles (ragged last tile included) against
    the float64 oracle with the same BF16 roundings.  Tolerance: FP32
    accumulation order, plus the rare first-layer unit whose FP32 sum lands on
    the other side of a BF16 rounding boundary (|dz| <= 0.02 (1 + |z|))."""
    p = omlp.init_params(11)
    gpu.mlp_set_params(p, 0.0)
    x = _features(n, 7 + n)
    z = gpu.mlp_score(x)
    zr, _ = omlp.forward(p, x)
    err = np.abs(z - zr)
    assert np.all(err <= 0.02 * (1.0 + np.abs(zr))), (np.max(err), np.argmax(err))
    assert np.median(err) <= 1e-4 * (1.0 + np.median(np.abs(zr)))


def test_training_gradient_matches_oracle(gpu):
    """One forward + backward of the training kernels against the oracle's
    analytic gradient at the same parameters (relative L2 error <= 1e-3)."""
    p = omlp.init_params(21)
    gpu.mlp_set_params(p, 0.0)
    n = 1000
    x = _features(n, 3)
    r = np.random.default_rng(4)
    y = (r.random(n) < 0.3).astype(np.float32)
    w = r.uniform(0.5, 2.0, n).astype(np.float32)
    g, loss = gpu.mlp_gradient(x, y, w)
    lr, gr = omlp.loss_and_grad(p, x, y, w)
    assert abs(loss - lr) <= 1e-5 * (1 + abs(lr))
    assert np.linalg.norm(g - gr) <= 1e-3 * np.linalg.norm(gr)
    for lo, hi in ((omlp.W1, omlp.B1), (omlp.W2, omlp.B2), (omlp.W3, omlp.B3)):
        assert np.linalg.norm(g[lo:hi] - gr[lo:hi]) <= 2e-3 * np.linalg.norm(gr[lo:hi])


def test_keep_all_equals_plain_chain(gpu, oracle_lib):
    """With a threshold below every logit the pre-filtered chain must produce
    exactly the plain chain's objects (the network scores the candidates
    through the float cuts and keeps them all); with one above every logit it
    keeps no tracklet (and leaves the stages that do not read tracklets
    untouched)."""
    from sdl_gb300 import FLAG_MLP, synth
    det = synth.detector("full")
    events = [synth.make_event(det, 960, "full", n_pu=1400), synth.make_event(det, 961, "full", n_pu=350)]
    gpu.upload_detector(det)
    gpu.set_events(events)
    gpu.run(4, 0)
    plain = [[oracle_lib.digest(gpu.objects(s, e)) for s in range(5)] for e in range(2)]
    counters = [gpu.counters(e) for e in range(2)]
    gpu.mlp_set_params(omlp.init_params(5), -1e30)
    gpu.run(4, FLAG_MLP)
    got = [[oracle_lib.digest(gpu.objects(s, e)) for s in range(5)] for e in range(2)]
    assert got == plain
    for e in range(2):
        assert np.array_equal(gpu.counters(e), counters[e])
    st = gpu.mlp_stats()
    n_cand = int(sum(c[44:55].sum() for c in counters))  # tracklet candidate counters
    assert st["candidates"] == n_cand and st["timeouts"] == 0
    assert st["kept"] == st["scored"] and gpu.counts(-1)[2] <= st["scored"] < n_cand
    gpu.mlp_set_threshold(1e30)
    gpu.run(4, FLAG_MLP)
    assert gpu.counts(-1)[2] == 0 and gpu.counts(-1)[4] == 0
    for e in range(2):
        for s in (0, 1, 3):
            assert oracle_lib.digest(gpu.objects(s, e)) == plain[e][s]
    st = gpu.mlp_stats()
    assert st["kept"] == 0 and st["candidates"] == n_cand and st["scored"] > 0


def test_collect_labels_match_chain(gpu, oracle_lib):
    """The collected positives are exactly the plain chain's tracklets (one
    sample per accepted candidate)."""
    from sdl_gb300 import synth
    det, ev = synth.workload_event("barrel_flat", 3)
    gpu.upload_detector(det)
    gpu.set_events([ev])
    gpu.run(4, 0)
    gpu.mlp_clear_samples()
    n = gpu.mlp_collect(neg_keep=1.0, seed=1)
    x, y = gpu.mlp_samples()
    assert len(y) == n and n > 0
    assert int(y.sum()) == gpu.counts(0)[2]
    assert np.all(np.isfinite(x)) and np.all(np.abs(x) <= 16)
    gpu.mlp_clear_samples()
    n_half = gpu.mlp_collect(neg_keep=0.5, seed=1)
    assert gpu.counts(0)[2] <= n_half < n
    gpu.mlp_clear_samples()
