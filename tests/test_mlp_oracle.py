"""CPU oracle of the learned tracklet pre-filter: BF16 rounding and the
analytic gradient (finite differences), before it is used to check the GPU
kernels."""
import numpy as np

from oracle import mlp


def test_bf16_round_to_nearest_even():
    v = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, 1.0 + 2.0 ** -9, -2.5, 0.0, 3.0e38], np.float32)
    r = mlp.bf16(v)
    assert r[0] == 1.0
    assert r[1] == 1.0                   # tie -> even
    assert r[2] == 1.0 + 2.0 ** -6       # tie -> even (up)
    assert r[3] == 1.0                   # below half an ulp
    assert r[4] == -2.5 and r[5] == 0.0
    assert np.isfinite(r[6])
    # idempotent, and 8 significant bits
    assert np.array_equal(mlp.bf16(r), r)
    x = np.random.default_rng(0).normal(size=1000).astype(np.float32)
    assert np.all(np.abs(mlp.bf16(x) - x) <= np.abs(x) * 2.0 ** -8)


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    p = mlp.init_params(3).astype(np.float64)
    x = rng.normal(size=(40, mlp.N_IN))
    y = (rng.random(40) < 0.3).astype(np.float64)
    w = rng.uniform(0.5, 2.0, 40)
    _, g = mlp.loss_and_grad(p, x, y, w, exact=True)
    idx = np.concatenate([rng.choice(np.arange(mlp.W1, mlp.B1), 20), rng.choice(np.arange(mlp.W2, mlp.B2), 30),
                          np.arange(mlp.B2, mlp.B2 + 5), np.arange(mlp.W3, mlp.W3 + 5), [mlp.B3],
                          np.arange(mlp.B1, mlp.B1 + 5)])
    h = 1e-6
    for k in idx:
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (mlp.loss_and_grad(pp, x, y, w, exact=True)[0] - mlp.loss_and_grad(pm, x, y, w, exact=True)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 + 1e-4 * abs(g[k]), (k, fd, g[k])


def test_rounded_forward_close_to_exact():
    p = mlp.init_params(5)
    x = np.random.default_rng(2).normal(size=(500, mlp.N_IN)).astype(np.float32)
    z0, _ = mlp.forward(p, x, exact=True)
    z1, _ = mlp.forward(p, x)
    assert np.max(np.abs(z1 - z0)) < 0.05 * (1 + np.max(np.abs(z0)))
