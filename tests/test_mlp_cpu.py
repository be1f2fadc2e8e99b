"""The MLP oracle's gradient against finite differences of its own loss
(float64, no BF16 rounding), so the GPU gradient check compares against a
verified reference."""
import numpy as np

from oracle import mlp_oracle as mo


def _problem(C=7, n=5, seed=0):
    rng = np.random.default_rng(seed)
    nparam = C * 16 + 22 * 64 + 64 + 64 * 64 + 64 + 64 * C + C
    p = (rng.standard_normal(nparam) * 0.3).astype(np.float64)
    s = np.zeros(n, mo.SAMPLE_DTYPE)
    s["origin"] = rng.uniform(-1, 1, (n, 3))
    s["dir"] = rng.uniform(-1, 1, (n, 3))
    s["current"] = rng.integers(0, C, n)
    s["target"] = rng.integers(0, C, n)
    return p, s, C


def test_oracle_gradient_matches_finite_differences():
    p, s, C = _problem()
    loss, g = mo.loss_and_grad(p, s, C, round_bf16=False)
    rng = np.random.default_rng(1)
    idx = rng.choice(len(p), 60, replace=False)
    idx = np.concatenate([idx, np.arange(0, 16 * C, 9)])  # embedding rows too
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (mo.loss_and_grad(pp, s, C, round_bf16=False)[0] - mo.loss_and_grad(pm, s, C, round_bf16=False)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_bf16_rounding_ties_to_even():
    x = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e38, 1.5e-30], np.float32)
    r = mo.bf16_round(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125 and r[3] == -2.5
    assert np.all(np.abs(r - x) <= np.abs(x) * 2.0 ** -8)  # normal values: half a BF16 ulp
