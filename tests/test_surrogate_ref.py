"""The CPU reference of the surrogate network checks itself: its explicit
backward pass against central finite differences of its own float64 loss
(no bf16 rounding), on a random subset of parameters of every layer."""
import numpy as np

from oracle import surrogate_ref as R


def _params(seed):
    rng = np.random.default_rng(seed)
    parts = []
    for kind, ci, co, *_ in R.LAYERS:
        k = R._k(kind, ci)
        parts.append((rng.standard_normal((co, k)) * np.sqrt(2.0 / k), 0.05 * rng.standard_normal(co)))
    return R.join(parts)


def test_layer_table_size():
    assert R.param_count() == len(_params(0))
    assert 2.0e6 < R.param_count() < 2.6e6


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(1)
    p = _params(2)
    B = 1
    maps = rng.uniform(0, 1, (B, 64, 64, 2))
    sc = rng.uniform(0, 1, (B, 3))
    tgt = rng.standard_normal((B, 1024, 384)) * 0.1
    loss, g = R.loss_and_grads(p, maps, sc, tgt, bf16=False)
    # a few parameters of every layer (weights and biases)
    idx, q = [], 0
    for kind, ci, co, *_ in R.LAYERS:
        n = co * R._k(kind, ci) + co
        idx += list(q + rng.choice(n, 2, replace=False))
        q += n
    eps = 1e-5
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        fd = (R.loss_and_grads(pp, maps, sc, tgt, bf16=False)[0] - R.loss_and_grads(pm, maps, sc, tgt, bf16=False)[0]) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-4 * max(abs(fd), abs(g[i])) + 1e-10, (i, fd, g[i])


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 3.0e38], np.float32)
    r = R.to_bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == -2.5
