"""The surrogate MLP oracle (oracle/mlp.py) against finite differences and
hand-checkable cases.  The reference has no surrogate, so these checks are
what pins the oracle (parity against the reference: unpinned)."""
import numpy as np

from oracle import mlp


def _setup(seed=0, batch=6):
    rng = np.random.default_rng(seed)
    p = mlp.init_params(rng).astype(np.float64)
    x = rng.standard_normal((batch, mlp.IN)) * 2.0 + 1.0
    mean = rng.standard_normal(mlp.IN) * 0.5
    istd = rng.uniform(0.5, 1.5, mlp.IN)
    return rng, p, x, mean, istd


def test_param_count_and_layout():
    assert mlp.N_PARAMS == 256 * 16 + 256 + 2 * (256 * 256 + 256) + 256 + 1 == 136193
    P = mlp.unpack(np.arange(mlp.N_PARAMS, dtype=np.float64))
    assert P["W1"].shape == (256, 16) and P["W1"][0, 1] == 1
    assert P["b4"][0] == mlp.N_PARAMS - 1


def test_bf16_rounding_ties_to_even():
    vals = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -7, -2.5, 3.0e-39], np.float32)
    r = mlp.bf16(vals)
    assert r[0] == 1.0
    assert r[1] == 1.0                      # halfway, even mantissa kept
    assert r[2] == np.float32(1.0 + 2 ** -6)  # halfway, rounds to even (up)
    assert r[3] == np.float32(1.0 + 2 ** -7)
    assert r[4] == -2.5
    assert np.all(mlp.bf16(r) == r)


def test_backward_matches_finite_differences():
    rng, p, x, mean, istd = _setup()
    y, cache = mlp.forward(p, x, mean, istd, quantize=False)
    dy = rng.standard_normal(x.shape[0])
    g = mlp.backward(cache, dy)
    idx = np.concatenate([rng.choice(mlp.N_PARAMS, 40, replace=False), [mlp.N_PARAMS - 1, 0, 4096, 70000]])
    for i in idx:
        e = 1e-5
        pp = p.copy(); pp[i] += e
        pm = p.copy(); pm[i] -= e
        fd = ((mlp.forward(pp, x, mean, istd, quantize=False)[0] - mlp.forward(pm, x, mean, istd, quantize=False)[0])
              * dy).sum() / (2 * e)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_quantized_forward_close_to_exact():
    _, p, x, mean, istd = _setup(1, 32)
    yq, _ = mlp.forward(p, x, mean, istd, quantize=True)
    ye, _ = mlp.forward(p, x, mean, istd, quantize=False)
    assert np.abs(yq - ye).max() < 0.05 * (np.abs(ye).max() + 1)


def test_adam_first_step_is_signed_lr():
    g = np.array([0.5, -2.0, 0.0, 1e-3])
    p = np.ones(4)
    p1, m, v = mlp.adam(p, g, np.zeros(4), np.zeros(4), step=1, lr=0.1, eps=1e-12)
    # first bias-corrected step moves each coordinate by lr * sign(g)
    assert np.allclose(p1, [0.9, 1.1, 1.0, 0.9])
    p2, _, _ = mlp.adam(p, g, np.zeros(4), np.zeros(4), step=1, lr=0.1, eps=1e-12, weight_decay=0.5)
    assert np.allclose(p2, p1 - 0.05)
