"""Learned surrogate kernels on the GPU against the oracle (oracle/mlp.py) and
against each other, plus the estimator's gate and exact fallback.

Tolerances: the kernels compute SiLU through tanh.approx (max relative error
~2^-11) while the oracle uses the exact sigmoid; with bf16 activations this
flips an occasional bf16 rounding, so forward values are compared at
1e-2 * (1 + |y|) and gradients at 3e-2 relative L2 norm.  Adam is FP32 vs
FP64 (1e-5 relative).  The tensor-core inference and the CUDA-core training
forward compute the same model in a different accumulation order:
1e-2 * (1 + |y|).
"""
import math

import numpy as np
import pytest
import torch

from oracle import mlp as O

pytestmark = pytest.mark.gpu


def _case(seed, batch, members):
    rng = np.random.default_rng(seed)
    params = np.concatenate([O.init_params(rng) for _ in range(members)])
    x = (rng.standard_normal((batch, 16)) * 3.0 + 1.0).astype(np.float32)
    mean = (rng.standard_normal(16) * 0.5).astype(np.float32)
    istd = rng.uniform(0.3, 0.6, 16).astype(np.float32)
    return rng, params, x, mean, istd


def _dev(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


@pytest.mark.parametrize("batch,members", [(200, 1), (1000, 4), (64, 2)])
def test_training_forward_matches_oracle(cuda_dev, batch, members):
    from fsk import ops

    _, params, x, mean, istd = _case(0, batch, members)
    P, X, M, S = (_dev(a, cuda_dev) for a in (params, x, mean, istd))
    ws = ops.mlp_train_workspace(members, batch, cuda_dev)
    y = ops.mlp_fwd(P, members, X, M, S, ws).cpu().numpy()
    for k in range(members):
        ref, _ = O.forward(params[k * O.N_PARAMS:(k + 1) * O.N_PARAMS], x, mean, istd, quantize=True)
        assert np.all(np.abs(y[k] - ref) <= 1e-2 * (1 + np.abs(ref))), np.abs(y[k] - ref).max()


def test_backward_matches_oracle(cuda_dev):
    from fsk import ops

    batch, members = 777, 2
    rng, params, x, mean, istd = _case(1, batch, members)
    dy = rng.standard_normal((members, batch)).astype(np.float32) / batch
    P, X, M, S, DY = (_dev(a, cuda_dev) for a in (params, x, mean, istd, dy))
    ws = ops.mlp_train_workspace(members, batch, cuda_dev)
    ops.mlp_fwd(P, members, X, M, S, ws)
    g = ops.mlp_bwd(P, members, batch, DY, ws).cpu().numpy()
    for k in range(members):
        pk = params[k * O.N_PARAMS:(k + 1) * O.N_PARAMS]
        _, cache = O.forward(pk, x, mean, istd, quantize=True)
        ref = O.backward(cache, dy[k].astype(np.float64))
        got = g[k * O.N_PARAMS:(k + 1) * O.N_PARAMS]
        for name, lo, hi in (("W1", 0, 4096), ("W2", 4352, 4352 + 65536), ("W3", 70144, 70144 + 65536),
                             ("w4", 135936, 136192), ("all", 0, O.N_PARAMS)):
            r = np.linalg.norm(got[lo:hi] - ref[lo:hi]) / np.linalg.norm(ref[lo:hi])
            assert r < 3e-2, (k, name, r)


def test_adam_matches_oracle(cuda_dev):
    from fsk import ops

    rng = np.random.default_rng(2)
    n = 5000
    p, g = rng.standard_normal(n).astype(np.float32), rng.standard_normal(n).astype(np.float32)
    m, v = (rng.standard_normal(n) * 0.1).astype(np.float32), rng.uniform(0, 0.1, n).astype(np.float32)
    P, G, Mt, Vt = (_dev(a, cuda_dev) for a in (p, g, m, v))
    ops.mlp_adam(P, G, Mt, Vt, step=7, lr=3e-3, weight_decay=0.01)
    # the kernel holds beta1, beta2 in FP32: give the oracle the same constants
    b1, b2 = float(np.float32(0.9)), float(np.float32(0.999))
    rp, rm, rv = O.adam(p, g, m, v, step=7, lr=3e-3, beta1=b1, beta2=b2, weight_decay=0.01)
    np.testing.assert_allclose(P.cpu().numpy(), rp, rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(Mt.cpu().numpy(), rm, rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(Vt.cpu().numpy(), rv, rtol=1e-5, atol=1e-9)


@pytest.mark.parametrize("batch", [1, 127, 129, 1000, 5000])
def test_tensor_core_inference_matches_training_forward(cuda_dev, batch):
    from fsk import ops

    members = 4
    _, params, x, mean, istd = _case(3, batch, members)
    P, X, M, S = (_dev(a, cuda_dev) for a in (params, x, mean, istd))
    ws = ops.mlp_train_workspace(members, batch, cuda_dev)
    y_train = ops.mlp_fwd(P, members, X, M, S, ws)
    packed = ops.mlp_pack(P, members, M, S, out_scale=2.0, out_shift=-1.5)
    y_inf = ops.mlp_infer(packed, members, X)
    ops.device_status(cuda_dev)
    a, b = y_inf.cpu().numpy(), (y_train * 2.0 - 1.5).cpu().numpy()
    assert np.all(np.isfinite(a))
    assert np.all(np.abs(a - b) <= 1e-2 * (1 + np.abs(b))), np.abs(a - b).max()


def test_combine_gate(cuda_dev):
    from fsk import ops

    rng = np.random.default_rng(4)
    members, batch = 3, 1000
    y = rng.standard_normal((members, batch)).astype(np.float32) * 0.02
    x = rng.standard_normal((batch, 16)).astype(np.float32) * 2
    mean = rng.standard_normal(16).astype(np.float32) * 0.1
    istd = rng.uniform(0.5, 1.0, 16).astype(np.float32)
    Y, X, M, S = (_dev(a, cuda_dev) for a in (y, x, mean, istd))
    mu, sp, served = ops.mlp_combine(Y, X, M, S, base_a=-3.0, base_b=-0.25, spread_tol=0.05, r2_max=20.0)
    r2 = (((x - mean) * istd) ** 2).sum(1)
    np.testing.assert_allclose(mu.cpu().numpy(), y.mean(0) - 3.0 - 0.25 * r2, rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(sp.cpu().numpy(), y.max(0) - y.min(0), rtol=1e-6, atol=1e-7)
    want = (y.max(0) - y.min(0) <= 0.05) & (r2 <= 20.0)
    got = served.cpu().numpy().astype(bool)
    # ties at the threshold may round either way
    assert np.mean(got == want) > 0.999 and want.any() and (~want).any()


def test_surrogate_learns_a_smooth_log_density(cuda_dev):
    """The training loop (own forward / backward / AdamW kernels) fits a smooth
    16-D log-density well: a Gaussian plus a product-of-sines ripple."""
    from flash_sd_kde.surrogate import SurrogateKDE

    g = torch.Generator(device=cuda_dev).manual_seed(3)
    def f(q):
        return -0.125 * (q * q).sum(1) + 0.5 * torch.sin(q[:, 0]) * torch.cos(0.7 * q[:, 1]) + 0.2 * q[:, 2]
    q = torch.randn((300_000, 16), generator=g, device=cuda_dev) * 2.0
    sur = SurrogateKDE(members=4, epochs=20, batch_size=4096, seed=2).fit(q[:1000], 1.0, queries=q, log_density=f(q))
    assert sur.history[-1] < 0.2 * sur.history[0]
    qt = torch.randn((50_000, 16), generator=g, device=cuda_dev) * 2.0
    mean, spread, served = sur.predict(qt)
    err = (mean - f(qt)).abs()
    assert float(err.median()) < 0.03, float(err.median())
    assert float(spread.median()) < 0.1


def test_surrogate_gate_and_exact_fallback(cuda_dev):
    """Mechanics of serving: queries the gate rejects get the exact KDE value
    (bit for bit that kernel's result for the same query set), served ones the
    ensemble mean; out-of-radius queries are never served."""
    from flash_sd_kde.surrogate import SurrogateKDE
    from fsk import ops, workloads

    x_np, _ = workloads.gmm8_16d(4096, 16)
    x = torch.from_numpy(x_np).to(cuda_dev)
    h = float(ops.silverman(x).item())
    sur = SurrogateKDE(members=4, epochs=2, batch_size=4096, spread_tol=0.5, seed=1).fit(x, h, n_pairs=100_000)
    g = torch.Generator(device=cuda_dev).manual_seed(9)
    idx = torch.randint(4096, (20000,), generator=g, device=cuda_dev)
    q_in = x[idx] + torch.randn((20000, 16), generator=g, device=cuda_dev) * h
    q_out = torch.randn((5000, 16), generator=g, device=cuda_dev) * 8.0
    q = torch.cat([q_in, q_out]).contiguous()
    logp, served = sur.score_samples(q, return_served=True)
    mean, spread, served2 = sur.predict(q)
    exact = sur._exact_logp(q)
    ops.device_status(cuda_dev)
    miss = ~served
    assert miss.any() and served.any()
    assert torch.equal(served, served2.bool())
    assert torch.equal(logp[served], mean[served])
    assert torch.equal(logp[miss], sur._exact_logp(q[miss].contiguous()))
    # far queries may underflow the FP32 kernel sum to log 0 = -inf on both sides
    fin = torch.isfinite(exact) & miss
    assert torch.equal(torch.isinf(logp[miss]), torch.isinf(exact[miss]))
    assert float((logp[fin] - exact[fin]).abs().max()) < 1e-4
    r2 = sur._radius2(q)
    assert not bool(served[r2 > sur.r2_max_].any())
    assert bool((spread[served] <= sur.spread_tol).all())


def test_surrogate_checkpoint_and_resume(cuda_dev, tmp_path):
    """save / load / resume: a loaded surrogate serves bit-identical values;
    resuming continues the step count and the AdamW state on the same
    (regenerated) training pairs, from the original and from the loaded copy
    alike; a surrogate fitted on given queries refuses to resume without
    them."""
    from flash_sd_kde.surrogate import SurrogateKDE
    from fsk import ops, workloads

    x_np, _ = workloads.gmm8_16d(4096, 16)
    x = torch.from_numpy(x_np).to(cuda_dev)
    h = float(ops.silverman(x).item())
    sur = SurrogateKDE(members=2, epochs=2, batch_size=4096, spread_tol=0.5, seed=4).fit(x, h, n_pairs=65536)
    steps = sur.step_
    assert steps == 2 * (65536 // 4096) and sur.total_steps_ == steps
    path = tmp_path / "sur.pt"
    sur.save(path)
    back = SurrogateKDE.load(path, device=cuda_dev)
    g = torch.Generator(device=cuda_dev).manual_seed(11)
    q = (x[torch.randint(4096, (5000,), generator=g, device=cuda_dev)]
         + torch.randn((5000, 16), generator=g, device=cuda_dev) * h).contiguous()
    for a, b in zip(sur.predict(q), back.predict(q)):
        assert torch.equal(a, b)
    assert torch.equal(sur.score_samples(q), back.score_samples(q))
    assert torch.equal(back.adam_m_, sur.adam_m_) and torch.equal(back.adam_v_, sur.adam_v_)
    assert back.history == sur.history and back.r2_max_ == sur.r2_max_
    sur.resume(2)
    back.resume(2)
    ops.device_status(cuda_dev)
    assert sur.step_ == back.step_ == 2 * steps and len(sur.history) == len(back.history) == 4
    # the same pairs in the same order from the same state: equal up to the order of the
    # weight-gradient atomics
    np.testing.assert_allclose(back.history, sur.history, rtol=2e-2)
    assert sur.history[3] < sur.history[0]
    assert not torch.equal(back.params_, SurrogateKDE.load(path, device=cuda_dev).params_)
    given = SurrogateKDE(members=2, epochs=1, batch_size=4096, seed=4).fit(x, h, queries=q,
                                                                          log_density=sur._exact_logp(q))
    with pytest.raises(ValueError):
        given.resume(1)
    given.resume(1, queries=q, log_density=sur._exact_logp(q))
    assert given.step_ == 2 * (5000 // 4096)
    with pytest.raises(ValueError):
        torch.save({"format": "other"}, tmp_path / "bad.pt")
        SurrogateKDE.load(tmp_path / "bad.pt", device=cuda_dev)


def test_surrogate_gain_over_exact_only(cuda_dev):
    """What the trained network gains over the method without it, on the
    learned-surrogate configuration (exact SD-KDE of 262144 8-component
    mixture points; training queries = data + N(0, h^2 I); held-out queries
    half the same recipe, half N(0, 9 I)), with a shorter training run:
    surrogate + exact fallback against exact-only on the same queries.
    * Every query the gate rejects carries the exact value (bit for bit).
    * The surrogate path answers a query at least 10x faster than the exact
      kernel (one query against 262144 points).
    * At the spread tolerance 0.3 the gate serves a measurable part of the
      in-support queries, never an out-of-radius one, and the served
      queries' median relative density error stays under 20 % (the full
      bench training reaches ~5-7 % along its whole frontier); the exact
      path's own error on them is ~1e-6.  The spec's 1 % target is out of
      reach for a smooth model of this KDE: at the median the single largest
      kernel term carries ~10 % of a held-out query's density."""
    from flash_sd_kde import emp_sd_kde_fit_transform
    from flash_sd_kde.surrogate import SurrogateKDE
    from fsk import ops, workloads

    gmm = workloads.GMM16(seed=0)
    x = torch.from_numpy(gmm.sample(262144, seed=1)).to(cuda_dev)
    h = float(ops.silverman(x).item())
    deb = emp_sd_kde_fit_transform(x, h, device=cuda_dev)
    sur = SurrogateKDE(members=4, epochs=4, spread_tol=0.3, seed=0).fit(deb, h, n_pairs=1_000_000)
    g = torch.Generator(device=cuda_dev).manual_seed(123)
    half = 100_000
    idx = torch.randint(deb.shape[0], (half,), generator=g, device=cuda_dev)
    q_in = deb[idx] + torch.randn((half, 16), generator=g, device=cuda_dev) * h
    q_out = torch.randn((half, 16), generator=g, device=cuda_dev) * 3.0
    q = torch.cat([q_in, q_out]).contiguous()

    def timed(fn):
        fn()
        torch.cuda.synchronize(cuda_dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        out = fn()
        e1.record()
        torch.cuda.synchronize(cuda_dev)
        return e0.elapsed_time(e1), out

    ms_exact, exact = timed(lambda: sur._exact_logp(q))
    ms_sur, (mean, spread, served) = timed(lambda: sur.predict(q))
    logp, served_g = sur.score_samples(q, return_served=True)
    ops.device_status(cuda_dev)
    assert ms_exact / ms_sur >= 10.0, (ms_exact, ms_sur)
    miss = ~served_g
    # fallback queries carry the exact kernel's value for that query set (its
    # split plan depends on the batch size, so compare with the same subset),
    # and that value agrees with the full batch's to FP32 summation order
    assert torch.equal(logp[miss], sur._exact_logp(q[miss].contiguous()))
    assert float(((logp[miss] - exact[miss]) / exact[miss]).abs().max()) < 1e-6
    assert torch.equal(logp[served_g], mean[served_g])
    assert not bool(served_g[sur._radius2(q) > sur.r2_max_].any())
    frac_in = float(served_g[:half].float().mean())
    rel = (torch.exp((logp - exact).double()) - 1).abs()
    assert frac_in > 0.05, frac_in
    med = float(rel[served_g].median())
    assert med < 0.2, med
