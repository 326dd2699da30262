"""FlashSDKDE (fit / score_samples / score) end to end on the GPU.

Tolerances: mode="kde" log densities within 1e-5 absolute of
log(reference density + 1e-12); mode="sd_kde" log(p + 1e-12) within 1e-5
relative of the FP64 pipeline (FP64 debias, then FP64 log-space KDE), and the
densities themselves within 1e-4 (the FP32 debiased points carry ~1e-7
relative rounding that the FP64 pipeline does not).
"""
import numpy as np
import pytest

from oracle import fp64

pytestmark = pytest.mark.gpu


def test_kde_mode_16d(cuda_dev, golden):
    from flash_sd_kde import FlashSDKDE

    g = golden("kde16_plain_4096x1024")
    est = FlashSDKDE(mode="kde", bandwidth="silverman").fit(g["train"])
    assert est.bandwidth_ == pytest.approx(float(g["h"]), rel=1e-6)
    lp = est.score_samples(g["queries"])
    assert lp.dtype == np.float32 and lp.shape == (1024,)
    np.testing.assert_allclose(lp, np.log(g["density"].astype(np.float64) + 1e-12), atol=1e-5, rtol=0)
    assert est.score(g["queries"]) == pytest.approx(float(np.mean(lp)), rel=1e-6)


def test_kde_mode_1d(cuda_dev, golden):
    from flash_sd_kde import FlashSDKDE

    g = golden("kde1d_seed0")
    est = FlashSDKDE(mode="kde", bandwidth=float(g["h"])).fit(g["train"][:, None])
    lp = est.score_samples(g["queries"][:, None])
    np.testing.assert_allclose(lp, np.log(g["density"].astype(np.float64) + 1e-12), atol=1e-5, rtol=0)


def test_sd_kde_mode_vs_fp64_pipeline(cuda_dev):
    from flash_sd_kde import FlashSDKDE
    from fsk import workloads

    g = workloads.GMM16(seed=0)
    x = g.sample(4096, seed=1)
    q = g.sample(512, seed=2)
    est = FlashSDKDE(mode="sd_kde").fit(x)
    lp = est.score_samples(q).astype(np.float64)
    h = est.bandwidth_
    deb = fp64.debias(x, h)
    logp = fp64.log_density(deb, q, h)
    ref = np.log(np.exp(logp) + est.eps)       # score_samples returns log(p + eps)
    rel = np.abs(lp - ref) / np.abs(ref)
    assert rel.max() < 1e-5, rel.max()
    # the densities themselves (no eps floor) through kde_eval
    from flash_sd_kde import kde_eval

    dens = kde_eval(est._fit_eval_data, q, h).cpu().numpy().astype(np.float64)
    assert (np.abs(dens - np.exp(logp)) / np.exp(logp)).max() < 1e-4


def test_errors(cuda_dev):
    from flash_sd_kde import FlashSDKDE

    with pytest.raises(ValueError):
        FlashSDKDE().score_samples(np.zeros((3, 16), np.float32))
    with pytest.raises(ValueError):   # at most 64 features
        FlashSDKDE(mode="sd_kde").fit(np.zeros((10, 65), np.float32))
    with pytest.raises(ValueError):
        FlashSDKDE(mode="bogus").fit(np.zeros((10, 16), np.float32))
    est = FlashSDKDE(mode="kde", bandwidth=1.0).fit(np.zeros((10, 16), np.float32))
    with pytest.raises(ValueError):
        est.score_samples(np.zeros((3, 4), np.float32))
