"""Feature counts other than 16 through the public API against the FP64
oracle: 1 <= d <= 16 zero-padded to 16 on the device (tensor-core kernels),
16 < d <= 64 on the CUDA-core kernels for any d; KDE in both precision modes,
the Laplace-corrected KDE, the SD-KDE debias shift and the estimator end to
end.  Tolerances as for 16-D: densities 1e-5 relative, debiased points 1e-5
relative with a 1e-5 * max|x| floor."""
import numpy as np
import pytest
import torch

from conftest import rel_err
from oracle import fp64

pytestmark = pytest.mark.gpu


def _data(d, n, m, seed):
    rng = np.random.default_rng(seed)
    scale = rng.uniform(0.5, 2.0, d)
    x = (rng.standard_normal((n, d)) * scale).astype(np.float32)
    q = (x[rng.integers(0, n, m)] + 0.5 * rng.standard_normal((m, d)) * scale).astype(np.float32)
    return x, q


@pytest.mark.parametrize("precision", ["fast_tf32", "fp32_ieee"])
@pytest.mark.parametrize("d", [2, 5, 15])
def test_kde_eval_general_d(cuda_dev, d, precision):
    from flash_sd_kde import kde_eval

    x, q = _data(d, 3000, 400, d)
    h = fp64.silverman_nd(x)
    out = kde_eval(torch.from_numpy(x).to(cuda_dev), torch.from_numpy(q).to(cuda_dev), h, device=cuda_dev,
                   precision_mode=precision).cpu().numpy()
    truth = np.exp(fp64.log_density(x, q, h))
    assert rel_err(out, truth).max() < 1e-5


@pytest.mark.parametrize("backend", ["flash_sd_kde", "ordered_splitk", "symmetric_atomic"])
def test_sd_kde_general_d(cuda_dev, backend):
    from flash_sd_kde import emp_sd_kde_fit_transform

    x, _ = _data(7, 2500, 1, 11)
    h = fp64.silverman_nd(x)
    deb, pdf, w, score = emp_sd_kde_fit_transform(torch.from_numpy(x).to(cuda_dev), h, device=cuda_dev,
                                                  emp_score_backend=backend, return_debug=True)
    p64, w64, s64 = fp64.empirical_score(x, h)
    assert deb.shape == (2500, 7) and w.shape == (2500, 7) and score.shape == (2500, 7)
    np.testing.assert_allclose(pdf.cpu().numpy(), p64, rtol=1e-5)
    np.testing.assert_allclose(w.cpu().numpy(), w64, rtol=1e-5, atol=1e-5 * np.abs(w64).max())
    d64 = fp64.debias(x, h)
    np.testing.assert_allclose(deb.cpu().numpy(), d64, rtol=1e-5, atol=1e-5 * np.abs(d64).max())


@pytest.mark.parametrize("mode", ["sd_kde", "kde"])
def test_estimator_general_d(cuda_dev, mode):
    from flash_sd_kde import FlashSDKDE

    x, q = _data(8, 2000, 300, 5)
    est = FlashSDKDE(mode=mode, device=cuda_dev).fit(x)
    h = est.bandwidth_
    assert abs(h - fp64.silverman_nd(x)) <= 1e-6 * h
    fit = fp64.debias(x, h) if mode == "sd_kde" else x
    ref = np.log(np.exp(fp64.log_density(fit, q, h)) + est.eps)   # score_samples: log(p + eps)
    out = est.score_samples(q)
    assert out.shape == (300,)
    assert (np.abs(out - ref) / np.abs(ref)).max() < 1e-5


@pytest.mark.parametrize("d", [17, 40, 64])
def test_kde_eval_above_16(cuda_dev, d):
    """d > 16: the CUDA-core kernels for any d (both precision modes take them)."""
    from flash_sd_kde import kde_eval

    x, q = _data(d, 2000, 300, d)
    h = fp64.silverman_nd(x)
    truth = np.exp(fp64.log_density(x, q, h))
    for precision in ("fast_tf32", "fp32_ieee"):
        out = kde_eval(torch.from_numpy(x).to(cuda_dev), torch.from_numpy(q).to(cuda_dev), h, device=cuda_dev,
                       precision_mode=precision).cpu().numpy()
        assert rel_err(out, truth).max() < 1e-5, (precision, rel_err(out, truth).max())


@pytest.mark.parametrize("d", [5, 33])
def test_laplace_general_d(cuda_dev, d):
    """Laplace-corrected KDE with the factor 1 + d/2 - dist/(2h^2) of the data's d."""
    from flash_sd_kde import kde_eval_linearized

    x, q = _data(d, 1500, 200, 3 + d)
    h = 1.5 * fp64.silverman_nd(x)
    out = kde_eval_linearized(torch.from_numpy(x).to(cuda_dev), torch.from_numpy(q).to(cuda_dev), h,
                              device=cuda_dev).cpu().numpy().astype(np.float64)
    truth = np.exp(fp64.log_density(x, q, h, laplace=True))   # |sum phi (1 + d/2 - dist/(2h^2))| / norm
    big = np.abs(out) > 1e-3 * np.abs(out).max()             # the corrected sum cancels elsewhere
    assert rel_err(np.abs(out[big]), truth[big]).max() < 1e-4


def test_sd_kde_above_16(cuda_dev):
    from flash_sd_kde import FlashSDKDE, emp_sd_kde_fit_transform

    x, q = _data(24, 1500, 200, 24)
    h = fp64.silverman_nd(x)
    deb, pdf, w, score = emp_sd_kde_fit_transform(torch.from_numpy(x).to(cuda_dev), h, device=cuda_dev,
                                                  return_debug=True)
    p64, w64, _ = fp64.empirical_score(x, h)
    assert deb.shape == (1500, 24) and w.shape == (1500, 24)
    np.testing.assert_allclose(pdf.cpu().numpy(), p64, rtol=1e-5)
    np.testing.assert_allclose(w.cpu().numpy(), w64, rtol=1e-5, atol=1e-5 * np.abs(w64).max())
    d64 = fp64.debias(x, h)
    np.testing.assert_allclose(deb.cpu().numpy(), d64, rtol=1e-5, atol=1e-5 * np.abs(d64).max())
    est = FlashSDKDE(mode="sd_kde", bandwidth=h, device=cuda_dev).fit(x)
    ref = np.log(np.exp(fp64.log_density(d64, q, h)) + est.eps)
    assert (np.abs(est.score_samples(q) - ref) / np.abs(ref)).max() < 1e-5


def test_general_d_argument_errors(cuda_dev):
    from flash_sd_kde import FlashSDKDE, kde_eval
    from flash_sd_kde.kde import kde_eval_log

    x5 = np.zeros((10, 5), np.float32)
    with pytest.raises(ValueError):
        kde_eval(x5, np.zeros((3, 6), np.float32), 1.0, device=cuda_dev)
    with pytest.raises(ValueError):
        kde_eval(np.zeros((10, 65), np.float32), np.zeros((3, 65), np.float32), 1.0, device=cuda_dev)
    with pytest.raises(ValueError):   # exact log output: up to 16 features
        kde_eval_log(np.zeros((10, 20), np.float32), np.zeros((3, 20), np.float32), 1.0, eps=0.0, device=cuda_dev)
    with pytest.raises(ValueError):
        FlashSDKDE(mode="sd_kde", device=cuda_dev).fit(np.random.default_rng(0).standard_normal((50, 65)))


@pytest.mark.parametrize("d", [17, 64])
@pytest.mark.parametrize("m,n", [(1, 1), (3, 33), (130, 31), (257, 65)])
def test_any_d_ragged_shapes(cuda_dev, d, m, n):
    """Any-d kernels at tiny and ragged sizes (partial 32-point tiles, one
    query, one point): KDE, empirical score and debias vs FP64."""
    from fsk import ops

    rng = np.random.default_rng(d * 1000 + m * 7 + n)
    x = rng.standard_normal((n, d)).astype(np.float32)
    q = (x[rng.integers(0, n, m)] + 0.3 * rng.standard_normal((m, d))).astype(np.float32)
    h = 1.2
    out = ops.kde_nd_sum(torch.from_numpy(q).to(cuda_dev), torch.from_numpy(x).to(cuda_dev), h).cpu().numpy()
    ref = np.exp(fp64.log_density(x, q, h)) * ((2.0 * np.pi) ** (d / 2.0) * h ** d * n)   # unnormalised sums
    assert rel_err(out, ref).max() < 1e-5
    pdf, w = ops.empscore_nd(torch.from_numpy(x).to(cuda_dev), h)
    deb = ops.debias_nd(torch.from_numpy(x).to(cuda_dev), pdf, w, h, 1e-12)
    ops.device_status(cuda_dev)
    p64, w64, _ = fp64.empirical_score(x, h)
    np.testing.assert_allclose(pdf.cpu().numpy(), p64, rtol=1e-5)
    np.testing.assert_allclose(w.cpu().numpy(), w64, rtol=1e-5, atol=1e-5 * np.abs(w64).max())
    d64 = fp64.debias(x, h)
    np.testing.assert_allclose(deb.cpu().numpy(), d64, rtol=1e-5, atol=1e-5 * np.abs(d64).max())
