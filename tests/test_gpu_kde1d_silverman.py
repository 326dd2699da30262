"""1-D KDE / KDE score, the 1-D SD-KDE step and the GPU Silverman rules.

Tolerances: 1-D densities 1e-5 relative to the reference outputs and FP64;
1-D score 1e-4 (the reference's own score is FP32 deriv/pdf); bandwidths
1e-12 relative to the FP64-statistics rule and 1e-6 to the reference's
float32 statistics.
"""
import numpy as np
import pytest
import torch

from conftest import rel_err
from oracle import fp64
from oracle import reference_numpy as R

pytestmark = pytest.mark.gpu


def test_kde1d_vs_reference(cuda_dev, golden):
    from flash_sd_kde import kde_eval, kde_eval_linearized

    g = golden("kde1d_seed0")
    out = kde_eval(g["train"], g["queries"], float(g["h"]), device="cuda").cpu().numpy()
    assert rel_err(out, g["density"]).max() < 1e-5
    assert rel_err(out, fp64.density(g["train"], g["queries"], float(g["h"]))).max() < 1e-5
    g = golden("kde1d_lin_seed6")
    lin = kde_eval_linearized(g["train"], g["queries"], float(g["h"]), device="cuda").cpu().numpy()
    np.testing.assert_allclose(lin, g["density"], rtol=1e-5, atol=1e-6)


def test_kde1d_atomic_matches_splitk(cuda_dev):
    from flash_sd_kde import kde_eval
    from fsk import workloads

    x = workloads.gmm3_1d(100_000, seed=1)
    q = workloads.grid_1d(4097)
    a = kde_eval(x, q, 0.05, kde_backend="splitk_stream").cpu().numpy()
    b = kde_eval(x, q, 0.05, kde_backend="atomic").cpu().numpy()
    assert rel_err(b, a).max() < 1e-6
    ref = R.kde_eval_1d_numpy(q[::64], x, 0.05)
    assert rel_err(a[::64], ref).max() < 1e-5


def test_kde1d_score_vs_reference(cuda_dev, golden):
    from kernels.flash_sd_kde import gaussian_kde_score_triton

    g = golden("kde1d_score_seed12")
    score, pdf, deriv = gaussian_kde_score_triton(g["train"], g["queries"], float(g["h"]))
    assert rel_err(pdf.cpu().numpy(), g["pdf"]).max() < 1e-5
    np.testing.assert_allclose(score.cpu().numpy(), g["score"], rtol=1e-4, atol=1e-4)


def test_sdkde_1d_vs_reference(cuda_dev, golden):
    from kernels.flash_sd_kde import empirical_sd_kde_triton

    g = golden("kde1d_score_seed12")
    deb, h = empirical_sd_kde_triton(g["mixture"])
    assert h == pytest.approx(float(g["h_sdkde"]), rel=1e-6)
    np.testing.assert_allclose(deb, g["debiased_1d"], rtol=1e-5, atol=1e-5)


def test_silverman_gpu(cuda_dev, golden):
    from flash_sd_kde.reference import silverman_bandwidth, silverman_bandwidth_nd

    g = golden("kde16_plain_4096x1024")
    assert silverman_bandwidth_nd(g["train"]) == pytest.approx(float(g["silverman_fp64"]), rel=1e-12)
    assert silverman_bandwidth_nd(g["train"]) == pytest.approx(float(g["h"]), rel=1e-6)
    s = golden("silverman_seed13")
    assert silverman_bandwidth_nd(s["data"]) == pytest.approx(fp64.silverman_nd(s["data"]), rel=1e-12)
    assert silverman_bandwidth_nd(s["data"]) == pytest.approx(float(s["h_nd"]), rel=1e-6)
    assert silverman_bandwidth(s["data"][:, 3]) == pytest.approx(float(s["h_1d"]), rel=1e-6)
    # ties, tiny and odd sizes
    for arr in (np.ones((5, 16), np.float32), np.arange(7, dtype=np.float32)[:, None].repeat(16, 1),
                np.random.default_rng(3).standard_normal((1, 16)).astype(np.float32)):
        assert silverman_bandwidth_nd(arr) == pytest.approx(fp64.silverman_nd(arr), rel=1e-12)
