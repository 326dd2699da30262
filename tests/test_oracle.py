"""The oracle restatement pinned against fixtures produced by the reference's
own CPU code (tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import fp64
from oracle import reference_numpy as R


@pytest.mark.parametrize("name", ["kde16_seed1", "kde16_seed11", "kde16_plain_4096x1024"])
def test_kde_nd_matches_reference(golden, name):
    g = golden(name)
    out = R.kde_eval_nd_numpy(g["queries"], g["train"], float(g["h"]))
    assert rel_err(out, g["density"]).max() < 2e-6


@pytest.mark.parametrize("name", ["kde16_lin_seed5", "kde16_lin_seed7"])
def test_kde_nd_linearized_matches_reference(golden, name):
    g = golden(name)
    out = R.kde_eval_nd_linearized_numpy(g["queries"], g["train"], float(g["h"]))
    np.testing.assert_allclose(out, g["density"], rtol=2e-6, atol=1e-12)


def test_kde_1d_matches_reference(golden):
    g = golden("kde1d_seed0")
    np.testing.assert_allclose(R.kde_eval_1d_numpy(g["queries"], g["train"], float(g["h"])), g["density"], rtol=1e-6)
    g = golden("kde1d_lin_seed6")
    np.testing.assert_allclose(R.kde_eval_1d_numpy(g["queries"], g["train"], float(g["h"]), laplace=True),
                               g["density"], rtol=1e-6, atol=1e-9)


@pytest.mark.parametrize("seed", [2, 3, 4, 10])
def test_empirical_score_matches_reference(golden, seed):
    g = golden(f"score16_seed{seed}")
    pdf, w, score = R.empirical_score_nd_numpy(g["train"], float(g["h"]))
    np.testing.assert_allclose(pdf, g["pdf_sum"], rtol=2e-6)
    np.testing.assert_allclose(w, g["weighted"], rtol=2e-5, atol=2e-5)
    deb = R.empirical_sd_kde_transform_nd_numpy(g["train"], float(g["h"]))
    np.testing.assert_allclose(deb, g["debiased"], rtol=1e-5, atol=1e-5)


def test_silverman_matches_reference(golden):
    g = golden("kde16_plain_4096x1024")
    assert R.silverman_bandwidth_nd(g["train"]) == pytest.approx(float(g["h"]), rel=1e-12)
    s = golden("silverman_seed13")
    assert R.silverman_bandwidth_nd(s["data"]) == pytest.approx(float(s["h_nd"]), rel=1e-12)
    assert R.silverman_bandwidth(s["data"][:, 3]) == pytest.approx(float(s["h_1d"]), rel=1e-12)
    assert fp64.silverman_nd(g["train"]) == pytest.approx(float(g["silverman_fp64"]), rel=1e-12)


def test_kde_score_1d_matches_reference(golden):
    g = golden("kde1d_score_seed12")
    score, pdf, _ = R.kde_score_1d(g["queries"], g["train"], float(g["h"]))
    np.testing.assert_allclose(pdf, g["pdf"], rtol=1e-5)
    np.testing.assert_allclose(score, g["score"], rtol=1e-4, atol=1e-4)
    assert R.sdkde_1d_bandwidth(g["mixture"]) == pytest.approx(float(g["h_sdkde"]), rel=1e-6)


def test_fp64_oracle_matches_reference_fp64(golden):
    g = golden("kde16_plain_4096x1024")
    lp = fp64.log_density(g["train"], g["queries"], float(g["h"]))
    np.testing.assert_allclose(lp, g["log_density_fp64"], rtol=1e-12, atol=1e-10)
    # and the reference's FP32 path is within 1e-5 of it (documented oracle fidelity)
    assert rel_err(g["density"], np.exp(g["log_density_fp64"])).max() < 1e-5


def test_fp64_laplace_matches_fp32_oracle(golden):
    g = golden("kde16_lin_seed5")
    d64 = fp64.density(g["train"], g["queries"], float(g["h"]), laplace=True)
    np.testing.assert_allclose(d64, np.abs(g["density"]), rtol=1e-4)


def test_fp64_gemm_oracle_matches_direct_differences():
    """The FP64 expansion-about-the-mean oracle used at full sizes agrees with
    the direct-difference FP64 oracle on offset heavy-tailed data (the
    cancellation-stress distribution) to ~1e-11 in log p."""
    from fsk import workloads

    x = workloads.student_t_16d(6000, seed=4)
    q = workloads.student_t_16d(200, seed=5)
    for h in (0.3, 1.0, 3.0):
        a = fp64.log_density(x, q, h)
        b = fp64.log_density_gemm(x, q, h, s_chunk=1000, q_chunk=64, threads=2)
        ok = np.isfinite(a)
        assert ok.all() == np.isfinite(b).all()
        assert np.abs(a[ok] - b[ok]).max() < 1e-10


def test_log_error_metrics():
    ref = np.array([-1.0, -2.0, -3.0, -np.inf])
    got = np.array([-1.0 + 1e-6, -2.0 - 2e-6, -3.0, -5.0])
    m = fp64.log_error_metrics(got, ref)
    assert m["finite_fraction"] == 1.0 and m["finite_fraction_ref"] == 0.75
    assert abs(m["max_abs_log_err"] - 2e-6) < 1e-12
    assert abs(m["mean_abs_log_err"] - 1e-6) < 1e-12
    assert abs(m["bias_log_err"] - (-1e-6 / 3)) < 1e-12


def test_timed_cpu_baseline_tiles_match_oracle():
    """The timed CPU baseline's tiled blocks compute the oracle's sums (FP32
    tolerance: only the grouping of the sums differs)."""
    from oracle import cpu_baseline as C

    rng = np.random.default_rng(5)
    n = 3 * C.COL_BLOCK + 77          # ragged last column tile
    x = rng.standard_normal((n, 16)).astype(np.float32)
    q = (rng.standard_normal((40, 16)) * 0.8).astype(np.float32)
    h = 0.9
    xn = (x * x).sum(axis=1)
    pdf, w = C._score_block(x, xn, 10, 50, h)
    pdf_ref, w_ref, _ = R.empirical_score_nd_numpy(x, h)
    np.testing.assert_allclose(pdf, pdf_ref[10:50], rtol=2e-5)
    np.testing.assert_allclose(w, w_ref[10:50], rtol=2e-4, atol=2e-4 * np.abs(w_ref[10:50]).max())
    norm = 1.0 / ((2.0 * np.pi) ** 8 * h ** 16 * n)
    np.testing.assert_allclose(norm * C._kde_block(x, xn, q, h), R.kde_eval_nd_numpy(q, x, h), rtol=2e-5)


def test_error_suite_smoke_configuration_oracle():
    """The reference's error-suite smoke run on the CPU (its fallback without
    CUDA): the FP64 log-space oracle gives finite log-densities for every test
    query of the 4-component diagonal mixture."""
    from fsk import workloads

    train, test = workloads.gm_diag_16d()
    assert train.shape == (8192, 16) and test.shape == (4096, 16)
    np.testing.assert_allclose(train.mean(axis=0), 0.0, atol=1e-5)
    np.testing.assert_allclose(train.std(axis=0, ddof=1), 1.0, rtol=1e-5)
    h = fp64.silverman_nd(train)
    ref = fp64.log_density(train, test, h)
    m = fp64.log_error_metrics(ref, ref)
    assert m["finite_fraction"] == 1.0 and m["max_abs_log_err"] == 0.0
    assert np.all(ref < 0) and np.all(ref > -200)
