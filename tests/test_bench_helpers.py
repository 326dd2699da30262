"""bench.py's own FP64 spot checks agree with the oracle (CPU only): the
bench reports its errors against FP64 with self-contained functions, so they
are pinned here to the oracle's FP64 log-space reference and score rows."""
import importlib.util
import sys
from pathlib import Path

import numpy as np

from oracle import fp64

ROOT = Path(__file__).resolve().parent.parent


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    argv, sys.argv = sys.argv, ["bench.py"]
    try:
        spec.loader.exec_module(mod)
    finally:
        sys.argv = argv
    return mod


def test_fp64_checks_match_the_oracle():
    b = _bench()
    rng = np.random.default_rng(7)
    x = (rng.standard_normal((3000, 16)) * 1.3 + 100.0).astype(np.float32)   # offset: cancellation
    q = (rng.standard_normal((200, 16)) * 1.3 + 100.0).astype(np.float32)
    for h in (0.4, 0.9):
        np.testing.assert_allclose(b.fp64_log_density(x, q, h), fp64.log_density(x, q, h), rtol=0, atol=1e-9)
    rows = [0, 17, 2999]
    p1, w1 = b.fp64_score_rows(x, rows, 0.9)
    p2, w2 = fp64.empirical_score_rows(x, rows, 0.9)
    np.testing.assert_allclose(p1, p2, rtol=1e-12)
    np.testing.assert_allclose(w1, w2, rtol=1e-12)


def test_error_measures():
    b = _bench()
    ref = np.array([-20.0, -30.0, -40.0])
    est = ref + np.array([1e-5, -2e-5, 0.0])
    m = b.log_error_stats(est, ref)
    om = fp64.log_error_metrics(est, ref)
    for k in ("max_abs_log_err", "mean_abs_log_err", "p95_abs_log_err", "max_rel_log_err"):
        assert abs(m[k] - om[k]) < 1e-15
    e = b.log_density_errors(np.exp(est), ref)
    assert abs(e["kde_max_abs_log_err_vs_fp64"] - 2e-5) < 1e-9
    assert abs(e["kde_max_rel_log_err_vs_fp64"] - 2e-5 / 30.0) < 1e-9
    assert e["kde_queries_checked"] == 3
