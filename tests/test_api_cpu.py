"""Host-side logic of the drop-in API that needs no GPU: validation order and
exception types (ValueError for bad arguments, as in the reference),
backend/precision validators, split heuristics and workload generators."""
import numpy as np
import pytest


def test_validators():
    from flash_sd_kde import config as C

    C.validate_precision_mode("fast_tf32")
    C.validate_precision_mode("fp32_ieee")
    with pytest.raises(ValueError):
        C.validate_precision_mode("bf16")
    with pytest.raises(ValueError):
        C.validate_kde_backend("nope")
    with pytest.raises(ValueError):
        C.validate_emp_score_backend("nope")
    assert C.select_emp_score_backend(10) == "flash_sd_kde"
    h = C.KernelHeuristics(default_emp_score_backend="ordered_splitk")
    assert C.select_emp_score_backend(10, heuristics=h) == "symmetric_atomic"
    assert C.select_emp_score_backend(10**6, heuristics=h) == "ordered_splitk"
    assert C.compute_splitk_splits(4096, block_n_iter=128, iters_per_split=8) == 4
    assert C.cap_splits_for_memory(1 << 22, 4096, features=16) == 1
    assert C.cap_splits_for_memory(1000, 7, features=16) == 7


def test_kde_eval_rejects_bad_arguments_before_device_work():
    from flash_sd_kde import emp_sd_kde_fit_transform, kde_eval

    x = np.zeros((8, 16), np.float32)
    with pytest.raises(ValueError):
        kde_eval(x, x, 0.0)
    with pytest.raises(ValueError):
        kde_eval(x, x, 1.0, device="cpu")
    with pytest.raises(ValueError):
        kde_eval(x, x, 1.0, precision_mode="tf64")
    with pytest.raises(ValueError):
        kde_eval(x, x, 1.0, kde_backend="bogus")
    with pytest.raises(ValueError):
        emp_sd_kde_fit_transform(x, -1.0)
    with pytest.raises(ValueError):
        emp_sd_kde_fit_transform(x, 1.0, emp_score_backend="bogus")
    with pytest.raises(ValueError):
        emp_sd_kde_fit_transform(x, 1.0, device="cpu")


def test_log_and_feature_count_arguments_before_device_work():
    """Host-side checks of the additions: exact log output needs eps >= 0,
    the padded rows take 1 <= d <= 16, the any-d rows 1 <= d <= 64."""
    import torch

    from flash_sd_kde.kde import kde_eval_log
    from fsk import ops

    x = np.zeros((8, 16), np.float32)
    with pytest.raises(ValueError):
        kde_eval_log(x, x, 1.0, eps=-1.0)
    with pytest.raises(ValueError):
        ops._as_rows(np.zeros((4, 65), np.float32), torch.device("cpu"))
    t = ops._as_rows(np.ones((4, 40), np.float32), torch.device("cpu"))
    assert t.shape == (4, 40) and t.is_contiguous()


def test_estimator_input_validation():
    from flash_sd_kde import FlashSDKDE

    est = FlashSDKDE()
    with pytest.raises(ValueError):
        est._validate_input(np.zeros(5, np.float32))
    with pytest.raises(ValueError):
        est._validate_input(np.zeros((0, 16), np.float32))
    with pytest.raises(ValueError):
        est._validate_input(np.zeros((3, 0), np.float32))
    with pytest.raises(ValueError):
        FlashSDKDE(mode="bogus")._validate_mode()
    with pytest.raises(ValueError):
        est.score_samples(np.zeros((3, 16), np.float32))


def test_padded_rows():
    """1 <= d <= 16 features are zero-padded to 16 (distances unchanged); more are rejected."""
    import torch

    from fsk import ops

    cpu = torch.device("cpu")
    x = np.arange(15, dtype=np.float32).reshape(3, 5)
    t, d = ops.as_padded_matrix(x, cpu)
    assert d == 5 and t.shape == (3, 16) and t.is_contiguous()
    assert np.array_equal(t[:, :5].numpy(), x) and not t[:, 5:].any()
    t16, d16 = ops.as_padded_matrix(np.ones((2, 16), np.float32), cpu)
    assert d16 == 16 and t16.shape == (2, 16)
    for bad in (np.zeros((3, 17), np.float32), np.zeros((3, 0), np.float32), np.zeros(4, np.float32)):
        with pytest.raises(ValueError):
            ops.as_padded_matrix(bad, cpu)


def test_kernel_wrappers_reject_bad_arguments():
    from kernels.flash_sd_kde import gaussian_kde_triton_nd, emp_score_16d_flash_sd_kde
    from kernels.kde_eval_16d_stream_splitk import kde_eval_16d_splitk

    x = np.zeros((4, 16), np.float32)
    with pytest.raises(ValueError):
        gaussian_kde_triton_nd(x, x, 0.0)
    with pytest.raises(ValueError):
        gaussian_kde_triton_nd(x, x, 1.0, device="cpu")
    with pytest.raises(ValueError):
        emp_score_16d_flash_sd_kde(x, 1.0, device="cpu")
    with pytest.raises(ValueError):
        kde_eval_16d_splitk(x, x, -2.0, device="cuda", precision_mode="fast_tf32",
                            use_precomputed_norms=True, autotune=False)


def test_workloads_are_seeded_and_shaped():
    from fsk import workloads as W

    a, b = W.plain_kde_16d()
    assert a.shape == (4096, 16) and b.shape == (1024, 16) and a.dtype == np.float32
    a2, _ = W.plain_kde_16d()
    assert np.array_equal(a, a2)
    g = W.GMM16(seed=0)
    assert np.isclose(g.weights.sum(), 1.0) and g.cov.shape == (8, 16, 16)
    s = g.sample(1000, seed=1)
    assert s.shape == (1000, 16) and np.isfinite(g.log_density(s)).all()
    t = W.student_t_16d(1000, seed=4)
    assert abs(np.median(t) - 100) < 5
    lr = W.lowrank_16d(10000)
    assert np.allclose(lr.std(0), np.arange(1, 17) ** -0.5, rtol=0.05)
    x1 = W.gmm3_1d(10000)
    assert x1.shape == (10000,)
    grid = W.grid_1d(11)
    assert grid[0] == -5 and grid[-1] == 6


def test_shard_partition_covers_rows():
    from fsk.workloads import shard

    for count in (1, 7, 1000, 1 << 20):
        for world in (1, 2, 3, 8):
            spans = [shard(count, world, r) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == count
            assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))


def test_exp2_poly_coefficients_and_error_bound():
    """The FMA-pipe exp2 (fsk_common.cuh, exp2_poly2) uses the coefficients
    its Remez generator (csrc/exp2_poly_remez.py) produces, and its FP32
    evaluation (round to nearest, exponent-field insertion) stays within
    2.5e-7 relative of FP64 2^x over x in [-125, 0] -- the error class of
    ex2.approx.f32."""
    import importlib.util
    import re

    import numpy as np

    from conftest import PKG

    src = (PKG / "csrc" / "fsk_common.cuh").read_text()
    body = src[src.index("float2 exp2_poly2"):]
    body = body[:body.index("\n}\n")]
    consts = [float(v) for v in re.findall(r"make_float2\(([0-9.e+-]+)f, \1f\)", body)]
    coeffs = [c for c in consts if 0.0 < c < 2.0]         # the polynomial (not the magic or the -1)
    spec = importlib.util.spec_from_file_location("remez", PKG / "csrc" / "exp2_poly_remez.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    c, err = mod.remez()
    want = [float(np.float32(v)) for v in c[::-1]]       # Horner order: c5 first
    assert len(coeffs) == 6
    np.testing.assert_allclose(coeffs, want, rtol=1e-8)
    assert err < 1e-7
    assert mod.fp32_check(c) < 2.5e-7
