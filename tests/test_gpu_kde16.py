"""16-D KDE through the C ABI on the GPU, both precision modes, against the
reference's own outputs (golden fixtures) and the FP64 oracle.

Tolerances (relative, on densities unless stated):
  * vs the reference FP32 CPU path: 1e-5 (the bar of the target spec);
  * vs the FP64 oracle: max 1e-5, median 1e-6;
  * relative log-density error vs FP64: 1e-6 (spec bar 1e-5).
"""
import numpy as np
import pytest
import torch

from conftest import rel_err
from oracle import fp64
from oracle import reference_numpy as R

pytestmark = pytest.mark.gpu
PRECISIONS = ["tensor", "ieee"]


def _kde(dev, q, x, h, precision="tensor", **kw):
    from fsk import ops

    norm = 1.0 / ((2.0 * np.pi) ** 8 * h ** 16 * x.shape[0])
    out = ops.kde16_sum(torch.from_numpy(np.ascontiguousarray(q)).to(dev),
                        torch.from_numpy(np.ascontiguousarray(x)).to(dev), h, precision=precision,
                        out_scale=kw.pop("scale", norm), **kw)
    ops.device_status(dev)
    return out.cpu().numpy().astype(np.float64)


def test_mma_probe_layout(cuda_dev):
    """Two K=16 tcgen05.mma steps (fp16, M=128, N=64) over the 64-byte-row
    operand images of the KDE kernel equal the host dot product of the
    fp16-rounded operands: pins the smem/instruction descriptors, the K-step
    offset and the TMEM lane/column mapping."""
    from fsk import ops

    g = torch.Generator().manual_seed(0)
    a = torch.randn(128, 32, generator=g) * 3
    b = torch.randn(64, 32, generator=g) * 3
    d = ops.mma_probe(a.to(cuda_dev), b.to(cuda_dev)).cpu().double()
    ah, bh = a.half().double(), b.half().double()
    ref = ah @ bh.T
    scale = ah.abs() @ bh.abs().T
    assert ((d - ref).abs() <= 2e-6 * scale + 1e-30).all(), float(((d - ref).abs() / scale).max())


@pytest.mark.parametrize("precision", PRECISIONS)
def test_plain_4096x1024_vs_reference_and_fp64(cuda_dev, golden, precision):
    g = golden("kde16_plain_4096x1024")
    out = _kde(cuda_dev, g["queries"], g["train"], float(g["h"]), precision)
    truth = np.exp(g["log_density_fp64"])
    e64 = rel_err(out, truth)
    assert e64.max() < 1e-5 and np.median(e64) < 1e-6, (e64.max(), np.median(e64))
    assert rel_err(out, g["density"]).max() < 1e-5
    rel_log = np.abs(np.log(out) - g["log_density_fp64"]) / np.abs(g["log_density_fp64"])
    assert rel_log.max() < 1e-6


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("name", ["kde16_seed1", "kde16_seed11"])
def test_reference_test_cases(cuda_dev, golden, precision, name):
    g = golden(name)
    out = _kde(cuda_dev, g["queries"], g["train"], float(g["h"]), precision)
    assert rel_err(out, g["density"]).max() < 1e-5


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("name", ["kde16_lin_seed5", "kde16_lin_seed7"])
def test_laplace_reference_cases(cuda_dev, golden, precision, name):
    g = golden(name)
    out = _kde(cuda_dev, g["queries"], g["train"], float(g["h"]), precision, laplace=True)
    ref = g["density"].astype(np.float64)
    np.testing.assert_allclose(out, ref, rtol=1e-5, atol=1e-5 * np.abs(ref).max())


@pytest.mark.parametrize("m,n", [(1, 1), (1, 300), (129, 1), (100, 127), (257, 129), (255, 4097), (513, 1000)])
@pytest.mark.parametrize("precision", PRECISIONS)
def test_ragged_and_tiny_shapes(cuda_dev, m, n, precision):
    rng = np.random.default_rng(m * 7919 + n)
    x = rng.standard_normal((n, 16)).astype(np.float32)
    q = (rng.standard_normal((m, 16)) * 0.8).astype(np.float32)
    h = 0.9
    out = _kde(cuda_dev, q, x, h, precision)
    truth = fp64.density(x, q, h)
    assert rel_err(out, truth).max() < 1e-5


@pytest.mark.parametrize("m,n", [(256, 64), (257, 65), (511, 191), (512, 192), (513, 193), (255, 320),
                                 (256, 383), (1, 384), (300, 385), (768, 1000)])
def test_tile_boundary_shapes(cuda_dev, m, n):
    """Query counts around the 256-query work unit and data counts around the
    128-point tile and its 64-point column halves (tensor-core path)."""
    rng = np.random.default_rng(m * 131 + n)
    x = rng.standard_normal((n, 16)).astype(np.float32)
    q = (x[rng.integers(0, n, m)] + 0.3 * rng.standard_normal((m, 16))).astype(np.float32)
    h = 0.7
    out = _kde(cuda_dev, q, x, h)
    truth = fp64.density(x, q, h)
    assert rel_err(out, truth).max() < 1e-5


@pytest.mark.parametrize("precision", PRECISIONS)
def test_offset_heavy_tail_cancellation(cuda_dev, precision):
    """Student-t data with a +100 offset: the norm expansion cancels
    catastrophically in FP32 without centring (the reference's FP32 path is
    off by up to 100% here); the kernels must stay at FP64-level accuracy."""
    from fsk import workloads

    x = workloads.student_t_16d(8192, seed=4)
    q = workloads.student_t_16d(512, seed=5)
    h0 = R.silverman_bandwidth_nd(x)
    for f in (0.5, 1.0, 2.0):
        h = h0 * f
        from fsk import ops

        lp = ops.kde16_sum(torch.from_numpy(q).to(cuda_dev), torch.from_numpy(x).to(cuda_dev), h,
                           precision=precision, out_scale=1.0 / ((2 * np.pi) ** 8 * h ** 16 * x.shape[0]),
                           log_eps=0.0).cpu().numpy().astype(np.float64)
        ref = fp64.log_density(x, q, h)
        ok = np.isfinite(ref) & (ref > -80.0)      # densities representable in FP32
        rel_log = np.abs(lp[ok] - ref[ok]) / np.abs(ref[ok])
        assert rel_log.max() < 1e-6, (f, rel_log.max())


def test_tensor_path_is_deterministic_and_atomic_agrees(cuda_dev, golden):
    g = golden("kde16_plain_4096x1024")
    a = _kde(cuda_dev, g["queries"], g["train"], float(g["h"]))
    b = _kde(cuda_dev, g["queries"], g["train"], float(g["h"]))
    assert np.array_equal(a, b)
    c = _kde(cuda_dev, g["queries"], g["train"], float(g["h"]), atomic=True)
    assert rel_err(c, a).max() < 1e-6


def test_query_chunking_invariance(cuda_dev, golden):
    """tests/large/test_consistency_large.py:59-73 of the reference."""
    g = golden("kde16_seed11")
    full = _kde(cuda_dev, g["queries"], g["train"], float(g["h"]))
    half = g["queries"].shape[0] // 2
    a = _kde(cuda_dev, g["queries"][:half], g["train"], float(g["h"]))
    b = _kde(cuda_dev, g["queries"][half:], g["train"], float(g["h"]))
    assert rel_err(np.concatenate([a, b]), full).max() < 1e-7


def test_log_output_matches(cuda_dev, golden):
    g = golden("kde16_plain_4096x1024")
    d = _kde(cuda_dev, g["queries"], g["train"], float(g["h"]))
    h = float(g["h"])
    lp = _kde(cuda_dev, g["queries"], g["train"], h, log_eps=1e-12)
    np.testing.assert_allclose(lp, np.log(d + 1e-12), rtol=1e-6)


def test_invalid_arguments_raise_value_error(cuda_dev):
    from fsk import ops

    x = torch.zeros(10, 16, device=cuda_dev)
    with pytest.raises(ValueError):
        ops.kde16_sum(x, x, 0.0)
    with pytest.raises(ValueError):
        ops.kde16_sum(x, x, float("nan"))
    with pytest.raises(ValueError):
        ops.kde16_sum(torch.zeros(10, 15, device=cuda_dev), x, 1.0)
    with pytest.raises(ValueError):
        ops.kde16_sum(torch.zeros(0, 16, device=cuda_dev), x, 1.0)


def test_bounded_wait_timeout_is_reported(cuda_dev):
    """A kernel waits on an mbarrier nothing arrives on; the wait gives up
    (~2 s), the status is read on the host and the context stays usable."""
    from fsk import _lib as L
    from fsk import ops

    flag = torch.full((1,), -1, dtype=torch.int32, device=cuda_dev)
    st = L.load().fsk_diag_wait_timeout_probe(flag.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert st == L.FSK_OK
    with pytest.raises(L.FskError) as ei:
        ops.device_status(cuda_dev)
    assert ei.value.status == L.FSK_ERR_DEVICE_TIMEOUT
    assert int(flag.item()) == 0
    ops.device_status(cuda_dev)          # cleared
    x = torch.randn(64, 16, device=cuda_dev)
    assert torch.isfinite(ops.kde16_sum(x, x, 1.0)).all()


# ---- exact log-densities (FSK_OUT_LOG_EXACT) ---------------------------------

def _far_case(seed, n=3000, m_near=300, m_far=300):
    """N(0, I) data; queries in support and 5-40 standard deviations away
    (every FP32 term of the far queries underflows)."""
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((n, 16)).astype(np.float32)
    near = rng.standard_normal((m_near, 16)).astype(np.float32)
    direc = rng.standard_normal((m_far, 16))
    direc /= np.linalg.norm(direc, axis=1, keepdims=True)
    radius = rng.uniform(5.0, 40.0, (m_far, 1))
    far = (direc * radius + 0.3 * rng.standard_normal((m_far, 16))).astype(np.float32)
    q = np.concatenate([near, far])
    q = q[rng.permutation(q.shape[0])]
    return x, q, float(R.silverman_bandwidth_nd(x))


def _log_exact(dev, q, x, h, precision="tensor"):
    from fsk import ops

    norm = 1.0 / ((2.0 * np.pi) ** 8 * h ** 16 * x.shape[0])
    out = ops.kde16_sum(torch.from_numpy(q).to(dev), torch.from_numpy(x).to(dev), h, precision=precision,
                        out_scale=norm, log_exact=True)
    ops.device_status(dev)
    return out.cpu().numpy().astype(np.float64)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_log_exact_far_queries(cuda_dev, precision):
    """log-densities of in-support and far queries vs the FP64 oracle:
    |error| <= 1e-5 + 2e-6 |log p| (FP32 squared distances of far queries carry
    ~1e-7 relative rounding, i.e. ~1e-4 absolute in log p at 30 h)."""
    x, q, h = _far_case(0)
    out = _log_exact(cuda_dev, q, x, h, precision)
    ref = fp64.log_density(x, q, h)
    assert np.isfinite(out).all()
    assert ref.min() < -1000.0          # far queries underflow FP32 by hundreds of nats
    err = np.abs(out - ref)
    assert (err <= 1e-5 + 2e-6 * np.abs(ref)).all(), float((err / (1e-5 + 2e-6 * np.abs(ref))).max())
    assert (err / np.abs(ref)).max() < 1e-6


def test_log_exact_matches_plain_log_in_support(cuda_dev):
    """Queries whose sum does not underflow take the plain path: bitwise the
    value of FSK_OUT_LOG with eps = 0."""
    from fsk import ops

    x, q, h = _far_case(1, m_far=0)
    norm = 1.0 / ((2.0 * np.pi) ** 8 * h ** 16 * x.shape[0])
    qd, xd = torch.from_numpy(q).to(cuda_dev), torch.from_numpy(x).to(cuda_dev)
    plain = ops.kde16_sum(qd, xd, h, out_scale=norm, log_eps=0.0).cpu().numpy()
    exact = ops.kde16_sum(qd, xd, h, out_scale=norm, log_exact=True).cpu().numpy()
    ops.device_status(cuda_dev)
    assert np.array_equal(plain, exact)


@pytest.mark.parametrize("n,m", [(1, 1), (33, 5), (31, 200), (4097, 1)])
def test_log_exact_all_far_ragged(cuda_dev, n, m):
    """Every query far away (all recomputed), ragged data tiles; two runs are
    bitwise identical although the recompute list order may differ."""
    rng = np.random.default_rng(n * 7 + m)
    x = rng.standard_normal((n, 16)).astype(np.float32)
    q = (rng.standard_normal((m, 16)) + 12.0).astype(np.float32)
    h = 0.5
    a = _log_exact(cuda_dev, q, x, h)
    b = _log_exact(cuda_dev, q, x, h)
    ref = fp64.log_density(x, q, h)
    assert np.array_equal(a, b)
    assert (np.abs(a - ref) <= 1e-5 + 2e-6 * np.abs(ref)).all()


def test_kde_eval_log_eps0_and_estimator_log_space(cuda_dev):
    """kde_eval_log(eps=0) and FlashSDKDE(log_space=True) return the exact
    log-density; the default estimator keeps the reference's log(p + eps)
    floor for far queries."""
    from flash_sd_kde import FlashSDKDE
    from flash_sd_kde.kde import kde_eval_log

    x, q, h = _far_case(2, n=2000, m_near=100, m_far=100)
    ref = fp64.log_density(x, q, h)
    tol = 1e-5 + 2e-6 * np.abs(ref)
    out = kde_eval_log(torch.from_numpy(x).to(cuda_dev), torch.from_numpy(q).to(cuda_dev), h, eps=0.0,
                       device=cuda_dev).cpu().numpy()
    assert (np.abs(out - ref) <= tol).all()
    est = FlashSDKDE(bandwidth=h, mode="kde", device=cuda_dev, log_space=True).fit(x)
    assert (np.abs(est.score_samples(q) - ref) <= tol).all()
    floor = FlashSDKDE(bandwidth=h, mode="kde", device=cuda_dev).fit(x).score_samples(q)
    far = ref < -200.0
    assert far.any() and np.allclose(floor[far], np.log(1e-12), rtol=0, atol=1e-5)



@pytest.mark.parametrize("precision", PRECISIONS)
def test_error_suite_smoke_configuration(cuda_dev, precision):
    """The reference's error-suite smoke run (experiments/error_suite_16d,
    configs/error_suite_16d/smoke.yaml: 4-component diagonal mixture, 8192
    train / 4096 test, standardised, Silverman-diag bandwidth, log-density
    output against the FP64 log-space reference): every log-density finite,
    max / p95 / mean absolute log error against FP64 within 1e-5 / 2e-6 / 1e-6
    (the reference's test asks for a finite maximum)."""
    from flash_sd_kde.kde import kde_eval_log
    from fsk import workloads

    train, test = workloads.gm_diag_16d()
    h = fp64.silverman_nd(train)
    ref = fp64.log_density(train, test, h)
    mode = "fast_tf32" if precision == "tensor" else "fp32_ieee"
    out = kde_eval_log(torch.from_numpy(train).to(cuda_dev), torch.from_numpy(test).to(cuda_dev), h, eps=0.0,
                       device=cuda_dev, precision_mode=mode).cpu().numpy()
    m = fp64.log_error_metrics(out, ref)
    assert m["finite_fraction"] == 1.0
    assert m["max_abs_log_err"] < 1e-5 and m["p95_abs_log_err"] < 2e-6 and m["mean_abs_log_err"] < 1e-6, m


@pytest.mark.parametrize("name", ["kde16_plain_4096x1024", "kde16_seed1", "kde16_seed11"])
def test_exp_offload_vs_reference_and_fp64(cuda_dev, golden, name):
    """FSK_EXP_OFFLOAD: a quarter of the exps by the FMA-pipe polynomial
    (exp2_poly2) instead of ex2.approx; the same bars as the default tensor
    path against the reference outputs and FP64, and within 1e-6 of it."""
    g = golden(name)
    h = float(g["h"])
    out = _kde(cuda_dev, g["queries"], g["train"], h, "tensor", exp_offload=True)
    base = _kde(cuda_dev, g["queries"], g["train"], h, "tensor")
    assert rel_err(out, g["density"]).max() < 1e-5
    assert rel_err(out, base).max() < 1e-6
    if "log_density_fp64" in g:
        e64 = rel_err(out, np.exp(g["log_density_fp64"]))
        assert e64.max() < 1e-5 and np.median(e64) < 1e-6, (e64.max(), np.median(e64))


def test_exp_offload_far_queries_and_flags(cuda_dev):
    """Queries far from the data: where the unnormalised sum is above
    n 2^-100 (so terms below FP32's 2^-126, which ex2.approx flushes and the
    polynomial clamps to ~2^-125, cannot move it by 1e-6) the densities agree
    to 1e-6; below that both are negligible.  The offload flag is refused
    outside fsk_kde16's tensor path."""
    from fsk import _lib as L

    rng = np.random.default_rng(3)
    n = 3000
    x = rng.standard_normal((n, 16)).astype(np.float32)
    q = np.concatenate([rng.standard_normal((200, 16)), rng.standard_normal((56, 16)) + 4.0]).astype(np.float32)
    for h in (0.3, 0.8):
        out = _kde(cuda_dev, q, x, h, "tensor", exp_offload=True, scale=1.0)
        base = _kde(cuda_dev, q, x, h, "tensor", scale=1.0)
        big = base > n * 2.0 ** -100
        assert big.sum() > 150
        assert rel_err(out[big], base[big]).max() < 1e-6
        assert (out[~big] <= 2.0 * n * 2.0 ** -100).all()
    lib = L.load()
    t = torch.zeros((4, 16), device=cuda_dev)
    pdf = torch.zeros(4, device=cuda_dev)
    st = lib.fsk_empscore16(t.data_ptr(), 4, 1.0, 0, L.FSK_EXP_OFFLOAD, pdf.data_ptr(), t.data_ptr(), None, 0,
                            torch.cuda.current_stream().cuda_stream)
    assert st == L.FSK_ERR_INVALID_ARGUMENT
