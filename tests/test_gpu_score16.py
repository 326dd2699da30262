"""Empirical-score accumulators, debias shift and the SD-KDE pipeline on the GPU
against the reference's outputs and the FP64 oracle.

Tolerances: pdf_sum 1e-5 relative; weighted_sum 1e-5 relative with an
absolute floor of 1e-5 * max|weighted| (signed sums cancel); debiased points
1e-5 relative / absolute; symmetric vs ordered 1e-5.
"""
import numpy as np
import pytest
import torch

from conftest import rel_err
from oracle import fp64

pytestmark = pytest.mark.gpu


def _close(a, b, rtol=1e-5, floor=1e-5):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    np.testing.assert_allclose(a, b, rtol=rtol, atol=floor * np.abs(b).max())


def test_mma_ts_probe_layout(cuda_dev):
    """Four K=16 tcgen05.mma steps (fp16, M=128, N=16) with the A operand in
    tensor memory (two fp16 per column) and B in the transposed-feature image
    layout equal the host product of the fp16-rounded operands: pins the
    A-in-TMEM packing, the 128-byte-row descriptors and the N=16 instruction
    descriptor used by the score kernel's weighted-sum product."""
    from fsk import ops

    g = torch.Generator().manual_seed(1)
    a = torch.rand(128, 64, generator=g) * 4
    b = torch.randn(16, 64, generator=g) * 3
    d = ops.mma_ts_probe(a.to(cuda_dev), b.to(cuda_dev)).cpu().double()
    ah, bh = a.half().double(), b.half().double()
    ref = ah @ bh.T
    scale = ah.abs() @ bh.abs().T
    assert ((d - ref).abs() <= 2e-6 * scale + 1e-30).all(), float(((d - ref).abs() / scale).max())


def test_tmem_cp_probe_layout(cuda_dev):
    """tcgen05.cp 128x256b of the query operand image (64-byte rows, K-major
    core matrices) lands row r in TMEM lane r with word c holding the fp16
    pair (2c, 2c+1): the layout the score kernel's S product reads its A
    operand in."""
    from fsk import ops

    g = torch.Generator().manual_seed(5)
    a = torch.randn(128, 32, generator=g) * 3
    out = ops.tmem_cp_probe(a.to(cuda_dev)).cpu()
    want = a.half().contiguous().view(torch.int32)   # (128, 16): pairs of fp16 per word
    assert torch.equal(out, want)


@pytest.mark.parametrize("seed", [2, 3, 4, 10])
@pytest.mark.parametrize("variant", ["ordered", "symmetric"])
def test_score_vs_reference(cuda_dev, golden, seed, variant):
    from fsk import ops

    g = golden(f"score16_seed{seed}")
    x = torch.from_numpy(g["train"]).to(cuda_dev)
    h = float(g["h"])
    pdf, w = ops.empscore16(x, h, variant=variant)
    deb, score = ops.debias16(x, pdf, w, h, 1e-12, return_score=True)
    ops.device_status(cuda_dev)
    _close(pdf.cpu().numpy(), g["pdf_sum"])
    _close(w.cpu().numpy(), g["weighted"])
    _close(deb.cpu().numpy(), g["debiased"])
    p64, w64, s64 = fp64.empirical_score(g["train"], h)
    _close(pdf.cpu().numpy(), p64, rtol=2e-6, floor=0)
    _close(w.cpu().numpy(), w64, rtol=2e-6, floor=2e-6)


def _kernel_ids(fn):
    """Library kernel ids (fsk.h measurement hooks) launched by fn()."""
    from fsk import _lib as L

    lib = L.load()
    torch.cuda.synchronize()
    ids, nl = np.zeros(16, np.int32), np.zeros(16, np.int64)
    ms, work = np.zeros(16), np.zeros(16)
    lib.fsk_timer_collect(ids.ctypes.data, nl.ctypes.data, ms.ctypes.data, work.ctypes.data, 16)
    lib.fsk_timer_enable(1)
    try:
        out = fn()
        torch.cuda.synchronize()
    finally:
        lib.fsk_timer_enable(0)
    rows = lib.fsk_timer_collect(ids.ctypes.data, nl.ctypes.data, ms.ctypes.data, work.ctypes.data, 16)
    return out, {int(ids[r]) for r in range(rows)}


SYMMETRIC_KERNELS = {4, 8}    # CUDA-core / tensor-core upper-triangle kernels
ORDERED_KERNELS = {3, 7}


@pytest.mark.parametrize("precision", ["tensor", "ieee"])
def test_symmetric_matches_ordered_1024(cuda_dev, golden, precision):
    """tests/large/test_consistency_large.py:21-56 of the reference (tolerance
    there 5e-3; here 1e-5).  The two variants must run different kernels:
    the symmetric one evaluates each pair's exp once (upper-triangle tiles)."""
    from fsk import ops

    g = golden("score16_seed10")
    x = torch.from_numpy(g["train"]).to(cuda_dev)
    (po, wo), ko = _kernel_ids(lambda: ops.empscore16(x, 1.0, variant="ordered", precision=precision))
    (ps, wsym), ks = _kernel_ids(lambda: ops.empscore16(x, 1.0, variant="symmetric", precision=precision))
    assert ko & ORDERED_KERNELS and not ko & SYMMETRIC_KERNELS
    assert ks & SYMMETRIC_KERNELS and not ks & ORDERED_KERNELS
    _close(ps.cpu().numpy(), po.cpu().numpy())
    _close(wsym.cpu().numpy(), wo.cpu().numpy())
    p64, w64, _ = fp64.empirical_score(g["train"], 1.0)
    _close(ps.cpu().numpy(), p64, rtol=2e-6, floor=0)
    _close(wsym.cpu().numpy(), w64, rtol=2e-6, floor=2e-6)


@pytest.mark.parametrize("n", [1, 2, 63, 64, 65, 127, 128, 129, 255, 256, 257, 300, 513, 1000])
def test_symmetric_tile_boundary_shapes(cuda_dev, n):
    """Point counts around the triangle kernel's tiles (diagonal tiles,
    ragged last tile): pdf and weighted sums vs the FP64 oracle."""
    from fsk import ops

    rng = np.random.default_rng(n + 29)
    xs = (rng.standard_normal((n, 16)) * 1.5).astype(np.float32)
    h = 0.8
    pdf, w = ops.empscore16(torch.from_numpy(xs).to(cuda_dev), h, variant="symmetric")
    ops.device_status(cuda_dev)
    p64, w64, _ = fp64.empirical_score(xs, h)
    _close(pdf.cpu().numpy(), p64, rtol=2e-6, floor=0)
    _close(w.cpu().numpy(), w64, rtol=2e-6, floor=2e-6)


def test_ordered_is_bitwise_deterministic(cuda_dev):
    from fsk import ops, workloads

    x = torch.from_numpy(workloads.lowrank_16d(3000, seed=1)).to(cuda_dev)
    a = ops.empscore16(x, 0.4)
    b = ops.empscore16(x, 0.4)
    assert torch.equal(a[0], b[0]) and torch.equal(a[1], b[1])


def test_flash_layout_is_feature_major_view(cuda_dev, golden):
    """emp_score_16d_flash_sd_kde returns weighted as a (n,16) view of a
    (16,n) buffer (kernels/flash_sd_kde/empirical.py:180,223)."""
    from kernels.flash_sd_kde import emp_score_16d_flash_sd_kde

    g = golden("score16_seed2")
    pdf, w = emp_score_16d_flash_sd_kde(g["train"], float(g["h"]))
    assert w.shape == (128, 16) and w.stride() == (1, 128)
    _close(w.cpu().numpy(), g["weighted"])


def test_fit_transform_backends(cuda_dev, golden):
    from flash_sd_kde import emp_sd_kde_fit_transform

    g = golden("score16_seed4")
    outs = []
    for backend in (None, "flash_sd_kde", "ordered_splitk", "symmetric_atomic"):
        deb = emp_sd_kde_fit_transform(g["train"], 1.0, device="cuda", precision_mode="fp32_ieee",
                                       emp_score_backend=backend, autotune=False)
        assert deb.shape == g["train"].shape and torch.isfinite(deb).all()
        outs.append(deb.cpu().numpy())
        _close(outs[-1], g["debiased"])
    deb, pdf, w, score = emp_sd_kde_fit_transform(g["train"], 1.0, return_debug=True)
    # the score (W/pdf - x)/h^2 cancels; compare with the FP64 oracle on the
    # scale of the score (the reference's own FP32 score is off by ~1e-6 abs)
    _, _, s64 = fp64.empirical_score(g["train"], 1.0)
    _close(score.cpu().numpy(), s64, rtol=1e-5, floor=1e-5)
    _close(g["score"], s64, rtol=1e-3, floor=1e-3)


@pytest.mark.parametrize("n", [1, 2, 63, 64, 65, 255, 256, 257, 300, 513])
def test_score_tile_boundary_shapes(cuda_dev, n):
    """Point counts around the 64-point data tile, its 32-column halves and
    the 256-row work unit: pdf and weighted sums vs the FP64 oracle."""
    from fsk import ops

    rng = np.random.default_rng(n + 17)
    xs = (rng.standard_normal((n, 16)) * 1.5).astype(np.float32)
    h = 0.8
    pdf, w = ops.empscore16(torch.from_numpy(xs).to(cuda_dev), h)
    ops.device_status(cuda_dev)
    p64, w64, _ = fp64.empirical_score(xs, h)
    _close(pdf.cpu().numpy(), p64, rtol=2e-6, floor=0)
    _close(w.cpu().numpy(), w64, rtol=2e-6, floor=2e-6)


def test_score_offset_data(cuda_dev):
    """Offset heavy-tailed data: weighted sums and debiased points vs FP64."""
    from fsk import ops, workloads

    xs = workloads.student_t_16d(2048, seed=7)
    h = 0.8
    x = torch.from_numpy(xs).to(cuda_dev)
    pdf, w = ops.empscore16(x, h)
    deb = ops.debias16(x, pdf, w, h, 1e-12)
    p64, w64, _ = fp64.empirical_score(xs, h)
    assert rel_err(pdf.cpu().numpy(), p64).max() < 1e-5
    d64 = fp64.debias(xs, h)
    assert np.abs(deb.cpu().numpy() - d64).max() < 1e-5 * np.abs(d64).max()


@pytest.mark.parametrize("return_tensor", [True, False])
def test_empirical_sd_kde_triton_nd_vs_reference(cuda_dev, golden, return_tensor):
    """kernels/flash_sd_kde/empirical.py:226-287 of the reference: the
    debiased points (tensor or numpy) and the bandwidth it returns, against
    the reference's outputs on the golden seeds and against FP64."""
    from kernels.flash_sd_kde import empirical_sd_kde_triton_nd

    for seed in (2, 3, 4, 10):
        g = golden(f"score16_seed{seed}")
        h = float(g["h"])
        deb, h_out = empirical_sd_kde_triton_nd(g["train"], h, return_tensor=return_tensor)
        assert h_out == h
        if return_tensor:
            assert isinstance(deb, torch.Tensor) and deb.is_cuda and deb.dtype == torch.float32
            deb = deb.cpu().numpy()
        else:
            assert isinstance(deb, np.ndarray) and deb.dtype == np.float32
        assert deb.shape == g["train"].shape
        _close(deb, g["debiased"])
        _close(deb, fp64.debias(g["train"], h), rtol=2e-6, floor=2e-6)


@pytest.mark.parametrize("splits,count,features", [(1, 1, None), (7, 1000, None), (64, 4097, None),
                                                    (5, 300, 16), (33, 129, 16), (1, 17, 3)])
def test_reduce_partials_vs_fixed_order_fp64(cuda_dev, splits, count, features):
    """kernels/reduce_partials.py:61-108 of the reference: the sum over the
    split axis of (splits, n) and (splits, n, features) FP32 partials.  Here
    the sum is formed in FP64 in split order, so it equals the FP64
    fixed-order sum rounded once to FP32."""
    from kernels.reduce_partials import reduce_pdf_partials, reduce_weighted_partials

    rng = np.random.default_rng(splits * 1000 + count)
    shape = (splits, count) if features is None else (splits, count, features)
    # magnitudes over many binades with cancelling signs: an FP32 running sum would differ
    p = (rng.standard_normal(shape) * 10.0 ** rng.uniform(-3, 3, size=shape)).astype(np.float32)
    pt = torch.from_numpy(p).to(cuda_dev)
    out = reduce_pdf_partials(pt) if features is None else reduce_weighted_partials(pt)
    ops_out = out.cpu().numpy()
    ref = np.zeros(shape[1:], np.float64)
    for s in range(splits):
        ref += p[s].astype(np.float64)
    assert ops_out.shape == ref.shape and ops_out.dtype == np.float32
    np.testing.assert_array_equal(ops_out, ref.astype(np.float32))


def test_reduce_partials_rejects_bad_shapes(cuda_dev):
    from kernels.reduce_partials import reduce_pdf_partials, reduce_weighted_partials

    with pytest.raises(ValueError):
        reduce_pdf_partials(torch.zeros((2, 3, 4), device=cuda_dev))
    with pytest.raises(ValueError):
        reduce_weighted_partials(torch.zeros((2, 3), device=cuda_dev))


@pytest.mark.parametrize("precision", ["tensor", "ieee"])
def test_one_call_sdkde_matches_two_calls_and_fp64(cuda_dev, precision):
    """fsk_sdkde16 (score -> debias -> KDE in one call) gives bit for bit the
    result of the public two-call path (emp_sd_kde_fit_transform with the
    ordered backend, then kde_eval), matches the FP64 pipeline, and replays
    identically from a captured CUDA graph."""
    from flash_sd_kde import emp_sd_kde_fit_transform, kde_eval
    from flash_sd_kde.kde import sd_kde_eval
    from fsk import ops, workloads

    g = workloads.GMM16(seed=0)
    x_np, q_np = g.sample(3000, seed=1), g.sample(700, seed=2)
    x = torch.from_numpy(x_np).to(cuda_dev)
    q = torch.from_numpy(q_np).to(cuda_dev)
    h = 0.7
    mode = "fp32_ieee" if precision == "ieee" else "fast_tf32"
    dens, deb = sd_kde_eval(x, q, h, precision_mode=mode, return_debiased=True)
    deb2 = emp_sd_kde_fit_transform(x, h, precision_mode=mode, emp_score_backend="ordered_splitk")
    dens2 = kde_eval(deb2, q, h, precision_mode=mode)
    ops.device_status(cuda_dev)
    assert torch.equal(deb, deb2) and torch.equal(dens, dens2)
    deb64 = fp64.debias(x_np, h)
    ref = np.exp(fp64.log_density(deb64, q_np, h))
    assert rel_err(dens.cpu().numpy(), ref).max() < 1e-5
    graph = ops.SDKDEGraph(x, q, h, precision=precision)
    out = graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(out, dens)
    # new inputs copied into the captured buffers
    x_b = torch.from_numpy(g.sample(3000, seed=5)).to(cuda_dev)
    graph.data.copy_(x_b)
    out_b = graph.replay().clone()
    ops.device_status(cuda_dev)
    assert torch.equal(out_b, sd_kde_eval(x_b, q, h, precision_mode=mode))
