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


def test_symmetric_matches_ordered_1024(cuda_dev, golden):
    """tests/large/test_consistency_large.py:21-56 of the reference (tolerance
    there 5e-3; here 1e-5)."""
    from fsk import ops

    g = golden("score16_seed10")
    x = torch.from_numpy(g["train"]).to(cuda_dev)
    po, wo = ops.empscore16(x, 1.0, variant="ordered")
    ps, wsym = ops.empscore16(x, 1.0, variant="symmetric")
    _close(ps.cpu().numpy(), po.cpu().numpy())
    _close(wsym.cpu().numpy(), wo.cpu().numpy())


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
