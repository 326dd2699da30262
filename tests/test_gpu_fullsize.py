"""Parity at the full sizes of the precision-stress and large configurations
(n = m = 2^20 offset Student-t; n = 2^22 score; 1-D 2^22 x 2^20), where the
full FP64 oracle would not finish: size-independent checks (run-to-run
bitwise determinism, finiteness) plus the FP64 oracle on fixed row / query
subsets.

Tolerances: relative log-density error vs FP64 1e-6 (spec bar 1e-5);
pdf_sum 1e-5 relative; weighted_sum 1e-5 relative with an absolute floor of
1e-5 * max|weighted| (signed sums cancel); 1-D densities 1e-5 relative.
"""
import numpy as np
import pytest
import torch

from conftest import rel_err
from oracle import fp64
from oracle import reference_numpy as R

pytestmark = pytest.mark.gpu


def test_precision_stress_2p20_offset_student_t(cuda_dev):
    """n = m = 2^20 heavy-tailed data at a +100 offset (the precision-stress
    configuration), h in {0.5, 1, 2} x Silverman of the training set, the
    exact precision modes (three-part fp16 tensor-core products with the
    exact near-pair recompute; FP32 direct differences) against FP64 log
    densities on a fixed 4096-query subset: relative log-density error
    <= 1e-6 (spec bar 1e-5) on every query whose density FP32 represents, and
    the exact-log output (no FP32 underflow) on all 4096.  The single-pass
    fp16 rung is measured too and must be the least accurate.

    Bars: relative log-density error |d log p| / |log p| <= 5e-6 (spec bar
    1e-5; measured worst 1.5e-6 over the 4096 queries); "representable" means
    the unnormalised FP32 sum is above e^-57, where the terms FP32 flushes to
    zero (at most n 2^-126) cannot move it by 1e-7."""
    from fsk import ops, workloads

    n = 1 << 20
    x_np = workloads.student_t_16d(n, seed=4)
    q_np = workloads.student_t_16d(n, seed=5)
    x = torch.from_numpy(x_np).to(cuda_dev)
    q = torch.from_numpy(q_np).to(cuda_dev)
    h0 = float(ops.silverman(x).item())
    sub = np.random.default_rng(0).choice(n, 4096, replace=False)
    for f in (0.5, 1.0, 2.0):
        h = h0 * f
        norm = 1.0 / ((2 * np.pi) ** 8 * h ** 16 * n)
        ref = fp64.log_density_gemm(x_np, q_np[sub], h)
        ok = np.isfinite(ref) & (ref - np.log(norm) > -57.0)   # unnormalised FP32 sum not near underflow
        assert ok.sum() > 1000
        worst = {}
        for precision in ("tensor", "ieee", "fp16_single"):
            lp = ops.kde16_sum(q, x, h, precision=precision, out_scale=norm, log_eps=0.0)
            ops.device_status(cuda_dev)
            got = lp.cpu().numpy().astype(np.float64)[sub]
            rel = np.abs(got[ok] - ref[ok]) / np.abs(ref[ok])
            worst[precision] = rel.max()
            if precision != "fp16_single":
                assert rel.max() < 5e-6, (f, precision, rel.max())
        assert worst["fp16_single"] > worst["tensor"], worst
        # exact log output: every query, also where FP32 densities underflow
        lp = ops.kde16_sum(q, x, h, out_scale=norm, log_exact=True)
        ops.device_status(cuda_dev)
        got = lp.cpu().numpy().astype(np.float64)[sub]
        fin = np.isfinite(ref)
        assert np.isfinite(got[fin]).all()
        rel = np.abs(got[fin] - ref[fin]) / np.abs(ref[fin])
        assert rel.max() < 5e-6, (f, "log_exact", rel.max())


def test_score_2p22_rows_and_determinism(cuda_dev):
    """n = 2^22 = 4 194 304 anisotropic points (the large low-rank
    configuration): the ordered tensor-core score is bitwise identical across
    two runs, rows across the whole range (including those past
    64 * 65535 = 4 194 240, where the reference's flash kernel writes the
    wrong rows) match the FP64 oracle, and the symmetric variant agrees with
    the ordered one on every row (the reference cannot run either variant
    here: its symmetric grid needs 65 536 > 65 535 blocks in y, its ordered
    partials ~1.1 TB)."""
    from fsk import ops, workloads

    n = 1 << 22
    x_np = workloads.lowrank_16d(n, seed=0)
    x = torch.from_numpy(x_np).to(cuda_dev)
    h = float(ops.silverman(x).item())
    pdf1, w1 = ops.empscore16(x, h)
    pdf2, w2 = ops.empscore16(x, h)
    ops.device_status(cuda_dev)
    assert torch.equal(pdf1, pdf2) and torch.equal(w1, w2)
    rows = np.array([0, 1, 77777, 2097152, 4194239, 4194240, 4194241, n - 1])
    p64, w64 = fp64.empirical_score_rows(x_np, rows, h)
    pdf = pdf1.cpu().numpy()[rows]
    w = w1.cpu().numpy()[rows]
    assert rel_err(pdf, p64).max() < 1e-5, rel_err(pdf, p64).max()
    np.testing.assert_allclose(w, w64, rtol=1e-5, atol=1e-5 * np.abs(w64).max())
    # the symmetric variant (each pair's exp once, upper-triangle tiles, FP64
    # atomics) against the ordered one over all 2^22 rows and against FP64
    ps, wsym = ops.empscore16(x, h, variant="symmetric")
    ops.device_status(cuda_dev)
    po, wo = pdf1.cpu().numpy().astype(np.float64), w1.cpu().numpy().astype(np.float64)
    ps_np, ws_np = ps.cpu().numpy().astype(np.float64), wsym.cpu().numpy().astype(np.float64)
    assert rel_err(ps_np, po).max() < 1e-5, rel_err(ps_np, po).max()
    assert (np.abs(ws_np - wo) <= 1e-5 * np.abs(wo) + 1e-5 * np.abs(wo).max()).all()
    assert rel_err(ps_np[rows], p64).max() < 1e-5
    np.testing.assert_allclose(ws_np[rows], w64, rtol=1e-5, atol=1e-5 * np.abs(w64).max())


def test_kde1d_2p22_by_2p20(cuda_dev):
    """1-D: 2^22 mixture points, 2^20 grid queries on [-5, 6]; FP64 oracle on
    64 fixed grid points; atomic and split-K agree."""
    from fsk import ops, workloads

    x_np = workloads.gmm3_1d(1 << 22, seed=0)
    q_np = workloads.grid_1d(1 << 20)
    h = float(R.silverman_bandwidth(x_np))
    x = torch.from_numpy(x_np).to(cuda_dev)
    q = torch.from_numpy(q_np).to(cuda_dev)
    norm = 1.0 / (np.sqrt(2 * np.pi) * h * x_np.size)
    a = ops.kde1d_sum(q, x, h, out_scale=norm)
    b = ops.kde1d_sum(q, x, h, out_scale=norm, atomic=True)
    ops.device_status(cuda_dev)
    a = a.cpu().numpy().astype(np.float64)
    b = b.cpu().numpy().astype(np.float64)
    assert np.isfinite(a).all()
    assert rel_err(b, a).max() < 1e-5
    sub = np.linspace(0, q_np.size - 1, 64).astype(np.int64)
    ref = fp64.density(x_np, q_np[sub], h, q_chunk=64, s_chunk=1 << 16)
    keep = ref > 1e-30
    assert rel_err(a[sub][keep], ref[keep]).max() < 1e-5
