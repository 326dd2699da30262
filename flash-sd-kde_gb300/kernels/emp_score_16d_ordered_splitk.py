"""Deterministic empirical-score accumulators: drop-in for
kernels/emp_score_16d_ordered_splitk.py:162-263.

Returns (pdf_sum (n,), weighted_sum (n,16)).  Per-split partials are
reduced in a fixed order in FP64 (bit-identical run to run); the split count
is bounded so the partial buffer stays a small multiple of the output.
"""
from __future__ import annotations

import torch

from fsk import ops
from globals import ND_FEATURES, PRECISION_FAST_TF32, PRECISION_FP32_IEEE


def emp_score_16d_ordered_splitk(
    data,
    bandwidth: float,
    *,
    device: torch.device,
    precision_mode: str,
    use_precomputed_norms: bool,
    autotune: bool,
):
    if bandwidth <= 0:
        raise ValueError("bandwidth must be positive.")
    device = ops._device(device)
    train = ops.as_matrix(data, device, ND_FEATURES)
    if train.shape[0] == 0:
        raise ValueError("data must be non-empty.")
    if precision_mode not in {PRECISION_FAST_TF32, PRECISION_FP32_IEEE}:
        raise ValueError(f"invalid precision_mode {precision_mode}.")
    prec = "ieee" if precision_mode == PRECISION_FP32_IEEE else "tensor"
    return ops.empscore16(train, bandwidth, variant="ordered", precision=prec)
