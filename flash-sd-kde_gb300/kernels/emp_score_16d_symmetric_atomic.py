"""Symmetric empirical-score accumulators (phi_ij = phi_ji, upper-triangle
tiles, each pair's exp evaluated once): drop-in for
kernels/emp_score_16d_symmetric_atomic.py:163-234.  Row and column
contributions are scattered with FP64 atomics.
"""
from __future__ import annotations

import torch

from fsk import ops
from globals import ND_FEATURES, PRECISION_FAST_TF32, PRECISION_FP32_IEEE


def emp_score_16d_symmetric_atomic(
    data,
    bandwidth: float,
    *,
    device: torch.device,
    precision_mode: str,
    use_precomputed_norms: bool,
    block_size: int = 64,
    autotune: bool = False,
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
    return ops.empscore16(train, bandwidth, variant="symmetric", precision=prec)
