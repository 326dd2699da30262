"""Empirical-score accumulators and one-step SD-KDE on GB300: drop-in for
kernels/flash_sd_kde/empirical.py.

emp_score_16d_flash_sd_kde   pdf_sum (n,), weighted_sum (n,16) view of a (16,n) buffer  (reference :134-223)
empirical_sd_kde_triton_nd   16-D debiased data and h                                 (reference :226-287)
empirical_sd_kde_triton      1-D debiased data with h = 0.4 sigma n^(-1/9)             (reference :290-362)

The debias shift x + h^2/2 (W/(pdf+1e-12) - x)/h^2 runs as one FP64 kernel.
"""
from __future__ import annotations

from typing import Sequence

import numpy as np
import torch

from fsk import ops

from .common import _ND_FEATURES, _check_cuda, _to_matrix_tensor, _to_torch_tensor
from .kde import _finish, gaussian_kde_score_triton

_EPS = 1e-12


def emp_score_16d_flash_sd_kde(
    data: Sequence[Sequence[float]] | torch.Tensor,
    bandwidth: float,
    *,
    block_m: int = 64,
    block_n: int = 2048,
    num_warps: int = 2,
    num_stages: int = 2,
    device: str | torch.device = "cuda",
    synchronize: bool = True,
) -> tuple[torch.Tensor, torch.Tensor]:
    """pdf_sum[i] = sum_j phi_ij and weighted_sum[i] = sum_j phi_ij x_j (self-pair included)."""
    if bandwidth <= 0:
        raise ValueError("bandwidth must be positive.")
    dev = _check_cuda(device, "emp_score_16d_flash_sd_kde")
    train = _to_matrix_tensor(data, dev, dim=_ND_FEATURES)
    if train.shape[0] == 0:
        raise ValueError("data must contain at least one element.")
    pdf, w = ops.empscore16(train, bandwidth, variant="ordered", feature_major=True)
    _finish(dev, synchronize)
    return pdf, w


def empirical_sd_kde_triton_nd(
    data: Sequence[Sequence[float]] | torch.Tensor,
    bandwidth: float,
    *,
    block_m: int = 64,
    block_n: int = 2048,
    num_warps: int = 2,
    num_stages: int = 2,
    device: str | torch.device = "cuda",
    return_tensor: bool = False,
    synchronize: bool = True,
) -> tuple[torch.Tensor | np.ndarray, float]:
    """One-step 16-D empirical SD-KDE debiasing; returns (debiased, bandwidth)."""
    if bandwidth <= 0:
        raise ValueError("bandwidth must be positive.")
    dev = _check_cuda(device, "empirical_sd_kde_triton_nd")
    train = _to_matrix_tensor(data, dev, dim=_ND_FEATURES)
    if train.shape[0] == 0:
        raise ValueError("data must contain at least one element.")
    pdf, w = ops.empscore16(train, bandwidth, variant="ordered", feature_major=True)
    debiased = ops.debias16(train, pdf, w, bandwidth, _EPS)
    _finish(dev, synchronize)
    if return_tensor:
        return debiased, bandwidth
    return debiased.detach().cpu().numpy(), bandwidth


def empirical_sd_kde_triton(
    data: Sequence[float] | torch.Tensor,
    *,
    block_m: int = 64,
    block_n: int = 128,
    num_warps: int = 1,
    num_stages: int = 2,
    device: str | torch.device = "cuda",
    return_tensor: bool = False,
    synchronize: bool = True,
) -> tuple[torch.Tensor | np.ndarray, float]:
    """One-step 1-D empirical SD-KDE; the bandwidth 0.4 min(std, IQR/1.34) n^(-1/9)
    is computed on the GPU.  Returns (debiased, h)."""
    dev = _check_cuda(device, "empirical_sd_kde_triton")
    train = _to_torch_tensor(data, dev).reshape(-1)
    if train.numel() == 0:
        raise ValueError("data must contain at least one element.")
    h = float(ops.silverman(train, rule="sdkde_1d").item())
    delta = 0.5 * h * h
    scores, _, _ = gaussian_kde_score_triton(train, train, h, device=dev, synchronize=synchronize)
    debiased = train + delta * scores
    _finish(dev, synchronize)
    if return_tensor:
        return debiased, h
    return debiased.detach().cpu().numpy(), h
