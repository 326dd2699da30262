"""Normalised Gaussian KDE on GB300: drop-in for kernels/flash_sd_kde/kde.py.

gaussian_kde_triton       1-D density, sum_j phi(z)/(sqrt(2 pi) h n)   (reference :147-225)
gaussian_kde_triton_nd    16-D density, sum_j phi/((2 pi)^8 h^16 n)    (reference :242-331)
gaussian_kde_score_triton 1-D score, pdf and derivative                (reference :348-438)

Tile/launch keywords (block_m, block_n, num_warps, num_stages) are accepted
for signature compatibility; the GB300 kernels choose their own tiling.  The
normalisation is applied in FP64 inside the split reduction.
"""
from __future__ import annotations

import math
from typing import Sequence

import numpy as np
import torch

from fsk import ops

from .common import _ND_FEATURES, _check_cuda, _to_matrix_tensor, _to_torch_tensor


def _finish(device: torch.device, synchronize: bool) -> None:
    if synchronize:
        torch.cuda.synchronize(device)
        ops.device_status(device)


def gaussian_kde_triton(
    data: Sequence[float] | torch.Tensor,
    queries: Sequence[float] | torch.Tensor,
    bandwidth: float,
    *,
    block_m: int = 128,
    block_n: int = 128,
    num_warps: int = 4,
    num_stages: int = 2,
    device: str | torch.device = "cuda",
    synchronize: bool = True,
) -> torch.Tensor:
    """1-D Gaussian KDE density at `queries` (shape (n_query,))."""
    if bandwidth <= 0:
        raise ValueError("bandwidth must be positive.")
    dev = _check_cuda(device, "gaussian_kde_triton")
    train = _to_torch_tensor(data, dev).reshape(-1)
    query = _to_torch_tensor(queries, dev).reshape(-1)
    if train.numel() == 0 or query.numel() == 0:
        raise ValueError("data and queries must contain at least one sample.")
    scale = 1.0 / (math.sqrt(2.0 * math.pi) * bandwidth * train.numel())
    out = ops.kde1d_sum(query, train, bandwidth, out_scale=scale)
    _finish(dev, synchronize)
    return out


def gaussian_kde_triton_numpy(data, queries, bandwidth: float, *, device="cuda") -> np.ndarray:
    return gaussian_kde_triton(data=data, queries=queries, bandwidth=bandwidth, device=device).detach().cpu().numpy()


def gaussian_kde_triton_nd(
    data: Sequence[Sequence[float]] | torch.Tensor,
    queries: Sequence[Sequence[float]] | torch.Tensor,
    bandwidth: float,
    *,
    block_m: int = 64,
    block_n: int = 64,
    num_warps: int = 4,
    num_stages: int = 2,
    device: str | torch.device = "cuda",
    synchronize: bool = True,
) -> torch.Tensor:
    """16-D Gaussian KDE density at `queries` (shape (n_query,))."""
    if bandwidth <= 0:
        raise ValueError("bandwidth must be positive.")
    dev = _check_cuda(device, "gaussian_kde_triton_nd")
    train = _to_matrix_tensor(data, dev, dim=_ND_FEATURES)
    query = _to_matrix_tensor(queries, dev, dim=_ND_FEATURES)
    n_data, n_query = train.shape[0], query.shape[0]
    if n_data == 0 or n_query == 0:
        raise ValueError("data and queries must contain at least one sample.")
    norm = (1.0 / bandwidth) ** _ND_FEATURES / (((2.0 * math.pi) ** (_ND_FEATURES / 2.0)) * n_data)
    out = ops.kde16_sum(query, train, bandwidth, out_scale=norm)
    _finish(dev, synchronize)
    return out


def gaussian_kde_triton_nd_numpy(data, queries, bandwidth: float, *, device="cuda") -> np.ndarray:
    return gaussian_kde_triton_nd(data=data, queries=queries, bandwidth=bandwidth, device=device).detach().cpu().numpy()


def gaussian_kde_score_triton(
    data: Sequence[float] | torch.Tensor,
    queries: Sequence[float] | torch.Tensor,
    bandwidth: float,
    *,
    block_m: int = 128,
    block_n: int = 128,
    num_warps: int = 4,
    num_stages: int = 2,
    device: str | torch.device = "cuda",
    synchronize: bool = True,
) -> tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    """(score, pdf, deriv) of the 1-D KDE at `queries`; score = deriv/(pdf + 1e-12)."""
    if bandwidth <= 0:
        raise ValueError("bandwidth must be positive.")
    dev = _check_cuda(device, "gaussian_kde_score_triton")
    train = _to_torch_tensor(data, dev).reshape(-1)
    query = _to_torch_tensor(queries, dev).reshape(-1)
    if train.numel() == 0 or query.numel() == 0:
        raise ValueError("data and queries must contain at least one sample.")
    res = ops.kde1d_score(query, train, bandwidth)
    _finish(dev, synchronize)
    return res
