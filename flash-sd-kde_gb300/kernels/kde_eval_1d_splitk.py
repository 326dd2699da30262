"""1-D KDE row sums: drop-in for kernels/kde_eval_1d_splitk.py:141-256.

Returns the unnormalised sum_j exp(-(q_i - x_j)^2 / (2h^2)) (Laplace factor
1.5 - z^2/2 with ``apply_laplacian_correction``).
"""
from __future__ import annotations

import torch

from fsk import ops


def _to_torch_tensor_1d(array_like, device: torch.device) -> torch.Tensor:
    try:
        return ops.as_vector(array_like, device)
    except ValueError:
        raise ValueError("expected 1D tensor for KDE eval.") from None


def kde_eval_1d_splitk(
    data,
    queries,
    bandwidth: float,
    *,
    device: torch.device,
    autotune: bool,
    apply_laplacian_correction: bool = False,
) -> torch.Tensor:
    if bandwidth <= 0:
        raise ValueError("bandwidth must be positive.")
    device = ops._device(device)
    train = _to_torch_tensor_1d(data, device)
    query = _to_torch_tensor_1d(queries, device)
    if train.numel() == 0 or query.numel() == 0:
        raise ValueError("data and queries must be non-empty.")
    return ops.kde1d_sum(query, train, bandwidth, laplace=apply_laplacian_correction)


def kde_eval_1d_atomic(
    data,
    queries,
    bandwidth: float,
    *,
    device: torch.device,
    block_m: int = 128,
    block_n: int = 128,
    apply_laplacian_correction: bool = False,
) -> torch.Tensor:
    if bandwidth <= 0:
        raise ValueError("bandwidth must be positive.")
    device = ops._device(device)
    train = _to_torch_tensor_1d(data, device)
    query = _to_torch_tensor_1d(queries, device)
    if train.numel() == 0 or query.numel() == 0:
        raise ValueError("data and queries must be non-empty.")
    return ops.kde1d_sum(query, train, bandwidth, laplace=apply_laplacian_correction, atomic=True)
