"""16-D KDE row sums: drop-in for kernels/kde_eval_16d_stream_splitk.py.

Both backends return the *unnormalised* sum_j exp(-||q_i - x_j||^2 / (2h^2))
(optionally Laplace-corrected) like the reference's pass A + reduce
(kde_eval_16d_stream_splitk.py:263-370, :373-452).  ``splitk_stream`` reduces
the data splits from an ordered FP64 partial buffer; ``atomic`` adds them with
FP64 atomics.  ``use_precomputed_norms`` and ``autotune`` are accepted for
compatibility: norms are always precomputed and the tile shape is fixed by
the tensor-core mapping.
"""
from __future__ import annotations

from typing import Sequence

import torch

from fsk import ops
from globals import ND_FEATURES, PRECISION_FAST_TF32, PRECISION_FP32_IEEE


def _precision(precision_mode: str) -> str:
    if precision_mode not in {PRECISION_FAST_TF32, PRECISION_FP32_IEEE}:
        raise ValueError(f"invalid precision_mode {precision_mode}.")
    return "ieee" if precision_mode == PRECISION_FP32_IEEE else "tensor"


def _to_matrix_tensor(array_like: Sequence[Sequence[float]] | torch.Tensor, device: torch.device) -> torch.Tensor:
    return ops.as_matrix(array_like, device, ND_FEATURES)


def kde_eval_16d_splitk(
    data,
    queries,
    bandwidth: float,
    *,
    device: torch.device,
    precision_mode: str,
    use_precomputed_norms: bool,
    autotune: bool,
    apply_laplacian_correction: bool = False,
) -> torch.Tensor:
    if bandwidth <= 0:
        raise ValueError("bandwidth must be positive.")
    device = ops._device(device)
    train = _to_matrix_tensor(data, device)
    query = _to_matrix_tensor(queries, device)
    if train.shape[0] == 0 or query.shape[0] == 0:
        raise ValueError("data and queries must be non-empty.")
    prec = _precision(precision_mode)
    return ops.kde16_sum(query, train, bandwidth, precision=prec, laplace=apply_laplacian_correction)


def kde_eval_16d_atomic(
    data,
    queries,
    bandwidth: float,
    *,
    device: torch.device,
    precision_mode: str,
    use_precomputed_norms: bool,
    block_m: int = 64,
    block_n: int = 64,
    autotune: bool = False,
    apply_laplacian_correction: bool = False,
) -> torch.Tensor:
    if bandwidth <= 0:
        raise ValueError("bandwidth must be positive.")
    device = ops._device(device)
    train = _to_matrix_tensor(data, device)
    query = _to_matrix_tensor(queries, device)
    if train.shape[0] == 0 or query.shape[0] == 0:
        raise ValueError("data and queries must be non-empty.")
    prec = _precision(precision_mode)
    return ops.kde16_sum(query, train, bandwidth, precision=prec, laplace=apply_laplacian_correction, atomic=True)
