"""Input conversion helpers (kernels/flash_sd_kde/common.py:17-41 of the reference).

The reference's grid-promotion helper exists because its Triton grids are
bounded by gridDim limits; the GB300 kernels use persistent grids sized to
the SM count, so no promotion (and no RuntimeWarning) is ever needed.
"""
from __future__ import annotations

from typing import Sequence

import torch

from fsk import ops

_ND_FEATURES = 16


def _to_torch_tensor(array_like: Sequence[float] | torch.Tensor, device: torch.device) -> torch.Tensor:
    if isinstance(array_like, torch.Tensor):
        t = array_like.to(device=device, dtype=torch.float32, copy=False)
    else:
        t = torch.as_tensor(array_like, dtype=torch.float32, device=device)
    return t.contiguous()


def _to_matrix_tensor(array_like, device: torch.device, *, dim: int) -> torch.Tensor:
    return ops.as_matrix(array_like, device, dim)


def _check_cuda(device, name: str) -> torch.device:
    dev = torch.device(device)
    if dev.type != "cuda":
        raise ValueError(f"{name} requires a CUDA device.")
    if not torch.cuda.is_available():
        raise RuntimeError(f"CUDA is not available but was requested for {name}.")
    return ops._device(dev)
