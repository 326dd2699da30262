"""Split-K partial reductions: drop-in for kernels/reduce_partials.py.

``reduce_pdf_partials`` sums a (n_splits, n_query) buffer over splits and
``reduce_weighted_partials`` a (n_splits, n_query, features) buffer, in FP64
and in split order (the reference sums in FP32).  Non-CUDA tensors are
rejected: there is no host path.
"""
from __future__ import annotations

import torch

from fsk import _lib as L


def _reduce(partials: torch.Tensor, out_shape) -> torch.Tensor:
    if partials.device.type != "cuda":
        raise ValueError("partials must be a CUDA tensor.")
    p = partials.to(dtype=torch.float32).contiguous()
    splits = p.shape[0]
    count = p[0].numel() if splits else 0
    out = torch.empty(out_shape, dtype=torch.float32, device=p.device)
    if splits == 0:
        return out.zero_()
    with torch.cuda.device(p.device):
        st = L.load().fsk_reduce_partials(p.data_ptr(), splits, count, out.data_ptr(),
                                          torch.cuda.current_stream(p.device).cuda_stream)
    L.check(st, "fsk_reduce_partials")
    return out


def reduce_pdf_partials(partials: torch.Tensor, *, block_m: int = 256) -> torch.Tensor:
    if partials.ndim != 2:
        raise ValueError("partials must be 2D (n_splits, n_query).")
    return _reduce(partials, (partials.shape[1],))


def reduce_weighted_partials(partials: torch.Tensor, *, block_m: int = 128) -> torch.Tensor:
    if partials.ndim != 3:
        raise ValueError("partials must be 3D (n_splits, n_query, features).")
    return _reduce(partials, (partials.shape[1], partials.shape[2]))
