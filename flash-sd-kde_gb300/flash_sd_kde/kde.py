"""Dispatch / public functional API: drop-in for flash_sd_kde/kde.py.

kde_eval                      route by ndim and backend, normalise   (reference :49-124)
kde_eval_linearized           Laplace-corrected KDE, fused           (reference :127-149)
kde_eval_linearized_nonfused  same quantity (see its docstring)      (reference :152-255)
emp_sd_kde_fit_transform      score backends + debias shift          (reference :258-326)

2-D inputs may have any 1 <= d <= 64 features (an addition: the reference
requires exactly 16).  Up to 16 the rows are zero-padded to 16 (which leaves
every squared distance unchanged) and take the 16-D kernels; above 16 the
CUDA-core kernels for any d (fp32_ieee arithmetic) run.  The normalisation
uses d.
"""
from __future__ import annotations

import math
from typing import Sequence, Tuple

import numpy as np
import torch

from flash_sd_kde.config import (
    DEFAULT_HEURISTICS,
    select_emp_score_backend,
    validate_emp_score_backend,
    validate_kde_backend,
    validate_precision_mode,
)
from fsk import ops
from globals import (
    DEFAULT_EMP_SCORE_BACKEND,
    DEFAULT_EPS,
    DEFAULT_KDE_BACKEND,
    DEFAULT_PRECISION_MODE,
    EMP_SCORE_BACKEND_FLASH_SD_KDE,
    EMP_SCORE_BACKEND_ORDERED_SPLITK,
    EMP_SCORE_BACKEND_SYMMETRIC_ATOMIC,
    KDE_BACKEND_ATOMIC,
    KDE_BACKEND_SPLITK_STREAM,
    ND_FEATURES,
    PRECISION_FP32_IEEE,
)


def _infer_ndim(data) -> int:
    if isinstance(data, (torch.Tensor, np.ndarray)):
        return data.ndim
    if len(data) == 0:
        return 1
    first = data[0]
    if isinstance(first, (list, tuple, np.ndarray)):
        return 2
    return 1


def _n_features(data) -> int:
    """Columns of 2-D input (0 when it has no second axis)."""
    if isinstance(data, (torch.Tensor, np.ndarray)):
        return int(data.shape[1]) if data.ndim == 2 else 0
    return len(data[0]) if len(data) and isinstance(data[0], (list, tuple, np.ndarray)) else 0


def _n_rows(data) -> int:
    return data.shape[0] if isinstance(data, (torch.Tensor, np.ndarray)) else len(data)


def _require_cuda(device, name: str) -> torch.device:
    device = torch.device(device)
    if device.type != "cuda":
        raise ValueError(f"{name} currently expects a CUDA device.")
    if not torch.cuda.is_available():
        raise RuntimeError("CUDA is not available but was requested.")
    return ops._device(device)


def _kde_eval_impl(data, queries, bandwidth, *, device, precision_mode, kde_backend,
                   apply_laplacian_correction, log_eps=None, log_exact=False):
    validate_precision_mode(precision_mode)
    validate_kde_backend(kde_backend)
    if bandwidth <= 0:
        raise ValueError("bandwidth must be positive.")
    device = _require_cuda(device, "kde_eval")
    atomic = kde_backend == KDE_BACKEND_ATOMIC
    ndim = _infer_ndim(data)
    if ndim == 1:
        if log_exact:
            raise ValueError("exact log-densities are available for 16-D data only.")
        train = ops.as_vector(data, device)
        query = ops.as_vector(queries, device)
        n_data = train.numel()
        if n_data == 0 or query.numel() == 0:
            raise ValueError("data and queries must be non-empty.")
        scale = 1.0 / (math.sqrt(2.0 * math.pi) * bandwidth) / n_data
        return ops.kde1d_sum(query, train, bandwidth, laplace=apply_laplacian_correction, atomic=atomic,
                             out_scale=scale, log_eps=log_eps)
    if ndim == 2:
        d = _n_features(data)
        # more than 16 features, or the Laplace factor 1 + d/2 - dist/(2h^2)
        # for d != 16 (the 16-D kernels build in d = 16): CUDA-core kernels for any d
        if d > ND_FEATURES or (apply_laplacian_correction and d != ND_FEATURES):
            if log_exact:
                raise ValueError(f"exact log-densities are available for up to {ND_FEATURES} features.")
            train, query = ops._as_rows(data, device), ops._as_rows(queries, device)
            if query.shape[1] != d:
                raise ValueError(f"data has {d} features but queries have {query.shape[1]}.")
            if train.shape[0] == 0 or query.shape[0] == 0:
                raise ValueError("data and queries must be non-empty.")
            norm = 1.0 / ((2.0 * math.pi) ** (d / 2.0) * (bandwidth ** d) * train.shape[0])
            return ops.kde_nd_sum(query, train, bandwidth, laplace=apply_laplacian_correction, out_scale=norm,
                                  log_eps=log_eps)
        train, d = ops.as_padded_matrix(data, device, ND_FEATURES)
        query, dq = ops.as_padded_matrix(queries, device, ND_FEATURES)
        if dq != d:
            raise ValueError(f"data has {d} features but queries have {dq}.")
        n_data = train.shape[0]
        if n_data == 0 or query.shape[0] == 0:
            raise ValueError("data and queries must be non-empty.")
        norm = 1.0 / ((2.0 * math.pi) ** (d / 2.0) * (bandwidth ** d) * n_data)
        prec = "ieee" if precision_mode == PRECISION_FP32_IEEE else "tensor"
        return ops.kde16_sum(query, train, bandwidth, precision=prec, laplace=apply_laplacian_correction,
                             atomic=atomic, out_scale=norm, log_eps=None if log_exact else log_eps,
                             log_exact=log_exact)
    raise ValueError("data must be 1D or 2D.")


def kde_eval(
    data: Sequence[float] | Sequence[Sequence[float]] | torch.Tensor,
    queries: Sequence[float] | Sequence[Sequence[float]] | torch.Tensor,
    bandwidth: float,
    *,
    device: str | torch.device = "cuda",
    precision_mode: str = DEFAULT_PRECISION_MODE,
    kde_backend: str = DEFAULT_KDE_BACKEND,
    use_precomputed_norms: bool = True,
    autotune: bool = True,
    apply_laplacian_correction: bool = False,
) -> torch.Tensor:
    """Evaluate a Gaussian KDE (1-D or 16-D) or its Laplacian-corrected variant."""
    return _kde_eval_impl(data, queries, bandwidth, device=device, precision_mode=precision_mode,
                          kde_backend=kde_backend, apply_laplacian_correction=apply_laplacian_correction)


def kde_eval_log(data, queries, bandwidth: float, *, eps: float = DEFAULT_EPS, device="cuda",
                 precision_mode: str = DEFAULT_PRECISION_MODE, kde_backend: str = DEFAULT_KDE_BACKEND) -> torch.Tensor:
    """log(kde_eval(...) + eps) with the log taken in FP64 inside the reduction
    (what FlashSDKDE.score_samples returns, flash_sd_kde/estimator.py:104-115).

    eps = 0 (16-D): the exact log-density, also where the density underflows
    FP32 (out-of-support queries are recomputed with a running-minimum shift
    and the log is assembled in FP64), instead of log(0) = -inf.
    """
    if eps < 0:
        raise ValueError("eps must be non-negative.")
    return _kde_eval_impl(data, queries, bandwidth, device=device, precision_mode=precision_mode,
                          kde_backend=kde_backend, apply_laplacian_correction=False, log_eps=float(eps),
                          log_exact=eps == 0)


def kde_eval_linearized(
    data,
    queries,
    bandwidth: float,
    *,
    device: str | torch.device = "cuda",
    precision_mode: str = DEFAULT_PRECISION_MODE,
    kde_backend: str = DEFAULT_KDE_BACKEND,
    use_precomputed_norms: bool = True,
    autotune: bool = True,
) -> torch.Tensor:
    """Linearized Emp-SD-KDE approximation K - (h^2/2) Laplacian(K), fused in the kernel."""
    return kde_eval(data, queries, bandwidth, device=device, precision_mode=precision_mode,
                    kde_backend=kde_backend, use_precomputed_norms=use_precomputed_norms, autotune=autotune,
                    apply_laplacian_correction=True)


def kde_eval_linearized_nonfused(
    data,
    queries,
    bandwidth: float,
    *,
    device: str | torch.device = "cuda",
    precision_mode: str = DEFAULT_PRECISION_MODE,
    kde_backend: str = DEFAULT_KDE_BACKEND,
    use_precomputed_norms: bool = True,
    autotune: bool = True,
    chunk_size: int | None = None,
) -> torch.Tensor:
    """The linearized KDE.  The reference computes it as base*(1+d/2) -
    norm/2 * sum phi*dist/h^2 in a second, torch-only pass to measure the gain
    of fusion; the value is identical to kde_eval_linearized, which is what is
    returned here (one fused launch).  ``chunk_size`` is accepted and unused."""
    if bandwidth <= 0:
        raise ValueError("bandwidth must be positive.")
    return kde_eval_linearized(data, queries, bandwidth, device=device, precision_mode=precision_mode,
                               kde_backend=kde_backend, use_precomputed_norms=use_precomputed_norms,
                               autotune=autotune)


def emp_sd_kde_fit_transform(
    data: Sequence[Sequence[float]] | torch.Tensor,
    bandwidth: float,
    *,
    device: str | torch.device = "cuda",
    precision_mode: str = DEFAULT_PRECISION_MODE,
    emp_score_backend: str | None = None,
    use_precomputed_norms: bool = True,
    autotune: bool = True,
    eps: float = DEFAULT_EPS,
    return_debug: bool = False,
) -> torch.Tensor | Tuple[torch.Tensor, torch.Tensor, torch.Tensor, torch.Tensor]:
    """One-step empirical SD-KDE: x + h^2/2 * (W/(pdf+eps) - x)/h^2."""
    if bandwidth <= 0:
        raise ValueError("bandwidth must be positive.")
    validate_precision_mode(precision_mode)
    if emp_score_backend is None:
        emp_score_backend = select_emp_score_backend(_n_rows(data), heuristics=DEFAULT_HEURISTICS)
    validate_emp_score_backend(emp_score_backend)
    device = _require_cuda(device, "emp_sd_kde_fit_transform")
    if _n_features(data) > ND_FEATURES:
        train = ops._as_rows(data, device)
        if train.shape[0] == 0:
            raise ValueError("data must be non-empty.")
        pdf_sum, weighted_sum = ops.empscore_nd(train, bandwidth)
        if return_debug:
            debiased, score = ops.debias_nd(train, pdf_sum, weighted_sum, bandwidth, eps, return_score=True)
            return debiased, pdf_sum, weighted_sum, score
        return ops.debias_nd(train, pdf_sum, weighted_sum, bandwidth, eps)
    train, d = ops.as_padded_matrix(data, device, ND_FEATURES)
    if train.shape[0] == 0:
        raise ValueError("data must be non-empty.")
    prec = "ieee" if precision_mode == PRECISION_FP32_IEEE else "tensor"
    if emp_score_backend == EMP_SCORE_BACKEND_SYMMETRIC_ATOMIC:
        pdf_sum, weighted_sum = ops.empscore16(train, bandwidth, variant="symmetric", precision=prec)
    else:
        pdf_sum, weighted_sum = ops.empscore16(
            train, bandwidth, variant="ordered", precision=prec,
            feature_major=emp_score_backend == EMP_SCORE_BACKEND_FLASH_SD_KDE)
    if return_debug:
        debiased, score = ops.debias16(train, pdf_sum, weighted_sum, bandwidth, eps, return_score=True)
        if d < ND_FEATURES:   # the padded columns are 0 in every output
            return debiased[:, :d].contiguous(), pdf_sum, weighted_sum[:, :d], score[:, :d].contiguous()
        return debiased, pdf_sum, weighted_sum, score
    debiased = ops.debias16(train, pdf_sum, weighted_sum, bandwidth, eps)
    return debiased[:, :d].contiguous() if d < ND_FEATURES else debiased


def sd_kde_eval(
    data,
    queries,
    bandwidth: float,
    *,
    device: str | torch.device = "cuda",
    precision_mode: str = DEFAULT_PRECISION_MODE,
    eps: float = DEFAULT_EPS,
    return_debiased: bool = False,
):
    """One-step empirical SD-KDE of `data` evaluated at `queries` in one
    library call: the same values as
    kde_eval(emp_sd_kde_fit_transform(data, h, emp_score_backend="ordered_splitk"), queries, h)
    (the reference runs these as two calls; flash_sd_kde/kde.py:49, :258).
    16-D inputs only."""
    if bandwidth <= 0:
        raise ValueError("bandwidth must be positive.")
    validate_precision_mode(precision_mode)
    device = _require_cuda(device, "sd_kde_eval")
    train = ops.as_matrix(data, device, ND_FEATURES)
    query = ops.as_matrix(queries, device, ND_FEATURES)
    if train.shape[0] == 0 or query.shape[0] == 0:
        raise ValueError("data and queries must be non-empty.")
    prec = "ieee" if precision_mode == PRECISION_FP32_IEEE else "tensor"
    return ops.sdkde16(train, query, bandwidth, precision=prec, eps=eps, return_debiased=return_debiased)
