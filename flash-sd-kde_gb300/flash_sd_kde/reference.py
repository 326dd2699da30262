"""Bandwidth rules, samplers and numpy-in/numpy-out evaluators with the names of
the reference's flash_sd_kde/reference.py.

Unlike the reference module (a CPU numpy implementation), every evaluator
here runs on the GPU through the fsk kernels and returns numpy arrays, so code
written against the reference's names keeps working on GB300.  The samplers
are plain numpy data generators (reference.py:8-21, :144-168).
"""
from __future__ import annotations

import math
from typing import Tuple

import numpy as np
import torch

from fsk import ops
from globals import DEFAULT_EPS, ND_FEATURES

mixture_params_list = [
    {"pi": 0.4, "mu1": -2, "sigma1": 0.5, "mu2": 2, "sigma2": 1.0},
    {"pi": 0.3, "mu1": -2, "sigma1": 0.4, "mu2": 4, "sigma2": 1.5},
    {"pi": 0.5, "mu1": 0, "sigma1": 0.4, "mu2": 1.5, "sigma2": 1.5},
]


def _dev() -> torch.device:
    return ops._device("cuda")


def _np32(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=np.float32))


def sample_from_mixture(n: int, params: dict[str, float]) -> np.ndarray:
    z = np.random.rand(n) < params["pi"]
    out = np.zeros(n)
    out[z] = np.random.normal(params["mu1"], params["sigma1"], size=z.sum())
    out[~z] = np.random.normal(params["mu2"], params["sigma2"], size=(~z).sum())
    return out


def sample_gaussian_mixture_16d(n: int, *, pi: float = 0.5, mean_offset: float = 1.5,
                                sigma1: float = 0.5, sigma2: float = 1.0) -> np.ndarray:
    """Isotropic two-component Gaussian mixture in 16 dimensions (float32)."""
    if not (0.0 < pi < 1.0):
        raise ValueError("pi must lie in (0, 1).")
    z = np.random.rand(n) < pi
    out = np.empty((n, 16), dtype=np.float32)
    n1 = int(z.sum())
    if n1:
        out[z] = np.random.normal(loc=-mean_offset, scale=sigma1, size=(n1, 16)).astype(np.float32)
    if n - n1:
        out[~z] = np.random.normal(loc=mean_offset, scale=sigma2, size=(n - n1, 16)).astype(np.float32)
    return out


def silverman_bandwidth(data: np.ndarray) -> float:
    x = _np32(data)
    if x.ndim != 1:
        raise ValueError("data must be 1D for silverman_bandwidth.")
    if x.size == 0:
        raise ValueError("data must contain at least one element.")
    return float(ops.silverman(torch.from_numpy(x).to(_dev())).item())


def silverman_bandwidth_1d(data: np.ndarray) -> float:
    return silverman_bandwidth(data)


def silverman_bandwidth_nd(data: np.ndarray) -> float:
    x = _np32(data)
    if x.ndim != 2:
        raise ValueError("data must be 2D for silverman_bandwidth_nd.")
    if x.shape[0] == 0:
        raise ValueError("data must contain at least one element.")
    return float(ops.silverman(torch.from_numpy(x).to(_dev())).item())


def kde_eval_1d_numpy(queries: np.ndarray, data: np.ndarray, bandwidth: float) -> np.ndarray:
    if bandwidth <= 0:
        raise ValueError("bandwidth must be positive.")
    d = _np32(data).reshape(-1)
    if d.size == 0:
        raise ValueError("data must contain at least one element.")
    dev = _dev()
    scale = 1.0 / (math.sqrt(2.0 * math.pi) * d.size * bandwidth)
    return ops.kde1d_sum(torch.from_numpy(_np32(queries).reshape(-1)).to(dev), torch.from_numpy(d).to(dev),
                         bandwidth, out_scale=scale).cpu().numpy()


def kde_eval_1d_linearized_numpy(queries: np.ndarray, data: np.ndarray, bandwidth: float) -> np.ndarray:
    if bandwidth <= 0:
        raise ValueError("bandwidth must be positive.")
    d = _np32(data).reshape(-1)
    if d.size == 0:
        raise ValueError("data must contain at least one element.")
    dev = _dev()
    scale = 1.0 / (math.sqrt(2.0 * math.pi) * d.size * bandwidth)
    return ops.kde1d_sum(torch.from_numpy(_np32(queries).reshape(-1)).to(dev), torch.from_numpy(d).to(dev),
                         bandwidth, laplace=True, out_scale=scale).cpu().numpy()


def _nd(queries, data, bandwidth, laplace: bool) -> np.ndarray:
    x, d = _np32(queries), _np32(data)
    if x.ndim != 2 or d.ndim != 2:
        raise ValueError("queries and data must be 2D arrays.")
    if x.shape[1] != d.shape[1]:
        raise ValueError("queries and data must share feature dimension.")
    if bandwidth <= 0:
        raise ValueError("bandwidth must be positive.")
    if d.shape[0] == 0:
        raise ValueError("data must contain at least one element.")
    dim = d.shape[1]
    norm = 1.0 / ((2.0 * math.pi) ** (dim / 2.0) * (bandwidth ** dim) * d.shape[0])
    dev = _dev()
    return ops.kde16_sum(torch.from_numpy(x).to(dev), torch.from_numpy(d).to(dev), bandwidth, laplace=laplace,
                         out_scale=norm).cpu().numpy()


def kde_eval_nd_numpy(queries: np.ndarray, data: np.ndarray, bandwidth: float) -> np.ndarray:
    return _nd(queries, data, bandwidth, False)


def kde_eval_nd_linearized_numpy(queries: np.ndarray, data: np.ndarray, bandwidth: float) -> np.ndarray:
    return _nd(queries, data, bandwidth, True)


def empirical_score_nd_numpy(data: np.ndarray, bandwidth: float, *, eps: float = DEFAULT_EPS
                             ) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    x = _np32(data)
    if x.ndim != 2:
        raise ValueError("data must be 2D.")
    if x.shape[1] != ND_FEATURES:
        raise ValueError(f"expected {ND_FEATURES} features, got {x.shape[1]}.")
    if bandwidth <= 0:
        raise ValueError("bandwidth must be positive.")
    t = torch.from_numpy(x).to(_dev())
    pdf, w = ops.empscore16(t, bandwidth, variant="ordered")
    _, score = ops.debias16(t, pdf, w, bandwidth, eps, return_score=True)
    return pdf.cpu().numpy(), w.cpu().numpy(), score.cpu().numpy()


def empirical_sd_kde_transform_nd_numpy(data: np.ndarray, bandwidth: float, *, eps: float = DEFAULT_EPS) -> np.ndarray:
    x = _np32(data)
    t = torch.from_numpy(x).to(_dev())
    pdf, w = ops.empscore16(t, bandwidth, variant="ordered")
    return ops.debias16(t, pdf, w, bandwidth, eps).cpu().numpy()
