"""FP32 numpy restatement of the reference's CPU implementation of the path.

Each function follows the cited function of the reference project's
flash_sd_kde/reference.py step by step (same FP32 arithmetic order per
element); evaluation is blocked over the data/query axes so sizes beyond a
single dense matrix still fit in memory.  Test infrastructure only.
"""
from __future__ import annotations

import math

import numpy as np

DEFAULT_EPS = 1e-12
ND = 16


def _f32(a) -> np.ndarray:
    return np.asarray(a, dtype=np.float32)


def silverman_bandwidth(data) -> float:
    """reference.py:24-36 -- 1-D Silverman rule with float32 statistics."""
    x = _f32(data)
    if x.ndim != 1:
        raise ValueError("data must be 1D")
    n = x.size
    if n == 0:
        raise ValueError("empty")
    sd = float(np.std(x))
    q75, q25 = np.percentile(x, 75), np.percentile(x, 25)
    sigma = min(sd, float(q75 - q25) / 1.34)
    if sigma <= 0:
        sigma = 1.0
    return float(0.9 * sigma * n ** (-1.0 / 5.0))


def silverman_bandwidth_nd(data) -> float:
    """reference.py:171-184 -- per-axis min(std, IQR/1.34), averaged."""
    x = _f32(data)
    if x.ndim != 2:
        raise ValueError("data must be 2D")
    n, d = x.shape
    if n == 0:
        raise ValueError("empty")
    sd = np.std(x, axis=0)
    q = np.percentile(x, [75, 25], axis=0)
    iqr = (q[0] - q[1]) / 1.34
    sigma = float(np.mean(np.minimum(sd, iqr)))
    if sigma <= 0:
        sigma = 1.0
    return float(0.9 * sigma * n ** (-1.0 / (d + 4)))


def sdkde_1d_bandwidth(data) -> float:
    """kernels/flash_sd_kde/empirical.py:328-333 -- h = 0.4 sigma n^(-1/9)."""
    x = _f32(data).reshape(-1)
    sd = float(x.std())
    iqr = float(np.percentile(x, 75) - np.percentile(x, 25))
    sigma = min(sd, iqr / 1.34)
    return 0.4 * sigma * (x.size ** (-1 / 9))


def _nd_rowsums(q: np.ndarray, d: np.ndarray, h: float, laplace: bool, block: int = 4096) -> np.ndarray:
    """sum_j phi over data blocks; per element the FP32 steps of
    reference.py:227-232 (or :250-258 with the Laplace factor)."""
    inv_h2 = 1.0 / (h * h)
    qn = (q * q).sum(axis=1, keepdims=True)
    out = np.zeros(q.shape[0], dtype=np.float32)
    for s in range(0, d.shape[0], block):
        db = d[s:s + block]
        dn = (db * db).sum(axis=1, keepdims=True).T
        dist = qn + dn - 2.0 * (q @ db.T)
        dist = np.maximum(dist, 0.0)
        if laplace:
            scaled = dist * inv_h2
            phi = np.exp(-0.5 * scaled) * (1.0 + 0.5 * q.shape[1] - 0.5 * scaled)
        else:
            phi = np.exp(-0.5 * dist * inv_h2)
        out += phi.sum(axis=1)
    return out


def kde_eval_nd_numpy(queries, data, bandwidth: float) -> np.ndarray:
    """reference.py:216-235 -- normalised d-D Gaussian KDE."""
    x, d = _f32(queries), _f32(data)
    if x.ndim != 2 or d.ndim != 2 or x.shape[1] != d.shape[1]:
        raise ValueError("bad shapes")
    if bandwidth <= 0 or d.shape[0] == 0:
        raise ValueError("bad bandwidth or empty data")
    dim = d.shape[1]
    norm = 1.0 / ((2.0 * math.pi) ** (dim / 2.0) * (bandwidth ** dim) * d.shape[0])
    return norm * _nd_rowsums(x, d, bandwidth, False)


def kde_eval_nd_linearized_numpy(queries, data, bandwidth: float) -> np.ndarray:
    """reference.py:238-260 -- Laplace-corrected ("linearized") d-D KDE."""
    x, d = _f32(queries), _f32(data)
    dim = d.shape[1]
    norm = 1.0 / ((2.0 * math.pi) ** (dim / 2.0) * (bandwidth ** dim) * d.shape[0])
    return norm * _nd_rowsums(x, d, bandwidth, True)


def kde_eval_1d_numpy(queries, data, bandwidth: float, *, laplace: bool = False, block: int = 8192) -> np.ndarray:
    """reference.py:187-197 (and :200-213 with laplace=True)."""
    x, d = _f32(queries).reshape(-1), _f32(data).reshape(-1)
    if bandwidth <= 0 or d.size == 0:
        raise ValueError("bad bandwidth or empty data")
    hb = np.float32(bandwidth)
    acc = np.zeros(x.size, dtype=np.float32)
    for s in range(0, d.size, block):
        diff = (x[:, None] - d[None, s:s + block]) / hb
        if laplace:
            sc = diff * diff
            phi = np.exp(-0.5 * sc) * (1.0 + 0.5 - 0.5 * sc)
        else:
            phi = np.exp(-0.5 * diff * diff)
        acc += phi.sum(axis=1)
    inv_norm = 1.0 / (math.sqrt(2.0 * math.pi) * d.size * bandwidth)
    return inv_norm * acc


def kde_score_1d(queries, data, bandwidth: float, *, block: int = 4096):
    """kernels/flash_sd_kde/kde.py:191-232 + :566-569 semantics (and
    reference.py:83-122): returns (score, pdf, deriv)."""
    x, d = _f32(queries).reshape(-1), _f32(data).reshape(-1)
    inv_h = np.float32(1.0) / np.float32(bandwidth)
    z_sum = np.zeros(x.size, dtype=np.float32)
    dz_sum = np.zeros(x.size, dtype=np.float32)
    for s in range(0, d.size, block):
        diff = (x[:, None] - d[None, s:s + block]) * inv_h
        phi = np.exp(np.float32(-0.5) * diff * diff)
        z_sum += phi.sum(axis=1)
        dz_sum += (-diff * phi).sum(axis=1)
    c = np.float32(1.0 / math.sqrt(2.0 * math.pi))
    pdf = (c * z_sum) / np.float32(d.size * bandwidth)
    deriv = (c * dz_sum) / np.float32(d.size * bandwidth * bandwidth)
    return deriv / (pdf + np.float32(1e-12)), pdf, deriv


def empirical_score_nd_numpy(data, bandwidth: float, *, eps: float = DEFAULT_EPS, block: int = 4096):
    """reference.py:263-284 -- (pdf_sum, weighted, score), self-pair included."""
    x = _f32(data)
    if x.ndim != 2 or x.shape[1] != ND:
        raise ValueError("expected (n, 16)")
    if bandwidth <= 0:
        raise ValueError("bandwidth must be positive")
    inv_h2 = 1.0 / (bandwidth * bandwidth)
    xn = (x * x).sum(axis=1, keepdims=True)
    pdf = np.zeros(x.shape[0], dtype=np.float32)
    w = np.zeros_like(x)
    for s in range(0, x.shape[0], block):
        xb = x[s:s + block]
        dist = xn + xn[s:s + block].T - 2.0 * (x @ xb.T)
        dist = np.maximum(dist, 0.0)
        phi = np.exp(-0.5 * dist * inv_h2)
        pdf += phi.sum(axis=1)
        w += phi @ xb
    score = (w / (pdf[:, None] + eps) - x) * inv_h2
    return pdf, w, score


def empirical_sd_kde_transform_nd_numpy(data, bandwidth: float, *, eps: float = DEFAULT_EPS) -> np.ndarray:
    """reference.py:287-295 -- x + (h^2/2) * score."""
    _, _, score = empirical_score_nd_numpy(data, bandwidth, eps=eps)
    return _f32(data) + 0.5 * (bandwidth ** 2) * score
