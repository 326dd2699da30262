"""FP64 log-space ground truth -- test infrastructure only.

Restates experiments/error_suite_16d/reference.py:32-82 of the reference
project: log p(y) = logsumexp_j(-||y - x_j||^2 / (2h^2)) + log_const with
log_const = -log n - d log h - (d/2) log(2 pi), accumulated chunk by chunk
with a running logaddexp.  The distance is formed from direct FP64
differences (exact enough that the FP64 expansion's cancellation does not
matter).  Also FP64 versions of the empirical score and the debias shift.
"""
from __future__ import annotations

import math

import numpy as np


def _logaddexp(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    return np.logaddexp(a, b)


def log_density(samples, queries, bandwidth: float, *, laplace: bool = False,
                q_chunk: int = 512, s_chunk: int = 8192) -> np.ndarray:
    """FP64 log-density of the Gaussian KDE (reference :32-82).  With
    laplace=True returns log |sum phi (1 + d/2 - dist/(2h^2))| (the corrected
    sum can be negative; tests compare densities for that case)."""
    x = np.asarray(samples, dtype=np.float64)
    q = np.asarray(queries, dtype=np.float64)
    if x.ndim == 1:
        x = x[:, None]
    if q.ndim == 1:
        q = q[:, None]
    n, d = x.shape
    log_const = -math.log(n) - d * math.log(bandwidth) - 0.5 * d * math.log(2.0 * math.pi)
    out = np.empty(q.shape[0], dtype=np.float64)
    inv2h2 = 1.0 / (2.0 * bandwidth * bandwidth)
    for qs in range(0, q.shape[0], q_chunk):
        qb = q[qs:qs + q_chunk]
        run = np.full(qb.shape[0], -np.inf)
        lap = np.zeros(qb.shape[0]) if laplace else None
        for ss in range(0, n, s_chunk):
            xb = x[ss:ss + s_chunk]
            dist = np.zeros((qb.shape[0], xb.shape[0]))
            for k in range(d):
                diff = qb[:, k:k + 1] - xb[None, :, k]
                dist += diff * diff
            expo = -dist * inv2h2
            if laplace:
                lap += (np.exp(expo) * (1.0 + 0.5 * d + expo)).sum(axis=1)
            else:
                mx = expo.max(axis=1)
                lse = mx + np.log(np.exp(expo - mx[:, None]).sum(axis=1))
                run = _logaddexp(run, lse)
        out[qs:qs + q_chunk] = (np.log(np.abs(lap)) if laplace else run) + log_const
    return out


def log_density_gemm(samples, queries, bandwidth: float, *, threads: int | None = None,
                     q_chunk: int = 256, s_chunk: int = 1 << 16) -> np.ndarray:
    """FP64 log-density as log_density, for large sample sets: distances by
    the FP64 expansion |q-c|^2 + |x-c|^2 - 2 (q-c).(x-c) about the sample
    mean c (BLAS matmul; FP64 leaves ~1e-16 (|q-c|^2 + |x-c|^2) absolute
    error, far below the FP32 errors being measured), query chunks on a
    thread pool, the same chunked logsumexp and normalising constant."""
    import concurrent.futures as cf
    import os

    x = np.asarray(samples, dtype=np.float64)
    q = np.asarray(queries, dtype=np.float64)
    if x.ndim == 1:
        x = x[:, None]
    if q.ndim == 1:
        q = q[:, None]
    n, d = x.shape
    c = x.mean(axis=0)
    x = x - c
    q = q - c
    xn = (x * x).sum(axis=1)
    qn = (q * q).sum(axis=1)
    log_const = -math.log(n) - d * math.log(bandwidth) - 0.5 * d * math.log(2.0 * math.pi)
    inv2h2 = 1.0 / (2.0 * bandwidth * bandwidth)

    def work(qs: int) -> np.ndarray:
        qb = q[qs:qs + q_chunk]
        run = np.full(qb.shape[0], -np.inf)
        for ss in range(0, n, s_chunk):
            dist = qb @ x[ss:ss + s_chunk].T
            dist *= -2.0
            dist += qn[qs:qs + q_chunk, None]
            dist += xn[None, ss:ss + s_chunk]
            np.maximum(dist, 0.0, out=dist)
            dist *= -inv2h2
            mx = dist.max(axis=1)
            dist -= mx[:, None]
            np.exp(dist, out=dist)
            run = np.logaddexp(run, mx + np.log(dist.sum(axis=1)))
        return run

    starts = list(range(0, q.shape[0], q_chunk))
    with cf.ThreadPoolExecutor(max_workers=threads or os.cpu_count() or 1) as ex:
        parts = list(ex.map(work, starts))
    return np.concatenate(parts) + log_const if parts else np.zeros(0)


def log_error_metrics(logp, ref_logp) -> dict:
    """Log-density error statistics over the queries finite in both
    (restating experiments/error_suite_16d/metrics.py:18-55 of the reference):
    finite fractions, max / mean / p95 absolute log error, RMSE and bias."""
    a = np.asarray(logp, dtype=np.float64)
    b = np.asarray(ref_logp, dtype=np.float64)
    fa, fb = np.isfinite(a), np.isfinite(b)
    ok = fa & fb
    out = {"finite_fraction": float(fa.mean()), "finite_fraction_ref": float(fb.mean())}
    if not ok.any():
        return {**out, "max_abs_log_err": float("nan"), "mean_abs_log_err": float("nan"),
                "rmse_log_err": float("nan"), "p95_abs_log_err": float("nan"), "bias_log_err": float("nan")}
    diff = a[ok] - b[ok]
    ad = np.abs(diff)
    return {**out, "max_abs_log_err": float(ad.max()), "mean_abs_log_err": float(ad.mean()),
            "rmse_log_err": float(np.sqrt((diff * diff).mean())), "p95_abs_log_err": float(np.quantile(ad, 0.95)),
            "bias_log_err": float(diff.mean()),
            "max_rel_log_err": float((ad / np.maximum(np.abs(b[ok]), 1e-300)).max())}


def density(samples, queries, bandwidth: float, **kw) -> np.ndarray:
    return np.exp(log_density(samples, queries, bandwidth, **kw))


def empirical_score(data, bandwidth: float, *, eps: float = 1e-12, chunk: int = 2048):
    """FP64 (pdf_sum, weighted_sum, score) of reference.py:263-284."""
    x = np.asarray(data, dtype=np.float64)
    n = x.shape[0]
    pdf = np.zeros(n)
    w = np.zeros_like(x)
    inv2h2 = 1.0 / (2.0 * bandwidth * bandwidth)
    for s in range(0, n, chunk):
        xb = x[s:s + chunk]
        dist = np.zeros((n, xb.shape[0]))
        for k in range(x.shape[1]):
            diff = x[:, k:k + 1] - xb[None, :, k]
            dist += diff * diff
        phi = np.exp(-dist * inv2h2)
        pdf += phi.sum(axis=1)
        w += phi @ xb
    score = (w / (pdf[:, None] + eps) - x) / (bandwidth * bandwidth)
    return pdf, w, score


def empirical_score_rows(data, rows, bandwidth: float, *, chunk: int = 1 << 20):
    """FP64 (pdf_sum, weighted_sum) of reference.py:263-284 for the selected
    rows only (self pair included), against all n data points: the checker
    for sizes whose full n^2 oracle would not finish."""
    x = np.asarray(data, dtype=np.float64)
    r = np.asarray(rows, dtype=np.int64)
    inv2h2 = 1.0 / (2.0 * bandwidth * bandwidth)
    pdf = np.zeros(r.size)
    w = np.zeros((r.size, x.shape[1]))
    for i, row in enumerate(r):
        q = x[row]
        for s in range(0, x.shape[0], chunk):
            xb = x[s:s + chunk]
            dist = ((xb - q) ** 2).sum(axis=1)
            phi = np.exp(-dist * inv2h2)
            pdf[i] += phi.sum()
            w[i] += phi @ xb
    return pdf, w


def debias(data, bandwidth: float, *, eps: float = 1e-12) -> np.ndarray:
    _, _, score = empirical_score(data, bandwidth, eps=eps)
    return np.asarray(data, dtype=np.float64) + 0.5 * bandwidth * bandwidth * score


def silverman_nd(data) -> float:
    """Silverman rule with FP64 statistics (the reference's
    experiments/error_suite_16d/reference.py:16-29 silverman_diag_bandwidth)."""
    x = np.asarray(data, dtype=np.float64)
    if x.ndim == 1:
        x = x[:, None]
    n, d = x.shape
    sd = np.std(x, axis=0)
    iqr = (np.percentile(x, 75, axis=0) - np.percentile(x, 25, axis=0)) / 1.34
    sigma = float(np.mean(np.minimum(sd, iqr)))
    if sigma <= 0:
        sigma = 1.0
    return float(0.9 * sigma * n ** (-1.0 / (d + 4)))


def sdkde_1d(data) -> float:
    x = np.asarray(data, dtype=np.float64).reshape(-1)
    sd = float(x.std())
    iqr = float(np.percentile(x, 75) - np.percentile(x, 25))
    return 0.4 * min(sd, iqr / 1.34) * x.size ** (-1 / 9)
