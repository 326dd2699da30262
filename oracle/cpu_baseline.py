"""Timed CPU baseline: the reference's CPU path (the FP32 numpy steps of
flash_sd_kde/reference.py, as restated in oracle.reference_numpy) on a
bounded sample of the SD-KDE workload, using all host cores -- TEST /
MEASUREMENT INFRASTRUCTURE ONLY.

The reference forms the full rows x n distance and weight matrices; here the
same element-wise steps run over 128-row x 4096-column tiles (so the working
set of each thread stays in cache and nothing of size rows x n is formed),
with the data norms computed once per run.  Run as a subprocess
(``python -m oracle.cpu_baseline ...``) so the BLAS thread count can be
pinned to one per worker thread before numpy loads; work is split over a
thread pool by row blocks (numpy releases the GIL inside the matmul / exp /
reductions).  Prints one JSON object.
"""
from __future__ import annotations

import os

for _v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
    os.environ.setdefault(_v, "1")

import argparse  # noqa: E402
import concurrent.futures as cf  # noqa: E402
import json  # noqa: E402
import sys  # noqa: E402
import time  # noqa: E402
from pathlib import Path  # noqa: E402

import numpy as np  # noqa: E402

ROOT = Path(__file__).resolve().parent.parent
sys.path[:0] = [str(ROOT / "flash-sd-kde_gb300"), str(ROOT)]

from oracle import reference_numpy as R  # noqa: E402

ROW_BLOCK = 128     # rows (data rows or queries) per work item
COL_BLOCK = 4096    # data columns per tile: a 2 MB FP32 tile per thread stays in cache


def block_rows(n: int) -> int:
    return ROW_BLOCK


def _tile_phi(xb, xbn, xt, xtn, inv_h2):
    """phi of one (rows x columns) tile with the FP32 steps of reference.py:227-232
    and :276-280: squared distances by the norm expansion, clamped at 0,
    exp(-0.5 * dist * inv_h2); computed in place in one buffer."""
    dist = xbn + xtn - 2.0 * (xb @ xt.T)
    np.maximum(dist, 0.0, out=dist)
    np.multiply(dist, -0.5, out=dist)
    np.multiply(dist, inv_h2, out=dist)
    return np.exp(dist, out=dist)


def _score_block(x, xn, r0, r1, h):
    """Empirical-score sums (reference.py:276-283: pdf_sum = phi.sum(1),
    weighted = phi @ x) for data rows r0..r1 against all of x, over column
    tiles so the full row block x n matrix is never formed."""
    inv_h2 = 1.0 / (h * h)
    xb, xbn = x[r0:r1], xn[r0:r1, None]
    pdf = np.zeros(r1 - r0, dtype=np.float32)
    w = np.zeros((r1 - r0, x.shape[1]), dtype=np.float32)
    for c in range(0, x.shape[0], COL_BLOCK):
        xt = x[c:c + COL_BLOCK]
        phi = _tile_phi(xb, xbn, xt, xn[None, c:c + COL_BLOCK], inv_h2)
        pdf += phi.sum(axis=1)
        w += phi @ xt
    return pdf, w


def _kde_block(x, xn, q, h):
    """Unnormalised KDE row sums (reference.py:216-235) of queries q against
    all of x, over column tiles."""
    inv_h2 = 1.0 / (h * h)
    qn = (q * q).sum(axis=1, keepdims=True)
    out = np.zeros(q.shape[0], dtype=np.float32)
    for c in range(0, x.shape[0], COL_BLOCK):
        out += _tile_phi(q, qn, x[c:c + COL_BLOCK], xn[None, c:c + COL_BLOCK], inv_h2).sum(axis=1)
    return out


def run(x, q, h, rows: int, threads: int) -> tuple[float, float]:
    """Time the score of `rows` data rows plus the KDE of `rows` queries;
    returns (seconds, pair evaluations)."""
    n = x.shape[0]
    blk = block_rows(n)
    starts = list(range(0, rows, blk))
    t0 = time.perf_counter()
    xn = (x * x).sum(axis=1)
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        futs = [ex.submit(_score_block, x, xn, s, min(rows, s + blk), h) for s in starts]
        futs += [ex.submit(_kde_block, x, xn, q[s:min(rows, s + blk)], h) for s in starts]
        for f in futs:
            f.result()
    dt = time.perf_counter() - t0
    return dt, 2.0 * rows * n


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=65536)
    ap.add_argument("--target-seconds", type=float, default=12.0)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    from fsk import workloads

    x, q = workloads.gmm8_16d(args.n, args.n)
    h = R.silverman_bandwidth_nd(x)
    # calibrate on one block per thread, then size the sample to the target
    blk = block_rows(args.n)
    dt, pairs = run(x, q, h, blk * args.threads, args.threads)
    rate = pairs / dt
    rows = int(min(args.n, max(blk, args.target_seconds * rate / (2.0 * args.n))))
    rows = max(blk, rows // blk * blk)
    times = []
    for _ in range(args.steps):
        dt, pairs = run(x, q, h, rows, args.threads)
        times.append(dt)
    total_t = float(sum(times))
    print(json.dumps({
        "value": pairs * len(times) / total_t,
        "unit": "pair-evals/s",
        "cores": args.threads,
        "kind": "port",
        "seconds": total_t,
        "sample": f"{rows} data rows x {args.n} (empirical score) + {rows} queries x {args.n} (KDE) of the "
                  f"gmm8_16d n={args.n} workload per step, FP32 numpy restatement of flash_sd_kde/reference.py "
                  f"over {ROW_BLOCK} x {COL_BLOCK} tiles, {args.threads} threads",
    }))


if __name__ == "__main__":
    main()
