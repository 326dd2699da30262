"""Timed CPU baseline: the reference's CPU path (the FP32 numpy restatement
in oracle.reference_numpy) on a bounded sample of the SD-KDE workload, using
all host cores -- TEST / MEASUREMENT INFRASTRUCTURE ONLY.

Run as a subprocess (``python -m oracle.cpu_baseline ...``) so the BLAS
thread count can be pinned to one per worker thread before numpy loads; work
is split over a thread pool by row blocks (numpy releases the GIL inside the
matmul / exp / reductions).  Prints one JSON object.
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

BLOCK = 128          # rows per work item at n <= 65536; fewer above (memory per item ~ rows * n * 12 B)


def block_rows(n: int) -> int:
    return max(8, min(BLOCK, BLOCK * 65536 // max(1, n)))


def _score_block(x, rows, h):
    """Empirical-score sums for data rows `rows` against all of x
    (reference.py:276-283 restricted to a row block)."""
    inv_h2 = 1.0 / (h * h)
    xb = x[rows]
    dist = (xb * xb).sum(1, keepdims=True) + (x * x).sum(1, keepdims=True).T - 2.0 * (xb @ x.T)
    phi = np.exp(-0.5 * np.maximum(dist, 0.0) * inv_h2)
    return phi.sum(1), phi @ x


def _kde_block(x, q, h):
    return R.kde_eval_nd_numpy(q, x, h)


def run(x, q, h, rows: int, threads: int) -> tuple[float, float]:
    """Time the score of `rows` data rows plus the KDE of `rows` queries;
    returns (seconds, pair evaluations)."""
    n = x.shape[0]
    blk = block_rows(n)
    starts = list(range(0, rows, blk))
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        futs = [ex.submit(_score_block, x, slice(s, min(rows, s + blk)), h) for s in starts]
        futs += [ex.submit(_kde_block, x, q[s:min(rows, s + blk)], h) for s in starts]
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
                  f"gmm8_16d n={args.n} workload per step, FP32 numpy restatement of flash_sd_kde/reference.py, "
                  f"{args.threads} threads",
    }))


if __name__ == "__main__":
    main()
