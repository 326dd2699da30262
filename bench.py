#!/usr/bin/env python
"""Benchmark of the Flash-SD-KDE hot path on GB300.

Workload (one step): one-step empirical SD-KDE followed by KDE evaluation,
d = 16, FP32 inputs: n_train = n_query = 2^20 by default (--n) drawn from the
8-component Gaussian mixture (weights Dirichlet(1), means N(0, 4I),
covariances A A^T/16 + 0.1 I), the queries fresh draws; bandwidth by
Silverman's rule.  A step is
  empirical score (pdf_sum, weighted_sum; n^2 pair evaluations)
  + debias shift + KDE of the debiased set at the queries (n*m pairs),
through the public API (emp_sd_kde_fit_transform + kde_eval, default
backends).  Metric: exact 16-D pair evaluations per second.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl fsk|reference] [--n N]

value      device-resident inputs, per-step CUDA events on the launching
           stream, L2 flushed (256 MiB write) before every timed step.
e2e        the same calls from pinned host buffers, the H2D copy of the
           inputs and the D2H copy of the densities inside the timing.
roofline   the dominant kernel's required exps/s (library timer: CUDA events
           on its own stream) against the exp-bound peak built from the SFU
           ex2 and FP32 FMA rates measured on this GPU.
triton_reference  the reference's own Triton kernels, unmodified, imported
           from baseline/_ref in a child process, timed on the same GPU and
           workload (paper protocol empirical_sd_kde_triton_nd +
           gaussian_kde_triton_nd, and the default public API), with their
           errors against FP64.
cpu_baseline  the reference CPU path (numpy restatement) on a bounded
           sample with all host cores, in a subprocess.
surrogate  the learned-surrogate workload (exact SD-KDE fit on 262144 points,
           4 MLPs trained on 4M pairs, 1M held-out queries).
Multi-GPU (torchrun): every rank runs an independent replica (own query
set, shared training set); value = all ranks' pairs / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "flash-sd-kde_gb300"
REF_DIR = ROOT / "baseline" / "_ref"
sys.path[:0] = [str(PKG), str(ROOT)]

N_DEFAULT = 1 << 20
EPS = 1e-12
# FP32-pipe lane operations per pair in the tensor-core KDE epilogue besides
# the exp (scale-add, query offset, accumulate) and per polynomial exp2; used
# for the exp-bound peak P = R_sfu / (1 - f*), f* = (R_fma - c R_sfu) / (R_fma + k R_sfu).
C_OPS_PER_PAIR = 3.0
K_OPS_PER_POLY_EXP = 10.0
KERNEL_NAMES = {1: "kde16_tc_kernel", 2: "kde16_simt_kernel", 3: "score16_simt_kernel",
                4: "score16_sym_simt_kernel", 5: "kde1d_kernel", 6: "kde1d_score_kernel",
                7: "score16_tc_kernel", 9: "mlp_infer_kernel", 10: "kde16_logspace_kernel",
                11: "kde_nd_kernel", 12: "score_nd_kernel"}
# Tensor-core flops per pair evaluation.  "issued": what the tcgen05 kernels
# execute (three-part fp16 operands: seven K=16 MMAs for the exponent; the
# score kernel's weighted sums as fp16 hi/lo weights times [X_hi | X_lo] and
# X_hi).  "algorithmic": the contraction itself, 2*16 flops per pair for the
# exponent's dot product, plus 2*16 for the weighted sum of the score.
MMA_FLOPS_PER_PAIR = {"kde16_tc_kernel": {"issued": 7 * 2 * 16, "algorithmic": 2 * 16},
                      "score16_tc_kernel": {"issued": 7 * 2 * 16 + 2 * 128 * 16 * (4 * 32 + 4 * 16) / (128 * 64),
                                            "algorithmic": 2 * 2 * 16}}


# ---------------------------------------------------------------------------
# FP64 spot checks of the measured outputs (self-contained: the oracle package
# of the test suite is used only by the CPU-baseline leg)
# ---------------------------------------------------------------------------
def fp64_log_density(samples, queries, h: float, *, q_chunk: int = 256, s_chunk: int = 1 << 16):
    """FP64 log-density of the Gaussian KDE, log sum_j exp(-|q - x_j|^2 / 2h^2)
    - log n - d log h - (d/2) log 2 pi, by a chunked logsumexp; distances by
    the FP64 expansion about the sample mean (its rounding, ~1e-16 of the
    squared norms, is far below the FP32 errors being measured); query chunks
    on a thread pool."""
    import concurrent.futures as cf

    import numpy as np

    x = np.asarray(samples, dtype=np.float64)
    q = np.asarray(queries, dtype=np.float64)
    n, d = x.shape
    c = x.mean(axis=0)
    x, q = x - c, q - c
    xn, qn = (x * x).sum(axis=1), (q * q).sum(axis=1)
    log_const = -math.log(n) - d * math.log(h) - 0.5 * d * math.log(2.0 * math.pi)
    inv2h2 = 1.0 / (2.0 * h * h)

    def work(qs: int):
        run = np.full(min(q_chunk, q.shape[0] - qs), -np.inf)
        for ss in range(0, n, s_chunk):
            e = q[qs:qs + q_chunk] @ x[ss:ss + s_chunk].T
            e *= -2.0
            e += qn[qs:qs + q_chunk, None]
            e += xn[None, ss:ss + s_chunk]
            np.maximum(e, 0.0, out=e)
            e *= -inv2h2
            mx = e.max(axis=1)
            e -= mx[:, None]
            np.exp(e, out=e)
            run = np.logaddexp(run, mx + np.log(e.sum(axis=1)))
        return run

    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        parts = list(ex.map(work, range(0, q.shape[0], q_chunk)))
    return np.concatenate(parts) + log_const


def fp64_score_rows(data, rows, h: float):
    """FP64 (pdf_sum, weighted_sum) of the empirical score for the given data
    rows against all points (self pair included), by direct differences."""
    import numpy as np

    x = np.asarray(data, dtype=np.float64)
    pdf = np.zeros(len(rows))
    w = np.zeros((len(rows), x.shape[1]))
    for i, r in enumerate(rows):
        phi = np.exp(-((x - x[r]) ** 2).sum(axis=1) / (2.0 * h * h))
        pdf[i] = phi.sum()
        w[i] = phi @ x
    return pdf, w


def log_error_stats(logp, ref_logp) -> dict:
    """Log-density error statistics over the queries finite in both: finite
    fractions, max / mean / p95 absolute and max relative log error, RMSE,
    bias (the measures of the reference's error suite)."""
    import numpy as np

    a, b = np.asarray(logp, dtype=np.float64), np.asarray(ref_logp, dtype=np.float64)
    ok = np.isfinite(a) & np.isfinite(b)
    out = {"finite_fraction": float(np.isfinite(a).mean()), "finite_fraction_ref": float(np.isfinite(b).mean())}
    if not ok.any():
        return out
    diff = a[ok] - b[ok]
    ad = np.abs(diff)
    return {**out, "max_abs_log_err": float(ad.max()), "mean_abs_log_err": float(ad.mean()),
            "rmse_log_err": float(np.sqrt((diff * diff).mean())), "p95_abs_log_err": float(np.quantile(ad, 0.95)),
            "bias_log_err": float(diff.mean()),
            "max_rel_log_err": float((ad / np.maximum(np.abs(b[ok]), 1e-300)).max())}


def log_density_errors(dens, ref_logp) -> dict:
    """Errors of densities against FP64 log-densities: the density's relative
    error, the absolute log-density error and the relative log-density error
    |log p - log p64| / |log p64| (the error measure of the 1e-5 target)."""
    import numpy as np

    dens = np.asarray(dens, dtype=np.float64)
    ref = np.asarray(ref_logp, dtype=np.float64)
    rel = np.abs(dens - np.exp(ref)) / np.exp(ref)
    logp = np.log(np.maximum(dens, np.finfo(np.float64).tiny))
    abs_log = np.abs(logp - ref)
    return {"kde_max_rel_vs_fp64": float(rel.max()), "kde_median_rel_vs_fp64": float(np.median(rel)),
            "kde_max_abs_log_err_vs_fp64": float(abs_log.max()),
            "kde_max_rel_log_err_vs_fp64": float((abs_log / np.abs(ref)).max()),
            "kde_queries_checked": int(dens.size)}


def parse():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["fsk", "reference"], default="fsk")
    ap.add_argument("--n", type=int, default=N_DEFAULT, help="n_train = n_query of the SD-KDE workload")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-triton", action="store_true", help="leave the reference-Triton leg out")
    ap.add_argument("--triton-leg", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--triton-steps", type=int, default=3)
    ap.add_argument("--triton-small", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--triton-ieee", action="store_true",
                    help="also time the reference's fp32_ieee path (slow: CUDA-core FP32)")
    ap.add_argument("--h", type=str, default=None, help=argparse.SUPPRESS)
    ap.add_argument("--surrogate", action="store_true",
                    help="run only the learned-surrogate workload (C4) and print its JSON line")
    ap.add_argument("--no-surrogate", action="store_true", help="leave the surrogate object out of the bench line")
    ap.add_argument("--sur-train", type=int, default=262144, help="surrogate workload: exact SD-KDE fit points")
    ap.add_argument("--sur-pairs", type=int, default=4_000_000, help="surrogate workload: training pairs")
    ap.add_argument("--sur-eval", type=int, default=1_000_000, help="surrogate workload: held-out queries")
    ap.add_argument("--op", choices=["kde16", "kde16_offload", "kde16_logexact", "score16", "score16_sym", "kde1d",
                                     "precision", "sdkde_latency"],
                    default=None,
                    help="time one operation alone on n GMM8 points (profiling case; no contract line)")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def metric_name() -> str:
    return "16D pair-evals/s exact (SD-KDE: empirical score + debias + KDE)"


def workload_config(n: int) -> dict:
    return {
        "workload": f"sdkde_gmm8_16d_n{n}_m{n}",
        "n_train": n,
        "n_query": n,
        "d": 16,
        "bandwidth": "silverman",
        "pairs_per_step": n * n + n * n,
        "api": "flash_sd_kde.emp_sd_kde_fit_transform + flash_sd_kde.kde_eval (default backends)",
        "l2": "flushed before each timed step (256 MiB write)",
        "precision_mode": "fast_tf32 (three-part fp16 tensor-core exponents + exact FP32 near-pair recompute)",
    }


def gmm_inputs(n: int, query_seed: int = 2):
    from fsk import workloads

    gmm = workloads.GMM16(seed=0)
    return gmm.sample(n, seed=1), gmm.sample(n, seed=query_seed)


# ---------------------------------------------------------------------------
# CPU baseline / reference arm
# ---------------------------------------------------------------------------
REFERENCE_ARM_SECONDS = 90.0   # CPU work of the reference arm's timed steps, all together


def cpu_baseline(n: int, target_seconds: float, steps: int = 1) -> dict:
    cmd = [sys.executable, "-m", "oracle.cpu_baseline", "--n", str(n),
           "--target-seconds", str(target_seconds), "--steps", str(steps)]
    env = dict(os.environ, OMP_NUM_THREADS="1", OPENBLAS_NUM_THREADS="1", MKL_NUM_THREADS="1")
    res = subprocess.run(cmd, cwd=str(ROOT), capture_output=True, text=True, env=env, timeout=900)
    if res.returncode != 0:
        raise RuntimeError(f"cpu baseline failed: {res.stderr[-2000:]}")
    return json.loads(res.stdout.strip().splitlines()[-1])


def run_reference_arm(args) -> None:
    world, rank, _ = dist_env()
    if rank != 0:
        return
    warm = cpu_baseline(args.n, 2.0, steps=max(1, min(args.warmup, 1)))
    # the whole timed run is held to ~90 s of CPU work whatever --steps is:
    # each step is a sample of row blocks sized to 90 s / steps
    per_step = max(0.05, min(6.0, REFERENCE_ARM_SECONDS / max(1, args.steps)))
    t0 = time.perf_counter()
    res = cpu_baseline(args.n, per_step, steps=args.steps)
    wall = time.perf_counter() - t0
    pairs_step = res["value"] * res["seconds"] / args.steps
    line = {
        "impl": "reference",
        "metric": metric_name(),
        "value": res["value"],
        "unit": "pair-evals/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * res["seconds"] / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded 8-component Gaussian mixture)",
        "config": workload_config(args.n),
        "cpu_baseline": {"value": res["value"], "unit": "pair-evals/s", "cores": res["cores"],
                         "kind": res["kind"], "sample": res["sample"]},
        "e2e": {"value": res["value"], "unit": "pair-evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "notes": f"each step is a bounded sample of {pairs_step:.3e} pair evaluations of the workload; "
                 f"warm-up {warm['seconds']:.1f}s, timed wall {wall:.1f}s",
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# reference Triton leg (child process)
# ---------------------------------------------------------------------------
def triton_leg(n: int, h: float, steps: int, ieee: bool) -> dict:
    """Runs this script with --triton-leg in a child process (the reference's
    packages share module names with this package, so they get a process of
    their own) and returns its JSON object."""
    if not (REF_DIR / "kernels" / "flash_sd_kde").is_dir():
        return {"unavailable": f"reference package not present under {REF_DIR.relative_to(ROOT)}"}
    cmd = [sys.executable, str(ROOT / "bench.py"), "--triton-leg", "--n", str(n), "--h", repr(h),
           "--triton-steps", str(steps)] + (["--triton-ieee"] if ieee else [])
    env = dict(os.environ)
    # Triton's bundled ptxas predates sm_103a; the toolkit's ptxas (CUDA 13)
    # compiles the same PTX for this GPU.  TRITON_PTXAS_PATH is Triton's own
    # switch for that; the reference's code is unchanged.
    for cand in ("/usr/local/cuda/bin/ptxas",):
        if os.path.exists(cand) and "TRITON_PTXAS_PATH" not in env:
            env["TRITON_PTXAS_PATH"] = cand
    try:
        res = subprocess.run(cmd, cwd=str(ROOT), capture_output=True, text=True, timeout=1500, env=env)
        out, err, rc = res.stdout, res.stderr, res.returncode
    except subprocess.TimeoutExpired as exc:
        out = exc.stdout.decode() if isinstance(exc.stdout, bytes) else (exc.stdout or "")
        err, rc = "timed out after 1500 s", None
    # the child prints its cumulative result after every leg
    lines = [ln for ln in out.strip().splitlines() if ln.startswith("{")]
    if not lines:
        return {"unavailable": f"reference Triton leg failed (rc {rc}): {err.strip()[-600:]}"}
    res = json.loads(lines[-1])
    if rc != 0:
        res["incomplete"] = f"rc {rc}: {err.strip()[-300:]}"
    return res


def triton_small_leg(hs, steps: int) -> dict:
    """The reference's public API at the latency op's sizes, in a child
    process (as triton_leg); hs = the bandwidths of the plain-KDE case and of
    each SD-KDE size."""
    if not (REF_DIR / "kernels" / "flash_sd_kde").is_dir():
        return {"unavailable": f"reference package not present under {REF_DIR.relative_to(ROOT)}"}
    cmd = [sys.executable, str(ROOT / "bench.py"), "--triton-leg", "--triton-small",
           "--h", ",".join(repr(h) for h in hs), "--steps", str(steps)]
    env = dict(os.environ)
    if os.path.exists("/usr/local/cuda/bin/ptxas") and "TRITON_PTXAS_PATH" not in env:
        env["TRITON_PTXAS_PATH"] = "/usr/local/cuda/bin/ptxas"
    try:
        res = subprocess.run(cmd, cwd=str(ROOT), capture_output=True, text=True, timeout=900, env=env)
        out, err, rc = res.stdout, res.stderr, res.returncode
    except subprocess.TimeoutExpired as exc:
        out = exc.stdout.decode() if isinstance(exc.stdout, bytes) else (exc.stdout or "")
        err, rc = "timed out after 900 s", None
    lines = [ln for ln in out.strip().splitlines() if ln.startswith("{")]
    if not lines:
        return {"unavailable": f"reference Triton small-size leg failed (rc {rc}): {err.strip()[-600:]}"}
    res = json.loads(lines[-1])
    if rc != 0:
        res["incomplete"] = f"rc {rc}: {err.strip()[-300:]}"
    return res


def run_triton_leg(args) -> None:
    """Child process: the reference's own kernels, unmodified, from
    baseline/_ref (its package directories as published), timed with CUDA
    events on the same GMM8 workload.  Paper protocol
    (experiments/runtime/benchmark_triton_kde.py:344-388 of the reference):
    empirical_sd_kde_triton_nd + gaussian_kde_triton_nd; default public API:
    emp_sd_kde_fit_transform + kde_eval (flash score backend, splitk_stream
    KDE, fast_tf32, autotune)."""
    import importlib.util

    sys.path[:] = [str(REF_DIR)] + [p for p in sys.path if p not in (str(PKG), str(ROOT))] + [str(ROOT)]
    import numpy as np
    import torch

    spec = importlib.util.spec_from_file_location("fsk_workloads", PKG / "fsk" / "workloads.py")
    wl = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(wl)
    import triton

    import flash_sd_kde as ref_api
    import kernels.flash_sd_kde as ref_k
    for mod in (ref_api, ref_k):
        if not str(Path(mod.__file__).resolve()).startswith(str(REF_DIR.resolve())):
            raise RuntimeError(f"{mod.__name__} resolved outside {REF_DIR}")
    dev = torch.device("cuda", 0)
    n, h = args.n, float(args.h)
    gmm = wl.GMM16(seed=0)
    x_np, q_np = gmm.sample(n, seed=1), gmm.sample(n, seed=2)
    x = torch.from_numpy(x_np).to(dev)
    q = torch.from_numpy(q_np).to(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def timed(fn, steps, warm):
        for _ in range(warm):
            out = fn()
        torch.cuda.synchronize(dev)
        ms = []
        for _ in range(steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            out = fn()
            e1.record()
            torch.cuda.synchronize(dev)
            ms.append(e0.elapsed_time(e1))
        return ms, out

    def paper_step():
        deb, _ = ref_k.empirical_sd_kde_triton_nd(x, h, device=dev, return_tensor=True, synchronize=False)
        return deb, ref_k.gaussian_kde_triton_nd(deb, q, h, device=dev, synchronize=False)

    def api_step():
        deb = ref_api.emp_sd_kde_fit_transform(x, h, device=dev)
        return deb, ref_api.kde_eval(deb, q, h, device=dev)

    pairs = 2.0 * n * n
    out = {"impl": "reference-triton", "triton": triton.__version__, "torch": torch.__version__,
           "ptxas": os.environ.get("TRITON_PTXAS_PATH", "triton bundled"),
           "source": "baseline/_ref (the reference's flash_sd_kde/, kernels/, globals.py, unmodified)",
           "workload": f"sdkde_gmm8_16d_n{n}_m{n}", "pairs_per_step": pairs, "bandwidth": h}
    sub_q = 64
    ref_logp = fp64_log_density(x_np, q_np[:sub_q], h)
    # FP64 debias of rows 0..63 (self pair included)
    rows = np.arange(64)
    pdf64, w64 = fp64_score_rows(x_np, rows, h)
    deb64 = x_np[:64].astype(np.float64) + 0.5 * (w64 / (pdf64[:, None] + EPS) - x_np[:64])

    def errors(deb, kde_of_x):
        dens = kde_of_x.detach().cpu().numpy().astype(np.float64)
        return {**log_density_errors(dens, ref_logp),
                "debias_max_abs_vs_fp64": float(np.abs(deb[:64].detach().cpu().numpy() - deb64).max()),
                "debias_rows_checked": 64}

    legs = {}
    out["legs"] = legs

    def report():
        best = max(legs, key=lambda k: legs[k]["pair_evals_per_s"])
        out["best_leg"] = best
        out["pair_evals_per_s"] = legs[best]["pair_evals_per_s"]
        print(json.dumps(out), flush=True)

    ms, (deb, _) = timed(paper_step, args.triton_steps, 1)
    kde_x = ref_k.gaussian_kde_triton_nd(x, q[:sub_q], h, device=dev)
    legs["paper_protocol_fast_tf32"] = {
        "calls": "empirical_sd_kde_triton_nd + gaussian_kde_triton_nd",
        "ms_per_step": statistics.median(ms), "step_ms": ms,
        "pair_evals_per_s": pairs / (statistics.median(ms) * 1e-3), **errors(deb, kde_x)}
    report()
    ms, (deb, _) = timed(api_step, args.triton_steps, 2)
    kde_x = ref_api.kde_eval(x, q[:sub_q], h, device=dev)
    legs["default_api_fast_tf32"] = {
        "calls": "emp_sd_kde_fit_transform + kde_eval (flash_sd_kde score backend, splitk_stream KDE, autotune)",
        "ms_per_step": statistics.median(ms), "step_ms": ms,
        "pair_evals_per_s": pairs / (statistics.median(ms) * 1e-3), **errors(deb, kde_x)}
    report()
    if args.triton_ieee:
        def ieee_step():
            deb = ref_api.emp_sd_kde_fit_transform(x, h, device=dev, precision_mode="fp32_ieee",
                                                   emp_score_backend="symmetric_atomic")
            return deb, ref_api.kde_eval(deb, q, h, device=dev, precision_mode="fp32_ieee")

        ms, (deb, _) = timed(ieee_step, 1, 1)
        kde_x = ref_api.kde_eval(x, q[:sub_q], h, device=dev, precision_mode="fp32_ieee")
        legs["default_api_fp32_ieee"] = {
            "calls": "emp_sd_kde_fit_transform(symmetric_atomic, fp32_ieee) + kde_eval(fp32_ieee)",
            "ms_per_step": statistics.median(ms), "step_ms": ms,
            "pair_evals_per_s": pairs / (statistics.median(ms) * 1e-3), **errors(deb, kde_x)}
        report()


LATENCY_SIZES = ((4096, 1024), (16384, 4096), (65536, 65536))


def latency_inputs(n: int, m: int, plain: bool):
    """Inputs of the small-size latency cases: the plain-KDE configuration
    (N(0, I), 4096 / 1024, seed 0) or the GMM8 SD-KDE workload at n / m."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("fsk_workloads", PKG / "fsk" / "workloads.py")
    wl = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(wl)
    if plain:
        return wl.plain_kde_16d(n, m)
    g = wl.GMM16(seed=0)
    return g.sample(n, seed=1), g.sample(m, seed=2)


def time_calls(fn, warm: int, reps: int, dev) -> tuple[float, float]:
    """(device us, host us) per call: CUDA events and wall clock around reps
    back-to-back calls after warm-up calls."""
    import torch

    for _ in range(warm):
        fn()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize(dev)
    return 1e3 * e0.elapsed_time(e1) / reps, 1e6 * (time.perf_counter() - t0) / reps


def run_triton_small(args) -> None:
    """Child process: the reference's own public API, unmodified, from
    baseline/_ref, at the small sizes of the latency op: kde_eval on the
    plain-KDE configuration, and emp_sd_kde_fit_transform + kde_eval on the
    GMM8 workload; bandwidths passed in by the parent so both arms use the
    same h."""
    sys.path[:] = [str(REF_DIR)] + [p for p in sys.path if p not in (str(PKG), str(ROOT))] + [str(ROOT)]
    import torch

    import flash_sd_kde as ref_api
    if not str(Path(ref_api.__file__).resolve()).startswith(str(REF_DIR.resolve())):
        raise RuntimeError(f"flash_sd_kde resolved outside {REF_DIR}")
    dev = torch.device("cuda", 0)
    hs = [float(v) for v in args.h.split(",")]
    rows = []
    x_np, q_np = latency_inputs(4096, 1024, plain=True)
    x, q = torch.from_numpy(x_np).to(dev), torch.from_numpy(q_np).to(dev)
    us, host = time_calls(lambda: ref_api.kde_eval(x, q, hs[0], device=dev), 5, max(10, args.steps), dev)
    rows.append({"case": "plain_kde", "n_train": 4096, "n_query": 1024, "kde_eval_us": us, "kde_eval_host_us": host})
    for (n, m), h in zip(LATENCY_SIZES, hs[1:]):
        x_np, q_np = latency_inputs(n, m, plain=False)
        x, q = torch.from_numpy(x_np).to(dev), torch.from_numpy(q_np).to(dev)
        fn = lambda: ref_api.kde_eval(ref_api.emp_sd_kde_fit_transform(x, h, device=dev), q, h, device=dev)
        us, host = time_calls(fn, 5, max(10, args.steps), dev)
        rows.append({"case": "sdkde", "n_train": n, "n_query": m, "two_calls_us": us, "two_calls_host_us": host})
        print(json.dumps({"impl": "reference-triton", "rows": rows}), flush=True)
    print(json.dumps({"impl": "reference-triton", "rows": rows}), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 100 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"fsk_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self) -> dict:
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        self.path.unlink(missing_ok=True)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def exp_peak(rates) -> dict:
    r_sfu, r_fma = float(rates[0]), float(rates[1])
    c, k = C_OPS_PER_PAIR, K_OPS_PER_POLY_EXP
    f = (r_fma - c * r_sfu) / (r_fma + k * r_sfu)
    peak = r_sfu / (1.0 - f) if f > 0 else min(r_sfu, r_fma / c)
    return {"peak": peak, "r_sfu": r_sfu, "r_fma": r_fma, "r_ffma2_lanes": float(rates[2]), "offload_fraction": max(f, 0.0)}


def tensor_roofline(kernel, pairs_per_s) -> dict | None:
    """Tensor-pipe view of the dominant kernel against the measured dense
    bf16 peak (the fp16 tensor rate is the same): the algorithmic contraction
    flops and the flops the kernel issues for its split-precision operands."""
    if not kernel or kernel not in MMA_FLOPS_PER_PAIR or not pairs_per_s:
        return None
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = peaks.get("bf16_tflops")
    src = "MEASURED_PEAKS.json bf16_tflops (burst, cuBLAS), of measured"
    if not peak:
        peak, src = 1900.0, "fallback 1.9 PFLOP/s, of fallback"
    fl = MMA_FLOPS_PER_PAIR[kernel]
    alg = pairs_per_s * fl["algorithmic"] / 1e12
    iss = pairs_per_s * fl["issued"] / 1e12
    return {"bound": "tensor", "kernel": kernel, "achieved": alg, "peak": peak, "unit": "TFLOP/s",
            "frac": alg / peak, "flops_per_pair": fl["algorithmic"],
            "issued": {"achieved": iss, "frac": iss / peak, "flops_per_pair": fl["issued"]},
            "peak_source": src}


def run_gpu_arm(args) -> None:
    import numpy as np
    import torch
    import torch.distributed as dist

    world, rank, local = dist_env()
    if world > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", rank=rank, world_size=world)
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)

    import __graft_entry__ as ge

    ge.build()
    from flash_sd_kde import emp_sd_kde_fit_transform, kde_eval
    from fsk import _lib, ops

    lib = _lib.load()
    n = args.n
    x_np, q_np = gmm_inputs(n, query_seed=2 + rank)
    x = torch.from_numpy(x_np).to(dev)
    q = torch.from_numpy(q_np).to(dev)
    h = float(ops.silverman(x).item())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step(xd, qd):
        deb = emp_sd_kde_fit_transform(xd, h, device=dev)
        return deb, kde_eval(deb, qd, h, device=dev)

    rates = np.zeros(3)
    _lib.check(lib.fsk_diag_pipe_rates(rates.ctypes.data, stream.cuda_stream), "pipe rates")
    peak = exp_peak(rates)

    for _ in range(args.warmup):
        step(x, q)
    ops.device_status(dev)

    # ---- device-resident timing -------------------------------------------------
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize(dev)
    launches0 = lib.fsk_launch_count()
    lib.fsk_timer_enable(1)
    sampler = ClockSampler(dev.index or 0)
    with sampler:
        for s_ev, e_ev in evs:
            flush.zero_()
            s_ev.record(stream)
            deb, dens = step(x, q)
            e_ev.record(stream)
        torch.cuda.synchronize(dev)
    lib.fsk_timer_enable(0)
    launches = lib.fsk_launch_count() - launches0
    step_ms = [s.elapsed_time(e) for s, e in evs]
    total_ms = float(sum(step_ms))
    ids = np.zeros(16, np.int32)
    nl = np.zeros(16, np.int64)
    kms = np.zeros(16)
    kwork = np.zeros(16)
    rows = lib.fsk_timer_collect(ids.ctypes.data, nl.ctypes.data, kms.ctypes.data, kwork.ctypes.data, 16)
    if world > 1:
        t = torch.tensor([total_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
        dist.barrier()
    ops.device_status(dev)
    pairs_step = 2.0 * float(n) * n
    value = world * pairs_step * args.steps / (total_ms * 1e-3)

    kernels = {}
    for r in range(max(rows, 0)):
        name = KERNEL_NAMES.get(int(ids[r]), str(int(ids[r])))
        kernels[name] = {"launches": int(nl[r]), "ms": float(kms[r]), "exps": float(kwork[r]),
                         "exps_per_s": float(kwork[r]) / (kms[r] * 1e-3) if kms[r] > 0 else None,
                         "share_of_step_time": float(kms[r]) / total_ms if total_ms > 0 else None}
    dom = max(kernels, key=lambda k: kernels[k]["ms"]) if kernels else None
    achieved = kernels[dom]["exps_per_s"] if dom else None
    traffic = None
    tfile = ROOT / "profiles" / "traffic.json"
    if dom and tfile.exists():
        try:
            # per-launch DRAM bytes of the dominant kernel, from an ncu capture at this n
            tr = json.loads(tfile.read_text()).get(dom, {}).get(str(n), {})
            traffic = tr.get("bytes_per_launch")
        except ValueError:
            traffic = None

    # ---- end-to-end through the public API from host buffers ----------------------
    x_pin = torch.from_numpy(x_np).pin_memory()
    q_pin = torch.from_numpy(q_np).pin_memory()
    out_pin = torch.empty(n, dtype=torch.float32).pin_memory()
    e2e_evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]

    def e2e_step():
        xd = x_pin.to(dev, non_blocking=True)
        qd = q_pin.to(dev, non_blocking=True)
        _, dd = step(xd, qd)
        out_pin.copy_(dd, non_blocking=True)

    for _ in range(max(1, args.warmup)):
        e2e_step()
    torch.cuda.synchronize(dev)
    if world > 1:
        dist.barrier()
    for s_ev, e_ev in e2e_evs:
        flush.zero_()
        s_ev.record(stream)
        e2e_step()
        e_ev.record(stream)
    torch.cuda.synchronize(dev)
    e2e_ms = float(sum(s.elapsed_time(e) for s, e in e2e_evs))
    if world > 1:
        t = torch.tensor([e2e_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
    e2e_value = world * pairs_step * args.steps / (e2e_ms * 1e-3)

    # ---- accuracy spot check against FP64 ------------------------------------------
    sub = slice(0, 64)
    deb_np = deb.cpu().numpy()
    dens_np = dens.cpu().numpy().astype(np.float64)
    ref_logp = fp64_log_density(deb_np, q_np[sub], h)
    kde_err = log_density_errors(dens_np[sub], ref_logp)
    pdf64, w64 = fp64_score_rows(x_np, np.arange(64), h)
    deb64 = x_np[:64].astype(np.float64) + 0.5 * (w64 / (pdf64[:, None] + EPS) - x_np[:64])
    deb_abs = float(np.abs(deb_np[:64] - deb64).max())

    triton = None
    if rank == 0 and not args.no_triton:
        torch.cuda.synchronize(dev)
        triton = triton_leg(n, h, args.triton_steps, args.triton_ieee)
        if "pair_evals_per_s" in triton:
            triton["value_vs_triton"] = value / triton["pair_evals_per_s"]
            triton["e2e_vs_triton"] = e2e_value / triton["pair_evals_per_s"]

    surrogate = None
    if rank == 0 and not args.no_surrogate:
        try:
            surrogate = surrogate_workload(args, dev)
        except Exception as exc:  # reported, not fatal
            surrogate = {"error": str(exc)[-300:]}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            cpu = cpu_baseline(n, 12.0)
        except Exception as exc:  # reported, not fatal
            cpu = {"error": str(exc)[-300:]}

    if rank == 0:
        line = {
            "metric": metric_name(),
            "value": value,
            "unit": "pair-evals/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": total_ms / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32",
            "data": "synthetic (seeded 8-component Gaussian mixture)",
            "config": workload_config(n),
            "e2e": {"value": e2e_value, "unit": "pair-evals/s",
                    "h2d_bytes_per_step": int(x_np.nbytes + q_np.nbytes), "d2h_bytes_per_step": int(n * 4),
                    "ms_per_step": e2e_ms / args.steps,
                    "api": "flash_sd_kde.emp_sd_kde_fit_transform + flash_sd_kde.kde_eval"},
            "gpu_launches": int(launches),
            "roofline": {"bound": "sfu", "kernel": dom, "achieved": achieved, "peak": peak["peak"],
                         "unit": "required exps/s (one exp per pair; n(n+1)/2 for the symmetric score)",
                         "frac": (achieved / peak["peak"]) if achieved else None,
                         "traffic": traffic,
                         "peak_source": "measured on this GPU: ex2.approx %.3e/s, fma.f32 %.3e/s "
                                        "(fsk_diag_pipe_rates); P = R_sfu/(1-f*), c=%g, k=%g"
                                        % (peak["r_sfu"], peak["r_fma"], C_OPS_PER_PAIR, K_OPS_PER_POLY_EXP),
                         "sfu_only_peak": peak["r_sfu"]},
            "roofline_tensor": tensor_roofline(dom, achieved),
            "kernels": kernels,
            "triton_reference": triton,
            "cpu_baseline": cpu,
            "surrogate": surrogate,
            "clocks": sampler.summary(),
            "accuracy": {**kde_err, "debias_max_abs_vs_fp64": deb_abs, "debias_rows_checked": 64},
            "step_ms": step_ms,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def surrogate_workload(args, dev) -> dict:
    """Learned surrogate (C4): exact SD-KDE fit on n GMM8 points, ensemble of
    4 MLPs trained on (data + N(0, h^2 I), exact log p) pairs, evaluated on
    held-out queries, half in-support (same recipe, new seed) and half
    N(0, 9 I).  Reports the gated path (surrogate + exact fallback), the
    surrogate alone and the exact KDE in queries/s, with the median relative
    density error over the served queries and the fallback rate."""
    import torch

    from flash_sd_kde import emp_sd_kde_fit_transform
    from flash_sd_kde.surrogate import SurrogateKDE
    from fsk import ops, workloads

    gmm = workloads.GMM16(seed=0)
    x = torch.from_numpy(gmm.sample(args.sur_train, seed=1)).to(dev)
    h = float(ops.silverman(x).item())
    deb = emp_sd_kde_fit_transform(x, h, device=dev)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    sur = SurrogateKDE(members=4).fit(deb, h, n_pairs=args.sur_pairs)
    torch.cuda.synchronize(dev)
    fit_s = time.perf_counter() - t0
    g = torch.Generator(device=dev).manual_seed(12345)
    half = args.sur_eval // 2
    idx = torch.randint(deb.shape[0], (half,), generator=g, device=dev)
    q_in = deb[idx] + torch.randn((half, 16), generator=g, device=dev) * h
    q_out = torch.randn((args.sur_eval - half, 16), generator=g, device=dev) * 3.0
    q = torch.cat([q_in, q_out]).contiguous()

    def timed(fn, reps=3):
        fn()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            out = fn()
        e1.record()
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / reps, out

    ms_exact, exact = timed(lambda: sur._exact_logp(q))
    ms_gated, (logp, served) = timed(lambda: sur.score_samples(q, return_served=True))
    ms_sur, _ = timed(lambda: sur.predict(q))
    ops.device_status(dev)
    # the exact path recomputes queries whose FP32 sum underflows (log 0 in a plain FP32 sum)
    norm = 1.0 / ((2.0 * math.pi) ** 8 * h ** 16 * deb.shape[0])
    plain = ops.kde16_sum(q, deb, h, out_scale=norm, log_eps=0.0)
    recomputed = int((~torch.isfinite(plain)).sum())
    fin = torch.isfinite(exact)
    rel = (torch.exp((logp - exact).double()) - 1).abs()
    srv = served.bool() & fin
    nq = q.shape[0]
    # gate frontier: served fraction and served error as the ensemble-spread tolerance varies
    mean_s, spread_s, _ = sur.predict(q)
    in_r = sur._radius2(q) <= sur.r2_max_
    rel_s = (torch.exp((mean_s - exact).double()) - 1).abs()
    frontier = []
    for tol in (0.005, 0.01, 0.02, 0.03, 0.05, 0.1, 0.2, float("inf")):
        sel = (spread_s <= tol) & in_r & fin
        frontier.append({"spread_tol": tol, "served_fraction": float(sel.float().mean()),
                         "served_fraction_in_support": float(sel[:half].float().mean()),
                         "median_rel_density_err_served": float(rel_s[sel].median()) if sel.any() else None})
    return {
        "workload": f"surrogate_gmm8_16d_fit{args.sur_train}_pairs{args.sur_pairs}_eval{nq}",
        "members": 4, "mlp": "16-256-256-256-1 SiLU, bf16 weights/activations, FP32 accumulation",
        "fit_seconds": fit_s, "train_mse_normalised": sur.history[-1] if sur.history else None,
        "exact_queries_per_s": nq / (ms_exact * 1e-3),
        "gated_queries_per_s": nq / (ms_gated * 1e-3),
        "surrogate_only_queries_per_s": nq / (ms_sur * 1e-3),
        "speedup_gated_vs_exact": ms_exact / ms_gated,
        "speedup_surrogate_only_vs_exact": ms_exact / ms_sur,
        "served_fraction": float(srv.float().mean()),
        "served_fraction_in_support": float(srv[:half].float().mean()),
        "served_fraction_out_of_support": float(srv[half:].float().mean()),
        "median_rel_density_err_served": float(rel[srv].median()) if srv.any() else None,
        "p90_rel_density_err_served": float(torch.quantile(rel[srv].float(), 0.9)) if srv.any() else None,
        "median_rel_density_err_all_surrogate": float(
            (torch.exp((sur.predict(q)[0] - exact).double()) - 1).abs()[fin].median()),
        "median_abs_log_err_in_support_surrogate": float((sur.predict(q)[0] - exact)[:half].abs().median()),
        "exact_recomputed_underflow_queries": recomputed,
        "exact_nonfinite_queries": int((~fin).sum()),
        "spread_tol": sur.spread_tol, "r2_max": sur.r2_max_,
        "gate_frontier": frontier,
    }


def run_surrogate(args) -> None:
    import torch

    import __graft_entry__ as ge

    ge.build()
    dev = torch.device("cuda", 0)
    print(json.dumps({"surrogate": surrogate_workload(args, dev)}), flush=True)


def run_precision(args) -> None:
    """The precision-stress configuration: n_train = n_query (default 2^20)
    multivariate Student-t (nu = 5) points, per-axis scale 10^U(-1, 1), +100
    offset; h in {0.5, 1, 2} x Silverman of the training set; every distance
    mode of the 16-D KDE (three-part fp16 tensor-core products with the exact
    near-pair recompute; FP32 direct differences; the single-pass fp16 rung;
    the exact-log output) over all queries, with FP64 log-density errors on a
    fixed 4096-query subset (max / mean / p95 absolute log error, as the
    reference's error suite reports them) and each mode's time."""
    import numpy as np
    import torch

    import __graft_entry__ as ge

    ge.build()
    from fsk import ops, workloads

    dev = torch.device("cuda", 0)
    n = args.n
    x_np = workloads.student_t_16d(n, seed=4)
    q_np = workloads.student_t_16d(n, seed=5)
    x = torch.from_numpy(x_np).to(dev)
    q = torch.from_numpy(q_np).to(dev)
    h0 = float(ops.silverman(x).item())
    sub = np.random.default_rng(0).choice(n, min(n, 4096), replace=False)
    rows = []
    for f in (0.5, 1.0, 2.0):
        h = h0 * f
        norm = 1.0 / ((2 * math.pi) ** 8 * h ** 16 * n)
        ref = fp64_log_density(x_np, q_np[sub], h)
        for mode in ("tensor", "ieee", "fp16_single", "tensor_log_exact"):
            if mode == "tensor_log_exact":
                fn = lambda: ops.kde16_sum(q, x, h, out_scale=norm, log_exact=True)
            else:
                fn = lambda mode=mode: ops.kde16_sum(q, x, h, precision=mode, out_scale=norm, log_eps=0.0)
            fn()
            torch.cuda.synchronize(dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            lp = fn()
            e1.record()
            torch.cuda.synchronize(dev)
            ops.device_status(dev)
            got = lp.cpu().numpy().astype(np.float64)[sub]
            rows.append({"h_factor": f, "h": h, "mode": mode, "ms": e0.elapsed_time(e1),
                         **log_error_stats(got, ref)})
            print(json.dumps(rows[-1]), file=sys.stderr, flush=True)
    print(json.dumps({"op": "precision", "workload": f"student_t5_offset100_16d_n{n}_m{n}",
                      "queries_checked": int(sub.size), "silverman_h": h0, "rows": rows}), flush=True)


def run_sdkde_latency(args) -> None:
    """Per-call time of the whole SD-KDE step (score + debias + KDE) at small
    sizes, where launch overhead matters: the public two-call path
    (emp_sd_kde_fit_transform + kde_eval), the one-call fsk_sdkde16, and that
    call replayed from a captured CUDA graph.  Sizes: 4096 train / 1024
    queries (the plain-KDE configuration's shape) and 65536 / 65536."""
    import torch

    import __graft_entry__ as ge

    ge.build()
    from flash_sd_kde import emp_sd_kde_fit_transform, kde_eval
    from fsk import ops, workloads

    dev = torch.device("cuda", 0)
    rows = []
    hs = []
    # the plain-KDE configuration (4096 N(0, I) points, 1024 queries): the public kde_eval
    x_np, q_np = latency_inputs(4096, 1024, plain=True)
    x, q = torch.from_numpy(x_np).to(dev), torch.from_numpy(q_np).to(dev)
    h = float(ops.silverman(x).item())
    hs.append(h)
    us, host = time_calls(lambda: kde_eval(x, q, h, device=dev), 5, max(10, args.steps), dev)
    rows.append({"case": "plain_kde", "n_train": 4096, "n_query": 1024, "kde_eval_us": us, "kde_eval_host_us": host})
    print(json.dumps(rows[-1]), file=sys.stderr, flush=True)
    for n, m in LATENCY_SIZES:
        g = workloads.GMM16(seed=0)
        x = torch.from_numpy(g.sample(n, seed=1)).to(dev)
        q = torch.from_numpy(g.sample(m, seed=2)).to(dev)
        h = float(ops.silverman(x).item())
        hs.append(h)
        graph = ops.SDKDEGraph(x, q, h)
        ws = ops._workspace(ops.L.load().fsk_sdkde16_workspace_bytes(n, m, 0), dev)
        out = torch.empty(m, dtype=torch.float32, device=dev)
        fns = {"two_calls": lambda: kde_eval(emp_sd_kde_fit_transform(x, h, device=dev), q, h, device=dev),
               "one_call": lambda: ops.sdkde16(x, q, h, out=out, workspace=ws),
               "graph_replay": graph.replay}
        row = {"case": "sdkde", "n_train": n, "n_query": m}
        for name, fn in fns.items():
            for _ in range(max(3, args.warmup)):
                fn()
            torch.cuda.synchronize(dev)
            reps = max(10, args.steps)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0 = time.perf_counter()
            e0.record()
            for _ in range(reps):
                fn()
            e1.record()
            torch.cuda.synchronize(dev)
            row[name + "_us"] = 1e3 * e0.elapsed_time(e1) / reps
            row[name + "_host_us"] = 1e6 * (time.perf_counter() - t0) / reps
        ops.device_status(dev)
        rows.append(row)
        print(json.dumps(row), file=sys.stderr, flush=True)
    ref = None
    if not args.no_triton:
        ref = triton_small_leg(hs, args.steps)
    print(json.dumps({"op": "sdkde_latency", "rows": rows, "reference_triton": ref}), flush=True)


def run_op(args) -> None:
    """One operation alone (the profiling case for ncu captures): n GMM8
    points as data and as queries, Silverman bandwidth, W warm-up and K timed
    launches with CUDA events on the launching stream.  kde16_logexact: exact
    log-densities with half the queries moved 60 bandwidths away from the data
    (every term of those underflows FP32, so they take the shifted recompute).
    kde1d: 4 n points of the 1-D three-component mixture against n grid
    queries on [-5, 6] (the large 1-D configuration at n = 2^20)."""
    import numpy as np
    import torch

    import __graft_entry__ as ge

    if args.op == "precision":
        return run_precision(args)
    if args.op == "sdkde_latency":
        return run_sdkde_latency(args)
    ge.build()
    from fsk import ops, workloads

    dev = torch.device("cuda", 0)
    if args.op == "kde1d":
        rng = np.random.default_rng(1)
        comp = rng.choice(3, size=4 * args.n, p=[0.3, 0.5, 0.2])
        x1 = (np.array([-2.0, 0.0, 3.0])[comp] + np.array([0.5, 1.0, 0.3])[comp] *
              rng.standard_normal(4 * args.n)).astype(np.float32)
        xd = torch.from_numpy(x1).to(dev)
        qd = torch.linspace(-5.0, 6.0, args.n, device=dev)
        h1 = float(fp_sdkde_1d(x1))
        fn = lambda: ops.kde1d_sum(qd, xd, h1)
        pairs = float(args.n) * 4 * args.n
        return _time_op(args, dev, fn, pairs, h1)
    x = torch.from_numpy(workloads.GMM16(seed=0).sample(args.n, seed=1)).to(dev)
    h = float(ops.silverman(x).item())
    pairs = float(args.n) * args.n
    if args.op == "kde16":
        fn = lambda: ops.kde16_sum(x, x, h)
    elif args.op == "kde16_offload":
        fn = lambda: ops.kde16_sum(x, x, h, exp_offload=True)
    elif args.op == "kde16_logexact":
        q = x.clone()
        q[::2] += 60.0 * h / 4.0      # offset 15 h per feature: 60 h away in 16-D
        fn = lambda: ops.kde16_sum(q, x, h, log_exact=True)
    elif args.op == "score16_sym":
        fn = lambda: ops.empscore16(x, h, variant="symmetric")
        pairs = float(args.n) * (args.n + 1) / 2.0
    else:
        fn = lambda: ops.empscore16(x, h)
    _time_op(args, dev, fn, pairs, h)


def fp_sdkde_1d(x) -> float:
    """Silverman-type 1-D bandwidth 0.9 min(std, IQR/1.34) n^(-1/5) in FP64 (host)."""
    import numpy as np

    x = np.asarray(x, np.float64)
    iqr = np.percentile(x, 75) - np.percentile(x, 25)
    return 0.9 * min(x.std(), iqr / 1.34) * x.size ** (-0.2)


def _time_op(args, dev, fn, pairs, h) -> None:
    import torch

    from fsk import ops

    for _ in range(args.warmup):
        fn()
    torch.cuda.synchronize(dev)
    s_ev, e_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stream = torch.cuda.current_stream(dev)
    s_ev.record(stream)
    for _ in range(args.steps):
        fn()
    e_ev.record(stream)
    torch.cuda.synchronize(dev)
    ops.device_status(dev)
    ms = s_ev.elapsed_time(e_ev) / args.steps
    print(json.dumps({"op": args.op, "n": args.n, "h": h, "ms_per_call": ms,
                      "required_exps_per_s": pairs / (ms * 1e-3)}), flush=True)


def main():
    args = parse()
    if args.triton_leg:
        if args.triton_small:
            run_triton_small(args)
        else:
            run_triton_leg(args)
        return
    if args.op:
        run_op(args)
        return
    if args.surrogate:
        run_surrogate(args)
        return
    if args.impl == "reference":
        run_reference_arm(args)
    else:
        run_gpu_arm(args)


if __name__ == "__main__":
    main()
