"""Backend/precision validation and launch heuristics (drop-in for
flash_sd_kde/config.py of the reference, same names and error messages).

Tile shapes of the GB300 kernels are fixed by the hardware mapping (one query
row per TMEM lane, 128-wide data tiles) and their split counts are chosen by
the C planner (plan_splits in csrc/fsk_tc_kde16.cu, which bounds the FP64
partial buffers), so the Triton tuning names below -- SplitKParams,
SymmetricParams, compute_splitk_splits, cap_splits_for_memory,
iter_autotune_candidates -- are kept only so code written against the
reference's module still imports and computes the same numbers; nothing in
this package's kernel path calls them.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Iterable

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
    PRECISION_FAST_TF32,
    PRECISION_FP32_IEEE,
)


@dataclass(frozen=True)
class SplitKParams:
    block_m: int
    block_n_iter: int
    iters_per_split: int
    num_warps: int
    num_stages: int


@dataclass(frozen=True)
class SymmetricParams:
    block_size: int
    num_warps: int
    num_stages: int


@dataclass(frozen=True)
class KernelHeuristics:
    n_sym_max: int = 50_000
    max_partial_weighted_bytes: int = 256 * 1024 * 1024
    eps: float = DEFAULT_EPS
    default_precision_mode: str = DEFAULT_PRECISION_MODE
    default_kde_backend: str = DEFAULT_KDE_BACKEND
    default_emp_score_backend: str = DEFAULT_EMP_SCORE_BACKEND


DEFAULT_HEURISTICS = KernelHeuristics()


def validate_precision_mode(precision_mode: str) -> None:
    valid = {PRECISION_FAST_TF32, PRECISION_FP32_IEEE}
    if precision_mode not in valid:
        raise ValueError(f"precision_mode must be one of {sorted(valid)}, got {precision_mode}.")


def validate_kde_backend(kde_backend: str) -> None:
    valid = {KDE_BACKEND_SPLITK_STREAM, KDE_BACKEND_ATOMIC}
    if kde_backend not in valid:
        raise ValueError(f"kde_backend must be one of {sorted(valid)}, got {kde_backend}.")


def validate_emp_score_backend(emp_score_backend: str) -> None:
    valid = {
        EMP_SCORE_BACKEND_ORDERED_SPLITK,
        EMP_SCORE_BACKEND_SYMMETRIC_ATOMIC,
        EMP_SCORE_BACKEND_FLASH_SD_KDE,
    }
    if emp_score_backend not in valid:
        raise ValueError(f"emp_score_backend must be one of {sorted(valid)}, got {emp_score_backend}.")


def select_emp_score_backend(n: int, *, heuristics: KernelHeuristics = DEFAULT_HEURISTICS) -> str:
    if heuristics.default_emp_score_backend == EMP_SCORE_BACKEND_FLASH_SD_KDE:
        return EMP_SCORE_BACKEND_FLASH_SD_KDE
    if n <= heuristics.n_sym_max:
        return EMP_SCORE_BACKEND_SYMMETRIC_ATOMIC
    return EMP_SCORE_BACKEND_ORDERED_SPLITK


def compute_splitk_splits(n_data: int, *, block_n_iter: int, iters_per_split: int) -> int:
    """Compatibility name: split count of the reference's Triton split-K grid
    (ceil(n_data / (block_n_iter * iters_per_split))); not used by the GB300
    kernels."""
    total = block_n_iter * iters_per_split
    if total <= 0:
        raise ValueError("block_n_total must be positive.")
    return int((n_data + total - 1) // total)


def cap_splits_for_memory(
    n_query: int,
    n_splits: int,
    *,
    features: int,
    heuristics: KernelHeuristics = DEFAULT_HEURISTICS,
) -> int:
    """Compatibility name: the largest split count whose FP32 weighted
    partials (n_query x features per split) fit the heuristic byte budget.
    The GB300 path bounds its own FP64 partial buffers in the C planner."""
    if n_splits <= 1:
        return n_splits
    bytes_per_split = n_query * features * 4
    if bytes_per_split <= 0:
        return n_splits
    max_splits = max(1, heuristics.max_partial_weighted_bytes // bytes_per_split)
    return int(min(n_splits, max_splits))


def iter_autotune_candidates(candidates: Iterable[SplitKParams]) -> list[SplitKParams]:
    """Compatibility name: the Triton autotune candidates as a list (the GB300
    kernels have fixed tile shapes and no autotuning)."""
    return list(candidates)
