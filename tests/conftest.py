"""Shared pytest setup: import paths, the `gpu` marker, golden fixtures and a
session fixture that builds/loads libfsk.so on a GPU host."""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "flash-sd-kde_gb300"
for p in (str(PKG), str(ROOT)):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the libfsk.so CUDA extension")


@pytest.fixture(scope="session")
def golden():
    cache: dict[str, dict] = {}

    def load(name: str) -> dict:
        if name not in cache:
            with np.load(GOLDEN / f"{name}.npz") as z:
                cache[name] = {k: z[k] for k in z.files}
        return cache[name]

    return load


@pytest.fixture(scope="session")
def cuda_dev():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("CUDA not available")
    from fsk import _build, _lib

    _build.build()          # no-op when libfsk.so is up to date
    _lib.load()
    return torch.device("cuda", 0)


def rel_err(a, b) -> np.ndarray:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
