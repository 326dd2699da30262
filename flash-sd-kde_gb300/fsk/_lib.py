"""ctypes binding of libfsk.so (the C ABI declared in include/fsk.h).

The library is loaded from this directory only; there is no fallback: if it is
missing or fails to load, every op raises RuntimeError.
"""
from __future__ import annotations

import ctypes
import os
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libfsk.so"

# status codes (include/fsk.h)
FSK_OK = 0
FSK_ERR_INVALID_ARGUMENT = 1
FSK_ERR_WORKSPACE_TOO_SMALL = 2
FSK_ERR_CUDA = 3
FSK_ERR_DEVICE_TIMEOUT = 4
FSK_ERR_UNSUPPORTED_DEVICE = 5
FSK_ERR_SCRATCH_LIMIT = 6
FSK_ERR_DEVICE_BOUNDS = 7

# flags
FSK_PREC_TENSOR = 0x0
FSK_PREC_IEEE = 0x1
FSK_LAPLACE = 0x2
FSK_OUT_LOG = 0x4
FSK_ATOMIC = 0x8
FSK_WEIGHTED_FEATURE_MAJOR = 0x10
FSK_OUT_LOG_EXACT = 0x20
FSK_PREC_FP16_SINGLE = 0x40
FSK_EXP_OFFLOAD = 0x80

FSK_ND_MAX = 64
FSK_NOALLOC_SCRATCH_BYTES = 32 << 20

FSK_SCORE_ORDERED = 0
FSK_SCORE_SYMMETRIC = 1

FSK_MLP_IN = 16
FSK_MLP_HIDDEN = 256
FSK_MLP_PARAMS = 136193

FSK_RULE_SILVERMAN = 0
FSK_RULE_SDKDE_1D = 1

_c = ctypes
_vp = _c.c_void_p
_i64 = _c.c_int64
_sz = _c.c_size_t
_d = _c.c_double
_int = _c.c_int

# name -> (restype, argtypes); every symbol fsk.h declares
SIGNATURES: dict[str, tuple] = {
    "fsk_kde16_workspace_bytes": (_sz, [_i64, _i64, _int]),
    "fsk_kde16": (_int, [_vp, _i64, _vp, _i64, _d, _int, _d, _d, _vp, _vp, _sz, _vp]),
    "fsk_kde16_noalloc": (_int, [_vp, _i64, _vp, _i64, _d, _int, _d, _d, _vp, _vp]),
    "fsk_kde_nd_workspace_bytes": (_sz, [_i64, _i64, _int, _int]),
    "fsk_kde_nd": (_int, [_vp, _i64, _vp, _i64, _int, _d, _int, _d, _d, _vp, _vp, _sz, _vp]),
    "fsk_empscore_nd_workspace_bytes": (_sz, [_i64, _int]),
    "fsk_empscore_nd": (_int, [_vp, _i64, _int, _d, _vp, _vp, _vp, _sz, _vp]),
    "fsk_debias_nd": (_int, [_vp, _i64, _int, _vp, _vp, _d, _d, _vp, _vp, _vp]),
    "fsk_empscore16_workspace_bytes": (_sz, [_i64, _int, _int]),
    "fsk_empscore16": (_int, [_vp, _i64, _d, _int, _int, _vp, _vp, _vp, _sz, _vp]),
    "fsk_debias16": (_int, [_vp, _i64, _vp, _vp, _i64, _i64, _d, _d, _vp, _vp, _vp]),
    "fsk_sdkde16_workspace_bytes": (_sz, [_i64, _i64, _int]),
    "fsk_sdkde16": (_int, [_vp, _i64, _vp, _i64, _d, _int, _d, _d, _d, _vp, _vp, _vp, _sz, _vp]),
    "fsk_kde1d_workspace_bytes": (_sz, [_i64, _i64, _int]),
    "fsk_kde1d": (_int, [_vp, _i64, _vp, _i64, _d, _int, _d, _d, _vp, _vp, _sz, _vp]),
    "fsk_kde1d_score": (_int, [_vp, _i64, _vp, _i64, _d, _vp, _vp, _vp, _vp, _sz, _vp]),
    "fsk_silverman_workspace_bytes": (_sz, [_i64, _int]),
    "fsk_silverman": (_int, [_vp, _i64, _int, _int, _vp, _vp, _sz, _vp]),
    "fsk_reduce_partials": (_int, [_vp, _i64, _i64, _vp, _vp]),
    "fsk_mlp_train_workspace_bytes": (_sz, [_int, _i64]),
    "fsk_mlp_fwd": (_int, [_vp, _int, _vp, _i64, _vp, _vp, _vp, _vp, _sz, _vp]),
    "fsk_mlp_bwd": (_int, [_vp, _int, _i64, _vp, _vp, _vp, _sz, _vp]),
    "fsk_mlp_mse": (_int, [_vp, _vp, _i64, _int, _vp, _vp, _vp]),
    "fsk_mlp_adam": (_int, [_vp, _vp, _vp, _vp, _i64, _c.c_float, _c.c_float, _c.c_float, _c.c_float,
                            _c.c_float, _int, _vp]),
    "fsk_mlp_packed_bytes": (_sz, [_int]),
    "fsk_mlp_pack": (_int, [_vp, _int, _vp, _vp, _c.c_float, _c.c_float, _vp, _vp]),
    "fsk_mlp_infer": (_int, [_vp, _int, _vp, _i64, _vp, _vp]),
    "fsk_mlp_combine": (_int, [_vp, _int, _i64, _vp, _vp, _vp, _c.c_float, _c.c_float, _c.c_float, _c.c_float,
                               _vp, _vp, _vp, _vp]),
    "fsk_device_status": (_int, [_vp]),
    "fsk_strerror": (_c.c_char_p, [_int]),
    "fsk_version": (_int, []),
    "fsk_launch_count": (_i64, []),
    "fsk_diag_mma_probe": (_int, [_vp, _vp, _vp, _vp]),
    "fsk_diag_mma_ts_probe": (_int, [_vp, _vp, _vp, _vp]),
    "fsk_diag_tmem_cp_probe": (_int, [_vp, _vp, _vp]),
    "fsk_diag_wait_timeout_probe": (_int, [_vp, _vp]),
    "fsk_diag_pipe_rates": (_int, [_vp, _vp]),
    "fsk_timer_enable": (None, [_int]),
    "fsk_timer_collect": (_int, [_vp, _vp, _vp, _vp, _int]),
}

_lock = threading.Lock()
_lib = None


def load(path: str | os.PathLike | None = None):
    """Load libfsk.so (once) and attach the ctypes signatures."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = Path(path) if path is not None else LIB_PATH
        if not p.exists():
            raise RuntimeError(
                f"{p} is missing: build the CUDA extension first "
                "(python -c 'import __graft_entry__ as g; g.build()')"
            )
        lib = ctypes.CDLL(str(p))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if path is None:
            _lib = lib
        return lib


def strerror(status: int) -> str:
    return load().fsk_strerror(status).decode()


class FskError(RuntimeError):
    """A non-argument failure reported by libfsk (CUDA error, device timeout...)."""

    def __init__(self, status: int, what: str):
        super().__init__(f"{what}: {strerror(status)} (status {status})")
        self.status = status


def check(status: int, what: str) -> None:
    """Map an fsk status to the reference's exception types."""
    if status == FSK_OK:
        return
    if status == FSK_ERR_INVALID_ARGUMENT:
        raise ValueError(f"{what}: {strerror(status)}")
    raise FskError(status, what)
