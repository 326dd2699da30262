"""The C-ABI library loads and exports every symbol include/fsk.h declares;
argument checks happen on the host before any device work.  CPU only (no
compute call reaches a GPU)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADERS = sorted((ROOT / "include").glob("*.h"))


@pytest.fixture(scope="module")
def lib():
    from fsk import _build, _lib

    _build.build()
    return _lib.load()


def declared_symbols():
    names = []
    for h in HEADERS:
        names += re.findall(r"FSK_API\s+[\w\s\*]+?\b(fsk_\w+)\s*\(", h.read_text())
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_symbols()
    for required in ("fsk_kde16", "fsk_empscore16", "fsk_debias16", "fsk_kde1d", "fsk_kde1d_score",
                     "fsk_silverman", "fsk_reduce_partials", "fsk_device_status", "fsk_strerror"):
        assert required in names


def test_every_declared_symbol_is_exported(lib):
    from fsk import _lib

    raw = ctypes.CDLL(str(_lib.LIB_PATH))
    for name in declared_symbols():
        assert hasattr(raw, name), name
        assert name in _lib.SIGNATURES, f"{name} has no ctypes signature"


def test_status_strings(lib):
    from fsk import _lib as L

    assert lib.fsk_version() >= 10000
    for code in range(7):
        assert L.strerror(code)
    assert "timed out" in L.strerror(L.FSK_ERR_DEVICE_TIMEOUT)


def test_argument_validation_is_host_side(lib):
    from fsk import _lib as L

    inval = L.FSK_ERR_INVALID_ARGUMENT
    assert lib.fsk_kde16(None, 10, None, 10, 1.0, 0, 1.0, 0.0, None, None, 0, None) == inval
    fake = ctypes.c_void_p(16)   # never dereferenced: the checks fail first
    assert lib.fsk_kde16(fake, 0, fake, 10, 1.0, 0, 1.0, 0.0, fake, fake, 1 << 20, None) == inval
    assert lib.fsk_kde16(fake, 10, fake, 10, -1.0, 0, 1.0, 0.0, fake, fake, 1 << 20, None) == inval
    assert lib.fsk_kde16(fake, 10, fake, 10, float("inf"), 0, 1.0, 0.0, fake, fake, 1 << 20, None) == inval
    assert lib.fsk_kde16(fake, 10, fake, 10, 1.0, 0x1000, 1.0, 0.0, fake, fake, 1 << 20, None) == inval
    # exact log output: needs FSK_OUT_LOG and out_eps = 0
    assert lib.fsk_kde16(fake, 10, fake, 10, 1.0, L.FSK_OUT_LOG_EXACT, 1.0, 0.0, fake, fake, 1 << 20, None) == inval
    assert lib.fsk_kde16(fake, 10, fake, 10, 1.0, L.FSK_OUT_LOG_EXACT | L.FSK_OUT_LOG, 1.0, 1e-12, fake, fake,
                         1 << 20, None) == inval
    assert lib.fsk_empscore16(fake, 10, 1.0, 7, 0, fake, fake, fake, 1 << 20, None) == inval
    # any-d entry points: 1 <= d <= FSK_ND_MAX, known flags, eps >= 0
    for d in (0, L.FSK_ND_MAX + 1):
        assert lib.fsk_kde_nd(fake, 10, fake, 10, d, 1.0, 0, 1.0, 0.0, fake, fake, 1 << 20, None) == inval
        assert lib.fsk_empscore_nd(fake, 10, d, 1.0, fake, fake, fake, 1 << 20, None) == inval
        assert lib.fsk_debias_nd(fake, 10, d, fake, fake, 1.0, 0.0, fake, None, None) == inval
        assert lib.fsk_kde_nd_workspace_bytes(10, 10, d, 0) == 0
        assert lib.fsk_empscore_nd_workspace_bytes(10, d) == 0
    assert lib.fsk_kde_nd(fake, 10, fake, 10, 20, 1.0, L.FSK_OUT_LOG_EXACT, 1.0, 0.0, fake, fake, 1 << 20,
                          None) == inval
    assert lib.fsk_debias_nd(fake, 10, 20, fake, fake, 1.0, -1.0, fake, None, None) == inval
    assert lib.fsk_silverman(fake, 10, 65, 0, fake, fake, 1 << 20, None) == inval
    assert lib.fsk_silverman(fake, 10, 2, 1, fake, fake, 1 << 20, None) == inval
    assert lib.fsk_kde1d(fake, 10, fake, 0, 1.0, 0, 1.0, 0.0, fake, fake, 1 << 20, None) == inval
    assert lib.fsk_reduce_partials(fake, 0, 10, fake, None) == inval
    assert lib.fsk_mlp_fwd(fake, 0, fake, 10, fake, fake, fake, fake, 1 << 20, None) == inval
    assert lib.fsk_mlp_fwd(fake, 9, fake, 10, fake, fake, fake, fake, 1 << 20, None) == inval
    assert lib.fsk_mlp_bwd(fake, 2, 0, fake, fake, fake, 1 << 20, None) == inval
    assert lib.fsk_mlp_adam(fake, fake, fake, fake, 10, 1e-3, 1.0, 0.999, 1e-8, 0.0, 1, None) == inval
    assert lib.fsk_mlp_adam(fake, fake, fake, fake, 10, 1e-3, 0.9, 0.999, 1e-8, 0.0, 0, None) == inval
    assert lib.fsk_mlp_infer(fake, 4, 17, 10, fake, None) == inval        # misaligned x
    assert lib.fsk_mlp_combine(fake, 4, 10, fake, None, None, 0.0, 0.0, 1.0, 1.0, None, None, None, None) == inval


def test_workspace_sizes(lib):
    from fsk import _lib as L

    # the exact log output adds its list and per-part (dmin, sum) rows: >= 100 B per query
    plain = lib.fsk_kde16_workspace_bytes(1 << 16, 1 << 16, L.FSK_OUT_LOG)
    exact = lib.fsk_kde16_workspace_bytes(1 << 16, 1 << 16, L.FSK_OUT_LOG | L.FSK_OUT_LOG_EXACT)
    assert exact >= plain + 100 * (1 << 16)
    a = lib.fsk_kde16_workspace_bytes(1 << 10, 1 << 12, 0)
    b = lib.fsk_kde16_workspace_bytes(1 << 20, 1 << 20, 0)
    assert 0 < a < b
    assert lib.fsk_kde16_workspace_bytes(0, 10, 0) == 0
    assert lib.fsk_mlp_train_workspace_bytes(4, 8192) >= 4 * 8192 * 256 * 4 * 7
    assert lib.fsk_mlp_train_workspace_bytes(0, 8192) == 0
    assert lib.fsk_mlp_packed_bytes(4) == 4 * (256 + 4096 + 8192 + 2 * 16 * 8192)
    assert lib.fsk_empscore16_workspace_bytes(1 << 16, 0, 0) > (1 << 16) * 17 * 8
    assert lib.fsk_silverman_workspace_bytes(100, 16) > 0
