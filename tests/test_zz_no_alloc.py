"""fsk_kde16_noalloc: the 16-D KDE for callers that cannot allocate device
memory (C-ABI/FFI hosts without a device allocator, processes whose GPU
memory another allocator owns, loops where cudaMalloc/cudaFree would
synchronise the device).  It keeps its scratch in a fixed device array
instead of a caller workspace.

Called through the C ABI with ctypes and compared with the workspace entry
point fsk_kde16 on two calls in a row (the array keeps the previous call's
contents, so the second call also shows nothing leaks between calls), at the
1e-6 relative tolerance used for same-path comparisons in these tests.  A
request larger than the array must be refused with FSK_ERR_SCRATCH_LIMIT.
This file is collected last so a stop-at-first-failure run has already run
every other test.
"""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _workspace_call(lib, q, x, h, flags, scale):
    out = torch.empty(q.shape[0], dtype=torch.float32, device=q.device)
    ws = torch.empty(max(lib.fsk_kde16_workspace_bytes(q.shape[0], x.shape[0], flags), 256),
                     dtype=torch.uint8, device=q.device)
    st = lib.fsk_kde16(q.data_ptr(), q.shape[0], x.data_ptr(), x.shape[0], h, flags, scale, 0.0,
                       out.data_ptr(), ws.data_ptr(), ws.numel(), torch.cuda.current_stream().cuda_stream)
    return st, out


def _noalloc_call(lib, q, x, h, flags, scale):
    out = torch.empty(q.shape[0], dtype=torch.float32, device=q.device)
    st = lib.fsk_kde16_noalloc(q.data_ptr(), q.shape[0], x.data_ptr(), x.shape[0], h, flags, scale, 0.0,
                               out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    return st, out


def test_noalloc_matches_workspace_entry_point(cuda_dev):
    from fsk import _lib as L
    from fsk import ops

    lib = L.load()
    # two calls in a row with different sizes, data and options
    cases = [(3001, 1000, 0.7, 0), (4096, 777, 0.55, L.FSK_ATOMIC)]
    for seed, (n, m, h, flags) in enumerate(cases):
        rng = np.random.default_rng(100 + seed)
        x = torch.from_numpy(rng.standard_normal((n, 16)).astype(np.float32)).to(cuda_dev)
        q = torch.from_numpy((rng.standard_normal((m, 16)) * 0.9).astype(np.float32)).to(cuda_dev)
        scale = 1.0 / ((2.0 * math.pi) ** 8 * h ** 16 * n)
        st_ref, ref = _workspace_call(lib, q, x, h, flags, scale)
        st, got = _noalloc_call(lib, q, x, h, flags, scale)
        assert st_ref == L.FSK_OK and st == L.FSK_OK
        ops.device_status(cuda_dev)
        a, b = got.cpu().numpy().astype(np.float64), ref.cpu().numpy().astype(np.float64)
        assert np.all(np.isfinite(a))
        np.testing.assert_allclose(a, b, rtol=1e-6, atol=0.0)


def test_noalloc_rejects_requests_beyond_its_scratch(cuda_dev):
    from fsk import _lib as L

    lib = L.load()
    n = m = 1 << 18          # needs ~84 MB of scratch, more than the fixed array holds
    assert lib.fsk_kde16_workspace_bytes(m, n, 0) > (32 << 20)
    x = torch.zeros((n, 16), dtype=torch.float32, device=cuda_dev)
    st, _ = _noalloc_call(lib, x, x, 1.0, 0, 1.0)
    assert st == L.FSK_ERR_SCRATCH_LIMIT
    assert "scratch" in L.strerror(st)
