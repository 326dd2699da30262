"""fsk_kde16_noalloc: the 16-D KDE for callers that cannot allocate device
memory (C-ABI/FFI hosts without a device allocator, processes whose GPU
memory another allocator owns, loops where cudaMalloc/cudaFree would
synchronise the device).  It keeps its scratch in a fixed device array
instead of a caller workspace.

Called through the C ABI with ctypes and compared with the workspace entry
point fsk_kde16, at the 1e-6 relative tolerance used for same-path
comparisons in these tests.  A large call runs first, then smaller calls of
every scratch layout (tensor-core split partials, the FP64 atomic
accumulator, the CUDA-core partials, the exact-log lists) back to back, so
each later call runs over the stale contents of the one before: equal
results show nothing leaks between calls.  The device's free memory and
torch's allocated bytes must not change across the calls (nothing is
allocated).  A request larger than the array must be refused with
FSK_ERR_SCRATCH_LIMIT.  This file is collected last so a stop-at-first-failure
run has already run every other test.
"""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _workspace_call(lib, q, x, h, flags, scale, eps):
    out = torch.empty(q.shape[0], dtype=torch.float32, device=q.device)
    ws = torch.empty(max(lib.fsk_kde16_workspace_bytes(q.shape[0], x.shape[0], flags), 256),
                     dtype=torch.uint8, device=q.device)
    st = lib.fsk_kde16(q.data_ptr(), q.shape[0], x.data_ptr(), x.shape[0], h, flags, scale, eps,
                       out.data_ptr(), ws.data_ptr(), ws.numel(), torch.cuda.current_stream().cuda_stream)
    return st, out


def _noalloc_call(lib, q, x, h, flags, scale, eps, out):
    return lib.fsk_kde16_noalloc(q.data_ptr(), q.shape[0], x.data_ptr(), x.shape[0], h, flags, scale, eps,
                                 out.data_ptr(), torch.cuda.current_stream().cuda_stream)


def test_noalloc_matches_workspace_entry_point(cuda_dev):
    from fsk import _lib as L
    from fsk import ops

    lib = L.load()
    log_exact = L.FSK_OUT_LOG | L.FSK_OUT_LOG_EXACT
    # (n, m, h, flags): a large call first, then smaller ones of each scratch layout
    cases = [(50000, 40000, 0.7, 0), (3001, 1000, 0.7, 0), (4096, 777, 0.55, L.FSK_ATOMIC),
             (2500, 513, 0.6, L.FSK_PREC_IEEE), (3000, 900, 0.5, log_exact), (1000, 300, 0.8, 0)]
    inputs = []
    for seed, (n, m, h, flags) in enumerate(cases):
        rng = np.random.default_rng(100 + seed)
        x = torch.from_numpy(rng.standard_normal((n, 16)).astype(np.float32)).to(cuda_dev)
        qn = rng.standard_normal((m, 16)) * 0.9
        if flags & L.FSK_OUT_LOG_EXACT:
            qn[::3] += 6.0      # ~24 from the data: these queries' FP32 sums underflow
        q = torch.from_numpy(qn.astype(np.float32)).to(cuda_dev)
        scale = 1.0 / ((2.0 * math.pi) ** 8 * h ** 16 * n)
        assert lib.fsk_kde16_workspace_bytes(m, n, flags) <= L.FSK_NOALLOC_SCRATCH_BYTES
        st_ref, ref = _workspace_call(lib, q, x, h, flags, scale, 0.0)
        assert st_ref == L.FSK_OK
        inputs.append((x, q, h, flags, scale, ref, torch.empty_like(ref)))
    ops.device_status(cuda_dev)
    # warm-up call (loads the library's device code into the context if needed)
    x, q, h, flags, scale, _, out = inputs[-1]
    assert _noalloc_call(lib, q, x, h, flags, scale, 0.0, out) == L.FSK_OK
    ops.device_status(cuda_dev)
    free0, alloc0 = torch.cuda.mem_get_info(cuda_dev)[0], torch.cuda.memory_allocated(cuda_dev)
    for rep in range(2):     # two passes over all cases: every call follows another layout
        for x, q, h, flags, scale, _, out in inputs:
            assert _noalloc_call(lib, q, x, h, flags, scale, 0.0, out) == L.FSK_OK
        ops.device_status(cuda_dev)
        for x, q, h, flags, scale, ref, out in inputs:
            a, b = out.cpu().numpy().astype(np.float64), ref.cpu().numpy().astype(np.float64)
            assert np.all(np.isfinite(a))
            if flags & L.FSK_OUT_LOG_EXACT:     # log-densities: compare on the density scale
                np.testing.assert_allclose(a, b, rtol=0.0, atol=1e-6)
            else:
                np.testing.assert_allclose(a, b, rtol=1e-6, atol=0.0)
    assert torch.cuda.mem_get_info(cuda_dev)[0] == free0
    assert torch.cuda.memory_allocated(cuda_dev) == alloc0


def test_noalloc_rejects_requests_beyond_its_scratch(cuda_dev):
    from fsk import _lib as L

    lib = L.load()
    n = m = 1 << 18          # needs ~84 MB of scratch, more than the fixed array holds
    assert lib.fsk_kde16_workspace_bytes(m, n, 0) > L.FSK_NOALLOC_SCRATCH_BYTES
    x = torch.zeros((n, 16), dtype=torch.float32, device=cuda_dev)
    out = torch.empty(m, dtype=torch.float32, device=cuda_dev)
    assert _noalloc_call(lib, x, x, 1.0, 0, 1.0, 0.0, out) == L.FSK_ERR_SCRATCH_LIMIT
    assert "scratch" in L.strerror(L.FSK_ERR_SCRATCH_LIMIT)
    # argument errors come first, as fsk_kde16 reports them
    assert _noalloc_call(lib, x, x, -1.0, 0, 1.0, 0.0, out) == L.FSK_ERR_INVALID_ARGUMENT
    assert _noalloc_call(lib, x, x, 1.0, 0x4000, 1.0, 0.0, out) == L.FSK_ERR_INVALID_ARGUMENT
