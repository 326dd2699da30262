"""The bounds-check build (libfsk_checked.so, compiled with -DFSK_BOUNDS_CHECK
by fsk._build.build(checked=True)): the hot kernels check the index of every
global write against the extent of the buffer it goes to and report
FSK_ERR_DEVICE_BOUNDS (the write skipped, nothing traps) instead of writing
out of range.  Run through the library's ops at tiny, ragged and tile-boundary
sizes of every path (tensor-core and CUDA-core KDE, ordered, symmetric and
any-d score, debias, exact-log output, 1-D KDE and score, one-call SD-KDE,
partial reduction), the checked library reports no out-of-range index and
returns bitwise the values of the normal library.  Compiling the checked
library takes a minute or two the first time.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1), (129, 257), (1000, 513), (4097, 300), (20000, 3000)]


def _run_all(dev):
    from fsk import ops

    outs = []
    rng = np.random.default_rng(3)
    for n, m in SHAPES:
        x = torch.from_numpy(rng.standard_normal((n, 16)).astype(np.float32)).to(dev)
        q = torch.from_numpy((rng.standard_normal((m, 16)) * 0.9).astype(np.float32)).to(dev)
        h = 0.8
        for prec in ("tensor", "ieee"):
            outs.append(ops.kde16_sum(q, x, h, precision=prec))
            outs.append(ops.kde16_sum(q, x, h, precision=prec, atomic=True))
            outs.append(ops.kde16_sum(q + 9.0, x, h, precision=prec, log_exact=True))
            for variant in ("ordered", "symmetric"):
                outs += list(ops.empscore16(x, h, variant=variant, precision=prec))
            outs += list(ops.empscore16(x, h, feature_major=True, precision=prec))
            outs.append(ops.sdkde16(x, q, h, precision=prec))
        pdf, w = ops.empscore16(x, h)
        outs.append(ops.debias16(x, pdf, w, h, 1e-12))
        outs += list(ops.empscore_nd(x[:, :11].contiguous(), h))
        outs.append(ops.kde_nd_sum(q[:, :11].contiguous(), x[:, :11].contiguous(), h))
        x1 = x[:, 0].contiguous()
        q1 = q[:, 0].contiguous()
        outs.append(ops.kde1d_sum(q1, x1, 0.3))
        outs.append(ops.kde1d_sum(q1, x1, 0.3, atomic=True))
        outs += [t for t in ops.kde1d_score(q1, x1, 0.3) if isinstance(t, torch.Tensor)]
    from kernels.reduce_partials import reduce_pdf_partials

    outs.append(reduce_pdf_partials(torch.rand((7, 1001), device=dev, generator=torch.Generator(dev).manual_seed(1))))
    ops.device_status(dev)
    return [t.detach().cpu() for t in outs]


def test_checked_build_reports_nothing_and_matches(cuda_dev, monkeypatch):
    from fsk import _build
    from fsk import _lib as L

    ref = _run_all(cuda_dev)
    checked = L.load(_build.build(checked=True))
    normal = L.load()
    monkeypatch.setattr(L, "_lib", checked)
    assert L.load() is checked
    got = _run_all(cuda_dev)       # device_status raises on FSK_ERR_DEVICE_BOUNDS
    monkeypatch.setattr(L, "_lib", normal)
    assert len(got) == len(ref)
    for a, b in zip(got, ref):
        # bitwise, except the atomic accumulations (order-dependent)
        assert a.shape == b.shape and a.dtype == b.dtype
        assert torch.equal(torch.isfinite(a), torch.isfinite(b))
        fin = torch.isfinite(b)
        assert torch.allclose(a[fin].double(), b[fin].double(), rtol=1e-6, atol=0.0)
    assert "bounds" in L.strerror(L.FSK_ERR_DEVICE_BOUNDS)
