"""Tensor-level wrappers over the libfsk C ABI.

Every op takes CUDA float32 tensors (converted with ``.to(device, float32,
copy=False).contiguous()`` like the reference's ``_to_matrix_tensor``), takes
its device workspace from torch's caching allocator, enqueues the kernels on
the current torch stream of the tensors' device and returns new tensors.
Nothing here runs on the CPU: a missing extension or a non-CUDA device is an
error.
"""
from __future__ import annotations

import math
from typing import Sequence

import torch

from . import _lib as L

ND_FEATURES = 16


def _device(device) -> torch.device:
    dev = torch.device(device)
    if dev.type != "cuda":
        raise ValueError("the GB300 kernels require a CUDA device.")
    if not torch.cuda.is_available():
        raise RuntimeError("CUDA is not available but was requested.")
    if dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    return dev


def as_matrix(x: Sequence[Sequence[float]] | torch.Tensor, device: torch.device, dim: int = ND_FEATURES) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        t = x.to(device=device, dtype=torch.float32, copy=False)
    else:
        t = torch.as_tensor(x, dtype=torch.float32, device=device)
    if t.ndim != 2 or t.shape[1] != dim:
        raise ValueError(f"expected tensor with shape (n, {dim}), got {tuple(t.shape)}")
    return t.contiguous()


def as_padded_matrix(x: Sequence[Sequence[float]] | torch.Tensor, device: torch.device,
                     width: int = ND_FEATURES) -> tuple[torch.Tensor, int]:
    """(n, d) rows with 1 <= d <= width as a contiguous (n, width) FP32 tensor,
    zero-padded, and d.  Zero coordinates add nothing to any squared distance,
    so every pairwise Gaussian sum (and weighted sum, in the first d columns)
    of the padded rows equals that of the original rows."""
    if isinstance(x, torch.Tensor):
        t = x.to(device=device, dtype=torch.float32, copy=False)
    else:
        t = torch.as_tensor(x, dtype=torch.float32, device=device)
    if t.ndim != 2 or not 1 <= t.shape[1] <= width:
        raise ValueError(f"expected tensor with shape (n, d), 1 <= d <= {width}, got {tuple(t.shape)}")
    d = int(t.shape[1])
    if d < width:
        t = torch.nn.functional.pad(t, (0, width - d))
    return t.contiguous(), d


def as_vector(x: Sequence[float] | torch.Tensor, device: torch.device) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        t = x.to(device=device, dtype=torch.float32, copy=False)
    else:
        t = torch.as_tensor(x, dtype=torch.float32, device=device)
    if t.ndim != 1:
        raise ValueError("expected a 1D tensor.")
    return t.contiguous()


def _ptr(t: torch.Tensor | None):
    return None if t is None else t.data_ptr()


def _stream(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def _workspace(nbytes: int, device: torch.device) -> torch.Tensor:
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)


def _check_bw(h: float) -> float:
    h = float(h)
    if not (h > 0.0) or not math.isfinite(h):
        raise ValueError("bandwidth must be positive.")
    return h


def kde16_sum(
    queries: torch.Tensor,
    data: torch.Tensor,
    bandwidth: float,
    *,
    precision: str = "tensor",
    laplace: bool = False,
    atomic: bool = False,
    out_scale: float = 1.0,
    log_eps: float | None = None,
    log_exact: bool = False,
    out: torch.Tensor | None = None,
    exp_offload: bool = False,
) -> torch.Tensor:
    """out[i] = out_scale * sum_j phi(q_i, x_j)  (or log(out_scale*sum + log_eps)).

    precision "tensor" (three-part fp16 tensor-core products + exact near-pair
    recompute), "ieee" (FP32 direct differences, CUDA cores) or "fp16_single"
    (one fp16 cross product, no recompute: the lowest precision rung).

    log_exact: out[i] = log(out_scale * sum) without the eps floor and without
    underflow (queries whose sum underflows are recomputed with a
    running-minimum shift); needs log_eps None or 0.
    """
    h = _check_bw(bandwidth)
    dev = _device(queries.device)
    q = as_matrix(queries, dev)
    x = as_matrix(data, dev)
    m, n = q.shape[0], x.shape[0]
    if m == 0 or n == 0:
        raise ValueError("data and queries must contain at least one sample.")
    if precision not in ("tensor", "ieee", "fp16_single"):
        raise ValueError(f"unknown precision {precision!r}")
    flags = {"tensor": L.FSK_PREC_TENSOR, "ieee": L.FSK_PREC_IEEE, "fp16_single": L.FSK_PREC_FP16_SINGLE}[precision]
    flags |= (L.FSK_LAPLACE if laplace else 0) | (L.FSK_ATOMIC if atomic else 0)
    flags |= L.FSK_EXP_OFFLOAD if exp_offload else 0
    if log_exact:
        if log_eps:
            raise ValueError("log_exact takes no log_eps (the log is taken without a floor).")
        log_eps = 0.0
        flags |= L.FSK_OUT_LOG_EXACT
    if log_eps is not None:
        flags |= L.FSK_OUT_LOG
    lib = L.load()
    with torch.cuda.device(dev):
        if out is None:
            out = torch.empty(m, dtype=torch.float32, device=dev)
        ws_bytes = lib.fsk_kde16_workspace_bytes(m, n, flags)
        ws = _workspace(ws_bytes, dev)
        st = lib.fsk_kde16(q.data_ptr(), m, x.data_ptr(), n, h, flags, float(out_scale),
                           float(log_eps or 0.0), out.data_ptr(), ws.data_ptr(), ws.numel(), _stream(dev))
    L.check(st, "fsk_kde16")
    return out


def empscore16(
    data: torch.Tensor,
    bandwidth: float,
    *,
    variant: str = "ordered",
    feature_major: bool = False,
    precision: str = "tensor",
) -> tuple[torch.Tensor, torch.Tensor]:
    """(pdf_sum (n,), weighted_sum (n,16)); feature_major returns a (16,n)-backed view.

    precision "tensor": the tcgen05 kernel (both variants); "ieee": the
    CUDA-core kernel of the requested variant."""
    h = _check_bw(bandwidth)
    dev = _device(data.device)
    x = as_matrix(data, dev)
    n = x.shape[0]
    if n == 0:
        raise ValueError("data must contain at least one element.")
    var = L.FSK_SCORE_SYMMETRIC if variant == "symmetric" else L.FSK_SCORE_ORDERED
    flags = L.FSK_WEIGHTED_FEATURE_MAJOR if feature_major else 0
    flags |= L.FSK_PREC_IEEE if precision == "ieee" else L.FSK_PREC_TENSOR
    lib = L.load()
    with torch.cuda.device(dev):
        pdf = torch.empty(n, dtype=torch.float32, device=dev)
        w = torch.empty((ND_FEATURES, n) if feature_major else (n, ND_FEATURES), dtype=torch.float32, device=dev)
        ws = _workspace(lib.fsk_empscore16_workspace_bytes(n, var, flags), dev)
        st = lib.fsk_empscore16(x.data_ptr(), n, h, var, flags, pdf.data_ptr(), w.data_ptr(), ws.data_ptr(),
                                ws.numel(), _stream(dev))
    L.check(st, "fsk_empscore16")
    return pdf, (w.t() if feature_major else w)


def sdkde16(
    data: torch.Tensor,
    queries: torch.Tensor,
    bandwidth: float,
    *,
    precision: str = "tensor",
    eps: float = 1e-12,
    out_scale: float | None = None,
    log_eps: float | None = None,
    log_exact: bool = False,
    atomic: bool = False,
    return_debiased: bool = False,
    out: torch.Tensor | None = None,
    workspace: torch.Tensor | None = None,
):
    """SD-KDE in one library call (fsk_sdkde16): the ordered empirical score of
    `data`, the debias shift and the KDE of the debiased set at `queries`.
    out_scale defaults to the 16-D Gaussian normalisation 1/((2 pi)^8 h^16 n).
    A caller that replays the call (or captures it in a CUDA graph) passes a
    persistent `workspace` and `out`."""
    h = _check_bw(bandwidth)
    dev = _device(data.device)
    x = as_matrix(data, dev)
    q = as_matrix(queries, dev)
    n, m = x.shape[0], q.shape[0]
    if n == 0 or m == 0:
        raise ValueError("data and queries must contain at least one sample.")
    if precision not in ("tensor", "ieee"):
        raise ValueError(f"unknown precision {precision!r}")
    flags = (L.FSK_PREC_IEEE if precision == "ieee" else 0) | (L.FSK_ATOMIC if atomic else 0)
    if log_exact:
        if log_eps:
            raise ValueError("log_exact takes no log_eps (the log is taken without a floor).")
        log_eps = 0.0
        flags |= L.FSK_OUT_LOG_EXACT
    if log_eps is not None:
        flags |= L.FSK_OUT_LOG
    if out_scale is None:
        out_scale = 1.0 / ((2.0 * math.pi) ** 8 * h ** 16 * n)
    lib = L.load()
    with torch.cuda.device(dev):
        if out is None:
            out = torch.empty(m, dtype=torch.float32, device=dev)
        deb = torch.empty_like(x) if return_debiased else None
        if workspace is None:
            workspace = _workspace(lib.fsk_sdkde16_workspace_bytes(n, m, flags), dev)
        st = lib.fsk_sdkde16(x.data_ptr(), n, q.data_ptr(), m, h, flags, float(eps), float(out_scale),
                             float(log_eps or 0.0), _ptr(deb), out.data_ptr(), workspace.data_ptr(),
                             workspace.numel(), _stream(dev))
    L.check(st, "fsk_sdkde16")
    return (out, deb) if return_debiased else out


class SDKDEGraph:
    """The one-call SD-KDE pipeline captured once in a CUDA graph and replayed
    as a single launch: for repeated evaluations on fixed-shape buffers
    (small problems, where launching ~20 kernels one by one costs more than
    running them).  Copy new inputs into .data / .queries, call replay(),
    read .out."""

    def __init__(self, data: torch.Tensor, queries: torch.Tensor, bandwidth: float, **kw):
        dev = _device(data.device)
        self.data = as_matrix(data, dev).clone()
        self.queries = as_matrix(queries, dev).clone()
        self.out = torch.empty(self.queries.shape[0], dtype=torch.float32, device=dev)
        flags = L.FSK_PREC_IEEE if kw.get("precision") == "ieee" else 0
        self.workspace = _workspace(L.load().fsk_sdkde16_workspace_bytes(self.data.shape[0], self.queries.shape[0],
                                                                         flags), dev)
        self._call = lambda: sdkde16(self.data, self.queries, bandwidth, out=self.out, workspace=self.workspace,
                                     **kw)
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):
            self._call()           # first call outside capture (one-time attribute setup)
        torch.cuda.current_stream(dev).wait_stream(side)
        torch.cuda.synchronize(dev)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, capture_error_mode="thread_local"):
            self._call()

    def replay(self) -> torch.Tensor:
        self.graph.replay()
        return self.out


def _as_rows(x, device: torch.device) -> torch.Tensor:
    t = x.to(device=device, dtype=torch.float32, copy=False) if isinstance(x, torch.Tensor) else \
        torch.as_tensor(x, dtype=torch.float32, device=device)
    if t.ndim != 2 or not 1 <= t.shape[1] <= L.FSK_ND_MAX:
        raise ValueError(f"expected tensor with shape (n, d), 1 <= d <= {L.FSK_ND_MAX}, got {tuple(t.shape)}")
    return t.contiguous()


def kde_nd_sum(queries, data, bandwidth: float, *, laplace: bool = False, out_scale: float = 1.0,
               log_eps: float | None = None) -> torch.Tensor:
    """out[i] = out_scale * sum_j phi(q_i, x_j) (or log(out_scale*sum + log_eps))
    for rows of any 1 <= d <= 64 features (CUDA-core kernel, fp32_ieee arithmetic)."""
    h = _check_bw(bandwidth)
    dev = _device(data.device if isinstance(data, torch.Tensor) else "cuda")
    q, x = _as_rows(queries, dev), _as_rows(data, dev)
    m, n, d = q.shape[0], x.shape[0], x.shape[1]
    if q.shape[1] != d:
        raise ValueError(f"data has {d} features but queries have {q.shape[1]}.")
    if m == 0 or n == 0:
        raise ValueError("data and queries must contain at least one sample.")
    flags = (L.FSK_LAPLACE if laplace else 0) | (L.FSK_OUT_LOG if log_eps is not None else 0)
    lib = L.load()
    with torch.cuda.device(dev):
        out = torch.empty(m, dtype=torch.float32, device=dev)
        ws = _workspace(lib.fsk_kde_nd_workspace_bytes(m, n, d, flags), dev)
        st = lib.fsk_kde_nd(q.data_ptr(), m, x.data_ptr(), n, d, h, flags, float(out_scale), float(log_eps or 0.0),
                            out.data_ptr(), ws.data_ptr(), ws.numel(), _stream(dev))
    L.check(st, "fsk_kde_nd")
    return out


def empscore_nd(data, bandwidth: float) -> tuple[torch.Tensor, torch.Tensor]:
    """(pdf_sum (n,), weighted_sum (n, d)) for rows of any 1 <= d <= 64 features."""
    h = _check_bw(bandwidth)
    dev = _device(data.device if isinstance(data, torch.Tensor) else "cuda")
    x = _as_rows(data, dev)
    n, d = x.shape
    if n == 0:
        raise ValueError("data must contain at least one element.")
    lib = L.load()
    with torch.cuda.device(dev):
        pdf = torch.empty(n, dtype=torch.float32, device=dev)
        w = torch.empty((n, d), dtype=torch.float32, device=dev)
        ws = _workspace(lib.fsk_empscore_nd_workspace_bytes(n, d), dev)
        st = lib.fsk_empscore_nd(x.data_ptr(), n, d, h, pdf.data_ptr(), w.data_ptr(), ws.data_ptr(), ws.numel(),
                                 _stream(dev))
    L.check(st, "fsk_empscore_nd")
    return pdf, w


def debias_nd(data, pdf_sum: torch.Tensor, weighted_sum: torch.Tensor, bandwidth: float, eps: float, *,
              return_score: bool = False):
    """The debias shift of debias16 for rows of any 1 <= d <= 64 features."""
    h = _check_bw(bandwidth)
    dev = _device(data.device if isinstance(data, torch.Tensor) else "cuda")
    x = _as_rows(data, dev)
    n, d = x.shape
    pdf = pdf_sum.to(device=dev, dtype=torch.float32).contiguous()
    w = weighted_sum.to(device=dev, dtype=torch.float32).contiguous()
    if w.shape != (n, d) or pdf.shape != (n,):
        raise ValueError("pdf_sum must be (n,) and weighted_sum (n, d).")
    lib = L.load()
    with torch.cuda.device(dev):
        deb = torch.empty_like(x)
        score = torch.empty_like(x) if return_score else None
        st = lib.fsk_debias_nd(x.data_ptr(), n, d, pdf.data_ptr(), w.data_ptr(), h, float(eps), deb.data_ptr(),
                               _ptr(score), _stream(dev))
    L.check(st, "fsk_debias_nd")
    return (deb, score) if return_score else deb


def debias16(
    data: torch.Tensor,
    pdf_sum: torch.Tensor,
    weighted_sum: torch.Tensor,
    bandwidth: float,
    eps: float,
    *,
    return_score: bool = False,
):
    """x + h^2/2 * score with score = (W/(pdf+eps) - x)/h^2, computed in FP64."""
    h = _check_bw(bandwidth)
    dev = _device(data.device)
    x = as_matrix(data, dev)
    n = x.shape[0]
    pdf = pdf_sum.to(device=dev, dtype=torch.float32).contiguous()
    w = weighted_sum.to(device=dev, dtype=torch.float32)
    if w.shape != (n, ND_FEATURES) or pdf.shape != (n,):
        raise ValueError("pdf_sum must be (n,) and weighted_sum (n, 16).")
    lib = L.load()
    with torch.cuda.device(dev):
        deb = torch.empty_like(x)
        score = torch.empty_like(x) if return_score else None
        st = lib.fsk_debias16(x.data_ptr(), n, pdf.data_ptr(), w.data_ptr(), w.stride(0), w.stride(1), h,
                              float(eps), deb.data_ptr(), _ptr(score), _stream(dev))
    L.check(st, "fsk_debias16")
    return (deb, score) if return_score else deb


def kde1d_sum(
    queries: torch.Tensor,
    data: torch.Tensor,
    bandwidth: float,
    *,
    laplace: bool = False,
    atomic: bool = False,
    out_scale: float = 1.0,
    log_eps: float | None = None,
) -> torch.Tensor:
    h = _check_bw(bandwidth)
    dev = _device(queries.device)
    q = as_vector(queries, dev)
    x = as_vector(data, dev)
    m, n = q.numel(), x.numel()
    if m == 0 or n == 0:
        raise ValueError("data and queries must be non-empty.")
    flags = (L.FSK_LAPLACE if laplace else 0) | (L.FSK_ATOMIC if atomic else 0)
    if log_eps is not None:
        flags |= L.FSK_OUT_LOG
    lib = L.load()
    with torch.cuda.device(dev):
        out = torch.empty(m, dtype=torch.float32, device=dev)
        ws = _workspace(lib.fsk_kde1d_workspace_bytes(m, n, flags), dev)
        st = lib.fsk_kde1d(q.data_ptr(), m, x.data_ptr(), n, h, flags, float(out_scale), float(log_eps or 0.0),
                           out.data_ptr(), ws.data_ptr(), ws.numel(), _stream(dev))
    L.check(st, "fsk_kde1d")
    return out


def kde1d_score(queries: torch.Tensor, data: torch.Tensor, bandwidth: float):
    """(score, pdf, deriv) of the 1-D Gaussian KDE at the queries."""
    h = _check_bw(bandwidth)
    dev = _device(queries.device)
    q = as_vector(queries, dev)
    x = as_vector(data, dev)
    m, n = q.numel(), x.numel()
    if m == 0 or n == 0:
        raise ValueError("data and queries must be non-empty.")
    lib = L.load()
    with torch.cuda.device(dev):
        score = torch.empty(m, dtype=torch.float32, device=dev)
        pdf = torch.empty_like(score)
        deriv = torch.empty_like(score)
        ws = _workspace(lib.fsk_kde1d_workspace_bytes(m, n, 0), dev)
        st = lib.fsk_kde1d_score(q.data_ptr(), m, x.data_ptr(), n, h, score.data_ptr(), pdf.data_ptr(),
                                 deriv.data_ptr(), ws.data_ptr(), ws.numel(), _stream(dev))
    L.check(st, "fsk_kde1d_score")
    return score, pdf, deriv


def silverman(data: torch.Tensor, *, rule: str = "silverman") -> torch.Tensor:
    """Bandwidth as a 0-d FP64 CUDA tensor (rule 'silverman' or 'sdkde_1d')."""
    dev = _device(data.device)
    x = data.to(device=dev, dtype=torch.float32, copy=False)
    if x.ndim == 1:
        x = x[:, None]
    if x.ndim != 2:
        raise ValueError("data must be 1D or 2D.")
    x = x.contiguous()
    n, d = x.shape
    if n == 0:
        raise ValueError("data must contain at least one element.")
    r = L.FSK_RULE_SDKDE_1D if rule == "sdkde_1d" else L.FSK_RULE_SILVERMAN
    lib = L.load()
    with torch.cuda.device(dev):
        h = torch.empty((), dtype=torch.float64, device=dev)
        ws = _workspace(lib.fsk_silverman_workspace_bytes(n, d), dev)
        st = lib.fsk_silverman(x.data_ptr(), n, d, r, h.data_ptr(), ws.data_ptr(), ws.numel(), _stream(dev))
    L.check(st, "fsk_silverman")
    return h


def device_status(device=None) -> None:
    """Synchronise and raise if a bounded in-kernel wait recorded a timeout."""
    dev = _device(device if device is not None else "cuda")
    with torch.cuda.device(dev):
        st = L.load().fsk_device_status(_stream(dev))
    L.check(st, "device status")


def mma_probe(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """tcgen05.mma of fp16(a) (128,32) by fp16(b) (64,32)^T -> (128,64) FP32."""
    dev = _device(a.device)
    a = a.to(device=dev, dtype=torch.float32).contiguous()
    b = b.to(device=dev, dtype=torch.float32).contiguous()
    if a.shape != (128, 32) or b.shape != (64, 32):
        raise ValueError("probe operands must be (128, 32) and (64, 32)")
    with torch.cuda.device(dev):
        d = torch.empty((128, 64), dtype=torch.float32, device=dev)
        st = L.load().fsk_diag_mma_probe(a.data_ptr(), b.data_ptr(), d.data_ptr(), _stream(dev))
    L.check(st, "fsk_diag_mma_probe")
    return d


def mma_ts_probe(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """tcgen05.mma with fp16(a) (128,64) read from tensor memory, by fp16(b) (16,64)^T -> (128,16)."""
    dev = _device(a.device)
    a = a.to(device=dev, dtype=torch.float32).contiguous()
    b = b.to(device=dev, dtype=torch.float32).contiguous()
    if a.shape != (128, 64) or b.shape != (16, 64):
        raise ValueError("probe operands must be (128, 64) and (16, 64)")
    with torch.cuda.device(dev):
        d = torch.empty((128, 16), dtype=torch.float32, device=dev)
        st = L.load().fsk_diag_mma_ts_probe(a.data_ptr(), b.data_ptr(), d.data_ptr(), _stream(dev))
    L.check(st, "fsk_diag_mma_ts_probe")
    return d


def tmem_cp_probe(a: torch.Tensor) -> torch.Tensor:
    """fp16(a) (128,32) in the operand image layout, tcgen05.cp to tensor memory,
    read back: (128,16) int32 words of packed fp16 pairs."""
    dev = _device(a.device)
    a = a.to(device=dev, dtype=torch.float32).contiguous()
    if a.shape != (128, 32):
        raise ValueError("probe operand must be (128, 32)")
    with torch.cuda.device(dev):
        out = torch.empty((128, 16), dtype=torch.int32, device=dev)
        st = L.load().fsk_diag_tmem_cp_probe(a.data_ptr(), out.data_ptr(), _stream(dev))
    L.check(st, "fsk_diag_tmem_cp_probe")
    return out


# ---- learned surrogate (include/fsk.h, "learned surrogate") ----------------------
MLP_PARAMS = L.FSK_MLP_PARAMS


def _mlp_check(params: torch.Tensor, members: int) -> None:
    if params.dtype != torch.float32 or not params.is_contiguous() or params.numel() != members * MLP_PARAMS:
        raise ValueError(f"params must be a contiguous float32 tensor of {members} x {MLP_PARAMS} values")


def mlp_train_workspace(members: int, batch: int, device) -> torch.Tensor:
    return _workspace(L.load().fsk_mlp_train_workspace_bytes(members, batch), _device(device))


def mlp_fwd(params, members, x, in_mean, in_inv_std, ws, y=None) -> torch.Tensor:
    """Training forward; keeps the activations in `ws` for mlp_bwd. y: (members, batch)."""
    _mlp_check(params, members)
    dev = _device(params.device)
    batch = x.shape[0]
    if y is None:
        y = torch.empty((members, batch), dtype=torch.float32, device=dev)
    with torch.cuda.device(dev):
        st = L.load().fsk_mlp_fwd(params.data_ptr(), members, x.data_ptr(), batch, in_mean.data_ptr(),
                                  in_inv_std.data_ptr(), y.data_ptr(), ws.data_ptr(), ws.numel(), _stream(dev))
    L.check(st, "fsk_mlp_fwd")
    return y


def mlp_bwd(params, members, batch, dy, ws, grads=None) -> torch.Tensor:
    _mlp_check(params, members)
    dev = _device(params.device)
    if grads is None:
        grads = torch.empty_like(params)
    with torch.cuda.device(dev):
        st = L.load().fsk_mlp_bwd(params.data_ptr(), members, batch, dy.data_ptr(), grads.data_ptr(),
                                  ws.data_ptr(), ws.numel(), _stream(dev))
    L.check(st, "fsk_mlp_bwd")
    return grads


def mlp_mse(y, target, dy, loss=None) -> None:
    members, batch = y.shape
    dev = _device(y.device)
    with torch.cuda.device(dev):
        st = L.load().fsk_mlp_mse(y.data_ptr(), target.data_ptr(), batch, members, dy.data_ptr(),
                                  _ptr(loss), _stream(dev))
    L.check(st, "fsk_mlp_mse")


def mlp_adam(params, grads, m, v, step, lr, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.0) -> None:
    dev = _device(params.device)
    with torch.cuda.device(dev):
        st = L.load().fsk_mlp_adam(params.data_ptr(), grads.data_ptr(), m.data_ptr(), v.data_ptr(),
                                   params.numel(), float(lr), float(beta1), float(beta2), float(eps),
                                   float(weight_decay), int(step), _stream(dev))
    L.check(st, "fsk_mlp_adam")


def mlp_pack(params, members, in_mean, in_inv_std, out_scale=1.0, out_shift=0.0) -> torch.Tensor:
    _mlp_check(params, members)
    dev = _device(params.device)
    lib = L.load()
    packed = torch.empty(lib.fsk_mlp_packed_bytes(members), dtype=torch.uint8, device=dev)
    with torch.cuda.device(dev):
        st = lib.fsk_mlp_pack(params.data_ptr(), members, in_mean.data_ptr(), in_inv_std.data_ptr(),
                              float(out_scale), float(out_shift), packed.data_ptr(), _stream(dev))
    L.check(st, "fsk_mlp_pack")
    return packed


def mlp_infer(packed, members, x, y=None) -> torch.Tensor:
    """Tensor-core inference of every member: (members, batch)."""
    dev = _device(packed.device)
    batch = x.shape[0]
    if y is None:
        y = torch.empty((members, batch), dtype=torch.float32, device=dev)
    with torch.cuda.device(dev):
        st = L.load().fsk_mlp_infer(packed.data_ptr(), members, x.data_ptr(), batch, y.data_ptr(), _stream(dev))
    L.check(st, "fsk_mlp_infer")
    return y


def mlp_combine(y, x=None, in_mean=None, in_inv_std=None, base_a=0.0, base_b=0.0, spread_tol=float("inf"),
                r2_max=float("inf")):
    """(mean + base, spread, served mask) over the members of y (members, batch)."""
    members, batch = y.shape
    dev = _device(y.device)
    mean = torch.empty(batch, dtype=torch.float32, device=dev)
    spread = torch.empty(batch, dtype=torch.float32, device=dev)
    served = torch.empty(batch, dtype=torch.uint8, device=dev)
    with torch.cuda.device(dev):
        st = L.load().fsk_mlp_combine(y.data_ptr(), members, batch, _ptr(x), _ptr(in_mean), _ptr(in_inv_std),
                                      float(base_a), float(base_b), float(spread_tol), float(r2_max),
                                      mean.data_ptr(), spread.data_ptr(), served.data_ptr(), _stream(dev))
    L.check(st, "fsk_mlp_combine")
    return mean, spread, served
