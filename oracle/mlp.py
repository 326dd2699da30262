"""CPU restatement of the surrogate MLP -- TEST INFRASTRUCTURE ONLY.

The reference has no surrogate (it is a new component of this build), so
this oracle is pinned by a finite-difference gradient check (tests) rather
than by reference outputs: "parity unpinned" against the reference.

Model (one ensemble member), the semantics the CUDA kernels implement:
  x_n = (x - in_mean) * in_inv_std                (FP32)
  a0  = bf16(x_n)
  z1  = bf16(W1) a0 + b1,  a1 = bf16(silu(z1))    W1: (256, 16)
  z2  = bf16(W2) a1 + b2,  a2 = bf16(silu(z2))    W2: (256, 256)
  z3  = bf16(W3) a2 + b3,  a3 = bf16(silu(z3))    W3: (256, 256)
  y   = bf16(w4) . a3 + b4                          w4: (256,)
Parameters of a member, FP32, contiguous in this order:
  W1 (256*16) b1 (256) W2 (256*256) b2 (256) W3 (256*256) b3 (256) w4 (256) b4 (1)
Backward treats the bf16 roundings as identity (straight-through) and
differentiates everything else exactly.  Adam is Kingma & Ba with bias
correction and decoupled weight decay (AdamW).
"""
from __future__ import annotations

import numpy as np

IN = 16
H = 256
SIZES = [("W1", (H, IN)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, H)), ("b3", (H,)),
         ("w4", (H,)), ("b4", (1,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SIZES)   # 136193


def unpack(p: np.ndarray) -> dict:
    out, o = {}, 0
    for name, shape in SIZES:
        k = int(np.prod(shape))
        out[name] = p[o:o + k].reshape(shape)
        o += k
    return out


def bf16(a: np.ndarray) -> np.ndarray:
    """Round FP32 values to the nearest bf16 (ties to even), returned as FP32."""
    a32 = np.ascontiguousarray(a, dtype=np.float32)
    u = a32.view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return r.astype(np.uint32).view(np.float32).reshape(a32.shape)


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def init_params(rng: np.random.Generator) -> np.ndarray:
    """Test parameters: weights uniform in +-sqrt(6/fan_in) (w4: +-1/sqrt(256)),
    small random biases."""
    fan = {"W1": IN, "W2": H, "W3": H}
    parts = []
    for name, shape in SIZES:
        if name in fan:
            b = np.sqrt(6.0 / fan[name])
        elif name == "w4":
            b = 1.0 / np.sqrt(H)
        else:
            b = 0.1
        parts.append(rng.uniform(-b, b, size=shape).ravel())
    return np.concatenate(parts).astype(np.float32)


def forward(p: np.ndarray, x: np.ndarray, in_mean, in_inv_std, quantize: bool = True, dtype=np.float64):
    """Returns y (batch,) and the cache for backward.  quantize=False gives
    the unrounded model (used by the finite-difference check)."""
    q = bf16 if quantize else (lambda a: np.asarray(a, dtype=dtype))
    P = unpack(p)
    ft = np.float32 if quantize else dtype
    xn = (np.asarray(x, ft) - np.asarray(in_mean, ft)) * np.asarray(in_inv_std, ft)
    a0 = q(xn).astype(dtype)
    W1, W2, W3, w4 = (q(P[k]).astype(dtype) for k in ("W1", "W2", "W3", "w4"))
    b1, b2, b3, b4 = (P[k].astype(dtype) for k in ("b1", "b2", "b3", "b4"))
    z1 = a0 @ W1.T + b1
    a1 = q(silu(z1)).astype(dtype)
    z2 = a1 @ W2.T + b2
    a2 = q(silu(z2)).astype(dtype)
    z3 = a2 @ W3.T + b3
    a3 = q(silu(z3)).astype(dtype)
    y = a3 @ w4 + b4[0]
    cache = dict(a0=a0, z1=z1, a1=a1, z2=z2, a2=a2, z3=z3, a3=a3, W1=W1, W2=W2, W3=W3, w4=w4)
    return y, cache


def backward(cache: dict, dy: np.ndarray) -> np.ndarray:
    """Gradient of sum(dy * y) w.r.t. the parameters (straight-through for
    the bf16 roundings), flattened in parameter order."""
    dy = np.asarray(dy, dtype=cache["a3"].dtype)
    g = {}
    g["w4"] = cache["a3"].T @ dy
    g["b4"] = np.array([dy.sum()])
    da3 = np.outer(dy, cache["w4"])
    dz3 = da3 * silu_grad(cache["z3"])
    g["W3"] = dz3.T @ cache["a2"]
    g["b3"] = dz3.sum(0)
    da2 = dz3 @ cache["W3"]
    dz2 = da2 * silu_grad(cache["z2"])
    g["W2"] = dz2.T @ cache["a1"]
    g["b2"] = dz2.sum(0)
    da1 = dz2 @ cache["W2"]
    dz1 = da1 * silu_grad(cache["z1"])
    g["W1"] = dz1.T @ cache["a0"]
    g["b1"] = dz1.sum(0)
    return np.concatenate([g[name].ravel() for name, _ in SIZES])


def adam(p, grad, m, v, step: int, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8,
         weight_decay: float = 0.0):
    """One AdamW update (step counts from 1); returns new (p, m, v) in FP64."""
    p, grad, m, v = (np.asarray(a, np.float64) for a in (p, grad, m, v))
    m = beta1 * m + (1 - beta1) * grad
    v = beta2 * v + (1 - beta2) * grad * grad
    mh = m / (1 - beta1 ** step)
    vh = v / (1 - beta2 ** step)
    p = p - lr * (mh / (np.sqrt(vh) + eps) + weight_decay * p)
    return p, m, v
