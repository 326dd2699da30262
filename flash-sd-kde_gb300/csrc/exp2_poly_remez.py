"""Coefficients of the FMA-pipe exp2 used beside ex2.approx (fsk_common.cuh,
exp2_poly): a degree-5 polynomial p(r) ~ 2^r on r in [-1/2, 1/2] with minimal
maximum *relative* error, found by the Remez exchange algorithm (equioscillation
of the weighted error p(r)/2^r - 1 at degree + 2 points), in FP64.

    python exp2_poly_remez.py          # prints the coefficients and the error

The kernel splits x = j + r (j = round(x), via the add-1.5*2^23 trick), takes
p(r) in FP32 Horner form and adds j to p's exponent field with one integer
multiply-add.  Run only to regenerate the constants; nothing imports it.
"""
from __future__ import annotations

import numpy as np

DEG = 5
LO, HI = -0.5, 0.5


def remez(deg: int = DEG, iters: int = 30) -> tuple[np.ndarray, float]:
    f = lambda r: np.exp2(r)
    k = np.arange(deg + 2)
    x = 0.5 * (LO + HI) + 0.5 * (HI - LO) * np.cos(np.pi * (deg + 1 - k) / (deg + 1))  # Chebyshev extrema
    grid = np.linspace(LO, HI, 200001)
    for _ in range(iters):
        # p(x_i) - f(x_i) = (-1)^i E f(x_i): unknowns c_0..c_deg, E
        a = np.zeros((deg + 2, deg + 2))
        for i, xi in enumerate(x):
            a[i, :deg + 1] = xi ** np.arange(deg + 1)
            a[i, deg + 1] = -((-1) ** i) * f(xi)
        sol = np.linalg.solve(a, f(x))
        c = sol[:deg + 1]
        err = np.polyval(c[::-1], grid) / f(grid) - 1.0
        # new reference: one extremum of the error in each sign run
        sign = np.sign(err)
        idx, start = [], 0
        for i in range(1, grid.size + 1):
            if i == grid.size or sign[i] != sign[start]:
                seg = np.abs(err[start:i])
                idx.append(start + int(np.argmax(seg)))
                start = i
        if len(idx) < deg + 2:
            break
        # keep deg + 2 alternating extrema with the largest magnitudes
        while len(idx) > deg + 2:
            drop = 0 if abs(err[idx[0]]) < abs(err[idx[-1]]) else len(idx) - 1
            idx.pop(drop)
        x = grid[idx]
    err = np.polyval(c[::-1], grid) / f(grid) - 1.0
    return c, float(np.abs(err).max())


def fp32_check(c: np.ndarray) -> float:
    """Max relative error of the FP32 evaluation (Horner with FMA, exponent
    insertion) against FP64 2^x over x in [-126, 0]."""
    c32 = c.astype(np.float32)
    x = np.linspace(-126.0, 0.0, 2000001).astype(np.float32)
    t = (x + np.float32(12582912.0)).astype(np.float32)
    j = (t - np.float32(12582912.0)).astype(np.float32)
    r = (x - j).astype(np.float32)
    p = np.full_like(r, c32[DEG])
    for k in range(DEG - 1, -1, -1):   # FP32 fma: FP64 product-sum rounded once
        p = (p.astype(np.float64) * r.astype(np.float64) + np.float64(c32[k])).astype(np.float32)
    bits = p.view(np.int32).astype(np.int64) + (j.astype(np.int64) << 23)
    y = bits.astype(np.int32).view(np.float32).astype(np.float64)
    ref = np.exp2(x.astype(np.float64))
    ok = ref > 2.0 ** -126
    return float((np.abs(y[ok] - ref[ok]) / ref[ok]).max())


if __name__ == "__main__":
    c, e = remez()
    print("relative minimax error (FP64):", e)
    for k, v in enumerate(c.astype(np.float32)):
        print(f"  c{k} = {float(v):.9e}f  ({v.view(np.uint32):#010x})")
    print("FP32 evaluation, max relative error over [-126, 0]:", fp32_check(c))
