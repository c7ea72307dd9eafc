"""Fit of the Ewald screening function used by the FP32 pair kernels.

erfc(x) = R(t) exp(-x^2) with t = 1 / (1 + p x): R is a polynomial in t fitted
to the scaled complementary error function erfc(x) exp(x^2) on 0 <= x <= 4
(Chebyshev-spaced samples, least squares on the relative error, Lawson
reweighting towards the minimax fit), p scanned for the smallest maximum
relative error.  Prints p and the coefficients c0..cD (R = sum c_k t^k) that
erfc_scaled / erfc_scaled2 in sdm_kernels.cu hold, and the error in FP64 and
in FP32 Horner evaluation.

    python openmm_sdm_plugin_gb300/csrc/fit_erfc.py [degree]
"""
import sys

import numpy as np
from scipy.special import erfc, erfcx

XMAX = 4.0


def fit(deg, p, x, y, iters=60):
    t = 1.0 / (1.0 + p * x)
    V = np.vander(t, deg + 1, increasing=True)
    w = np.ones_like(x)
    for _ in range(iters):
        c, *_ = np.linalg.lstsq(V * (w / y)[:, None], w, rcond=None)
        r = (V @ c) / y - 1.0
        w = w * np.sqrt(np.abs(r)) + 1e-300
        w /= w.max()
    return c, np.abs(r).max()


def eval_f32(c, p, x):
    """Horner in FP32 (fused multiply-adds emulated by FP64 products rounded once)."""
    x = np.asarray(x, np.float32)
    t = (np.float32(1.0) / (np.float32(1.0) + np.float32(p) * x)).astype(np.float32)
    c = np.asarray(c, np.float32)
    acc = np.full_like(t, c[-1])
    for k in range(len(c) - 2, -1, -1):
        acc = (acc.astype(np.float64) * t + c[k]).astype(np.float32)
    g = np.exp(-(x.astype(np.float64) ** 2)).astype(np.float32)
    return (acc.astype(np.float64) * g).astype(np.float32)


def main(deg=7):
    x = np.cos(np.linspace(0.0, np.pi, 20001))[::-1] * XMAX / 2 + XMAX / 2
    y = erfcx(x)
    best = None
    for p in np.round(np.linspace(0.2, 0.8, 61), 2):
        c, err = fit(deg, p, x, y)
        if best is None or err < best[2]:
            best = (p, c, err)
    p, c, err = best
    xs = np.linspace(0.0, XMAX, 400001)
    rel32 = np.abs(eval_f32(c, p, xs) / erfc(xs.astype(np.float32).astype(np.float64)) - 1.0).max()
    print(f"degree {deg}  p {p}  max rel error: fit {err:.3g}, FP32 {rel32:.3g}")
    for k, ck in enumerate(c):
        print(f"c{k} = {float(np.float32(ck))!r}")


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 7)
