"""Derives the polynomial coefficients of the portable sine/cosine shared by
the CUDA kernels (kgmt_gb300/csrc/kgmt_device.cuh, sincos_portable) and the
CPU restatement (oracle/kgmt_oracle.c, ko_sincosf).

On the reduced argument |r| <= pi/4 the forms are

    sin r = r + r^3 (s1 + s2 r^2 + s3 r^4)
    cos r = 1 - r^2 / 2 + r^4 (c2 + c3 r^2 + c4 r^4)

and the coefficients minimise the largest relative error, found by Lawson's
algorithm (iteratively reweighted least squares: each pass reweights the
sample points by their current error, which converges to the minimax
solution) on Chebyshev-clustered points.  Printed: the fitted coefficients,
their float roundings as C hex literals, and the relative errors before
rounding (about 3.8e-9 for sin, 1.2e-10 for cos, both well under float's
6e-8).

    python oracle/fit_sincos.py
"""
from __future__ import annotations

import numpy as np


def lawson(basis: np.ndarray, target: np.ndarray, weight: np.ndarray, iters: int = 400):
    w = np.ones(len(target))
    for _ in range(iters):
        sw = np.sqrt(w)
        c, *_ = np.linalg.lstsq(basis * sw[:, None], target * sw, rcond=None)
        e = np.abs(basis @ c - target) * weight
        w = w * e
        w /= w.sum()
    return c, float(np.max(np.abs(basis @ c - target) * weight))


def main() -> None:
    half = np.pi / 8
    x = np.cos(np.linspace(0.0, np.pi, 20001)) * half + half  # Chebyshev points on [0, pi/4]
    x = x[x > 1e-6]
    basis = np.stack([np.ones_like(x), x ** 2, x ** 4], 1)
    # (sin r - r) / r^3, error weighted relative to sin r
    cs, es = lawson(basis, (np.sin(x) - x) / x ** 3, x ** 3 / np.sin(x))
    # (cos r - 1 + r^2/2) / r^4, error weighted relative to cos r
    cc, ec = lawson(basis, (np.cos(x) - 1.0 + x ** 2 / 2.0) / x ** 4, x ** 4 / np.cos(x))
    for name, coef, err in (("s", cs, es), ("c", cc, ec)):
        print(f"{name}: max relative error {err:.3g}")
        for k, v in enumerate(coef):
            print(f"  {name}{k + 1 if name == 's' else k + 2} = {float(np.float32(v)).hex()}  ({v:.9g})")


if __name__ == "__main__":
    main()
