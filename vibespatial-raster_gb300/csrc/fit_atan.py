"""Fit the polynomial used by the kernels' degree-valued arctangent.

On t in [0, 1], atan(t) in DEGREES is approximated as t * P(t^2) with P of
degree N, fitted by Lawson's iteratively reweighted least squares (which
converges to the minimax fit) in float64 on Chebyshev-distributed nodes.  The
kernels reduce any (y, x) to t = min(|y|,|x|) / max(|y|,|x|) and unfold with
90 - a, 180 - a and the sign of y, so the axes map to exactly 0, 90 and 180.

Run ``python fit_atan.py`` to print the coefficients and the fit's maximum
absolute error (degrees); the values in horn.cu came from this script.
"""

from __future__ import annotations

import numpy as np

N = 8  # P has N + 1 coefficients


def fit(n: int = N, iters: int = 200):
    m = 4000
    u = 0.5 - 0.5 * np.cos(np.pi * (np.arange(m) + 0.5) / m)  # u = t^2 in [0, 1]
    t = np.sqrt(u)
    target = np.degrees(np.arctan(t))
    # a(t) = t * P(u); fit P via columns t * u^k, weighted for minimax of |a - target|
    A = np.stack([t * u**k for k in range(n + 1)], axis=1)
    w = np.ones(m)
    c = None
    for _ in range(iters):
        sw = np.sqrt(w)
        c, *_ = np.linalg.lstsq(A * sw[:, None], target * sw, rcond=None)
        err = np.abs(A @ c - target)
        w = w * err
        w = w / w.sum()
    tt = np.linspace(0, 1, 200001)
    e = np.abs(tt * np.polyval(c[::-1], tt * tt) - np.degrees(np.arctan(tt)))
    return c, float(e.max())


if __name__ == "__main__":
    c, e = fit()
    for k, v in enumerate(c):
        print(f"  {float(v):.17g}f,")
    print(f"max abs error {e:.3e} degrees")
