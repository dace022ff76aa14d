"""Derives the polynomial coefficients of include/pt_mathf.h.

Each kernel of pt_mathf is a minimax polynomial on a reduced interval,
fitted here by Lawson's iteratively re-weighted least squares (the weights
converge to the Chebyshev equioscillation of the minimax error) on a dense
Chebyshev grid, in float64, relative error weighted, then rounded to float32.
Run it to print the coefficient block of the header:

    python pathtracer_gb300/csrc/kernel/gen_pt_mathf.py
"""
from __future__ import annotations

import math

import numpy as np


def lawson_fit(target, lo, hi, degree, weight=None, basis=None, iters=400, npts=4000):
    """Minimax-weighted fit: minimise max |w(z) * (sum_k c_k b_k(z) - target(z))|."""
    k = np.arange(npts)
    z = 0.5 * (lo + hi) + 0.5 * (hi - lo) * np.cos(np.pi * (k + 0.5) / npts)
    t = target(z)
    w = np.ones_like(z) if weight is None else weight(z)
    B = np.stack([(z**j if basis is None else basis(z, j)) for j in range(degree + 1)], axis=1)
    lw = np.ones_like(z) / npts
    c = None
    for _ in range(iters):
        sw = np.sqrt(lw)
        c, *_ = np.linalg.lstsq(B * (w * sw)[:, None], t * w * sw, rcond=None)
        err = np.abs((B @ c - t) * w)
        lw = lw * err
        s = lw.sum()
        if s == 0:
            break
        lw /= s
    err = np.abs((B @ c - t) * w)
    return c, float(err.max())


def f32(x):
    return float(np.float32(x))


def main():
    out = {}
    # sin(r) = r + r^3 * P(r^2), r in [0, pi/4]; fit P(z) = (sin(sqrt z) - sqrt z) / z^1.5.
    zmax = (math.pi / 4) ** 2
    zs = lambda z: np.sqrt(np.maximum(z, 1e-300))
    P, e = lawson_fit(lambda z: (np.sin(zs(z)) - zs(z)) / (zs(z) ** 3), 1e-12, zmax, 3,
                      weight=lambda z: zs(z) ** 3 / np.sin(zs(z)))
    out["SIN"] = (P, e)
    # cos(r) = 1 - z/2 + z^2 * Q(z), z = r^2.
    Q, e = lawson_fit(lambda z: (np.cos(zs(z)) - 1 + z / 2) / z**2, 1e-12, zmax, 3,
                      weight=lambda z: z**2 / np.cos(zs(z)))
    out["COS"] = (Q, e)
    # exp(r) = 1 + r + r^2 * E(r), r in [-ln2/2, ln2/2].
    h = math.log(2) / 2
    E, e = lawson_fit(lambda r: np.where(np.abs(r) < 1e-8, 0.5 + r / 6, (np.expm1(r) - r) / np.where(r == 0, 1, r * r)),
                      -h, h, 5, weight=lambda r: r * r / np.exp(r))
    out["EXP"] = (E, e)
    # log(1+f) = 2s + s*z*R(z), s = f/(2+f), z = s^2, |s| <= (sqrt2-1)/(sqrt2+1).
    smax = (math.sqrt(2) - 1) / (math.sqrt(2) + 1)
    R, e = lawson_fit(lambda z: (2 * np.arctanh(zs(z)) - 2 * zs(z)) / (zs(z) ** 3), 1e-12, smax * smax, 3,
                      weight=lambda z: zs(z) ** 3 / (2 * np.arctanh(zs(z))))
    out["LOG"] = (R, e)
    # asin(x) = x + x^3 * A(x^2), x in [0, 1/2].
    A, e = lawson_fit(lambda z: (np.arcsin(zs(z)) - zs(z)) / (zs(z) ** 3), 1e-12, 0.25, 6,
                      weight=lambda z: zs(z) ** 3 / np.arcsin(zs(z)))
    out["ASIN"] = (A, e)
    # atan(r) = r + r^3 * T(r^2), r in [0, 1].
    T, e = lawson_fit(lambda z: (np.arctan(zs(z)) - zs(z)) / (zs(z) ** 3), 1e-12, 1.0, 8,
                      weight=lambda z: zs(z) ** 3 / np.arctan(zs(z)))
    out["ATAN"] = (T, e)
    for name, (c, err) in out.items():
        vals = ", ".join(f"{f32(v):.9e}f" for v in c)
        print(f"/* {name}: max weighted error {err:.2e} */")
        print(f"#define PTM_{name}_COEFFS {vals}")


if __name__ == "__main__":
    main()
