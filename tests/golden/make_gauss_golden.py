"""Exact Gauss-Legendre nodes and weights (40-digit mpmath, rounded to FP64)
for J = 64, 96, 160 -> gauss_legendre.npz.  The reference takes them from
scipy.special.roots_legendre (spectral_transform.py:80-114), whose weights
carry ~1e-12..3e-11 relative error near the poles; these values pin the GPU
geometry kernel to the exact quadrature instead.

Usage: python tests/golden/make_gauss_golden.py   (needs mpmath)
"""
from pathlib import Path

import mpmath as mp
import numpy as np


def nodes_weights(J: int):
    mp.mp.dps = 40
    xs, ws = [], []
    for k in range(J):
        x = -mp.cos(mp.pi * (k + mp.mpf(3) / 4) / (J + mp.mpf(1) / 2))
        for _ in range(60):
            p = mp.legendre(J, x)
            dp = J * (x * p - mp.legendre(J - 1, x)) / (x * x - 1)
            x = x - p / dp
        dp = J * (x * mp.legendre(J, x) - mp.legendre(J - 1, x)) / (x * x - 1)
        xs.append(float(x))
        ws.append(float(2 / ((1 - x * x) * dp * dp)))
    return np.array(xs), np.array(ws)


if __name__ == "__main__":
    out = {}
    for J in (64, 96, 160):
        x, w = nodes_weights(J)
        out[f"mu{J}"] = x
        out[f"w{J}"] = w
    np.savez_compressed(Path(__file__).resolve().parent / "gauss_legendre.npz", **out)
