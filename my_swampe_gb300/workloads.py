"""Seeded synthetic ensembles with the shapes and value distributions of the
benchmark configurations (there is no public dataset for this model).

``forced_ensemble`` is the forced synchronously-rotating regime: a = 8.2e7 m,
Omega = 3.2e-5 1/s, Phibar = 4e6, dt = 30 s, start from rest (eta = 2 Omega
mu, delta = U = V = 0) with Phi = seeded Gaussian noise of amplitude
1e-3 * Phibar on the spectral coefficients with n <= 10 (m <= n, m = 0 real),
synthesised to the grid; per member taurad, taudrag ~ log-uniform[1e4, 1e6] s
and DPhieq ~ uniform[1e5, 4e6] m^2/s^2, drawn from ``seed + member``.
"""
from __future__ import annotations

from typing import Dict

import numpy as np
import torch

from .engine import Engine

_GRID = {42: (64, 128), 63: (96, 192), 106: (160, 320)}


def synth_from_spectral(eng: Engine, coeffs: torch.Tensor, g: int = 0) -> torch.Tensor:
    """Grid field(s) (..., J, I) from spectral coefficients (..., M+1, N+1):
    inverse Legendre with the FP64 GPU basis, then the Hermitian inverse FFT."""
    geo = eng.geometry(g)
    gd = eng.groups[g]
    P = geo["Pmn"].to(torch.complex128)
    pos = torch.einsum("jmn,...mn->...jm", P, coeffs.to(torch.complex128))
    I = gd["I"]
    spec = torch.zeros(pos.shape[:-1] + (I // 2 + 1,), dtype=torch.complex128, device=pos.device)
    spec[..., : gd["M"] + 1] = pos * I
    return torch.fft.irfft(spec, n=I, dim=-1)


def forced_ensemble(eng: Engine, g: int = 0, seed: int = 1234, Phibar: float = 4.0e6, a: float = 8.2e7,
                    omega: float = 3.2e-5, dt: float = 30.0, K6: float = 1.24e33, nmax: int = 10,
                    amp_frac: float = 1e-3) -> Dict:
    gd = eng.groups[g]
    M, B, J, I = gd["M"], gd["B"], gd["J"], gd["I"]
    dev = eng.device
    tr = np.empty(B)
    td = np.empty(B)
    dp = np.empty(B)
    c = np.zeros((B, M + 1, M + 1), dtype=np.complex128)
    for b in range(B):
        rng = np.random.default_rng(seed + b)
        tr[b] = 10.0 ** rng.uniform(4.0, 6.0)
        td[b] = 10.0 ** rng.uniform(4.0, 6.0)
        dp[b] = rng.uniform(1.0e5, 4.0e6)
        for m in range(nmax + 1):
            for n in range(m, nmax + 1):
                re = rng.standard_normal()
                im = rng.standard_normal() if m > 0 else 0.0
                c[b, m, n] = amp_frac * Phibar * (re + 1j * im)
    Phi0 = synth_from_spectral(eng, torch.as_tensor(c, device=dev), g)
    mus = eng.geometry(g)["mus"]
    eta0 = (2.0 * omega * mus)[None, :, None].expand(B, J, I)
    z = torch.zeros((B, J, I), dtype=torch.float64, device=dev)
    ics = torch.stack((eta0, z, Phi0, z, z), 0).contiguous()
    params = dict(dt=dt, a=a, omega=omega, Phibar=Phibar, K6=K6, K6Phi=K6, alpha=0.01,
                  taurad=torch.as_tensor(tr, device=dev), taudrag=torch.as_tensor(td, device=dev),
                  DPhieq=torch.as_tensor(dp, device=dev))
    return dict(params=params, ics=ics)


def apply_params(eng: Engine, g: int, params: Dict) -> None:
    eng.set_params(g, **{k: v for k, v in params.items()})
