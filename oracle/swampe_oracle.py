"""CPU FP64 oracle for the SWAMPE-JAX time-stepping core.

TEST INFRASTRUCTURE ONLY.  This module is the oracle: it may be imported by
``tests/``, by ``__graft_entry__.smoke()`` and by the CPU-baseline leg of
``bench.py``.  The GPU product path never imports it.

It restates, in plain array code, the algorithm of the reference package
``my_swampe`` (imalsky/MY_SWAMPE, v0.1.35).  Every function cites the
reference file:line it follows (paths relative to the reference project
root).  The restatement keeps the reference's operation order (one einsum per
reference einsum, the same FFT scaling, the same quirks) so that it can be
pinned against the reference's own golden fixtures
(``unit_tests/fixtures/reference_case_*.npz``) at the reference tolerances.

Array backend: numpy float64/complex128 by default.  Passing ``xp=TORCH``
runs the identical code on torch CPU float64 tensors, which makes the oracle
differentiable with ``torch.autograd`` (used as the gradient oracle for the
hand-written adjoint).  All fields may carry leading ensemble axes
(``(..., J, I)`` physical, ``(..., J, M+1)`` Fourier); per-member scalars are
then arrays of shape ``(..., 1, 1)``.
"""

from __future__ import annotations

import math
from dataclasses import dataclass
from functools import lru_cache
from typing import Any, Dict

import numpy as np


# --------------------------------------------------------------------------
# array backends
# --------------------------------------------------------------------------
class _NumpyBackend:
    name = "numpy"
    fdtype = np.float64
    cdtype = np.complex128

    def asarray(self, x, complex_=False):
        return np.asarray(x, dtype=self.cdtype if complex_ else self.fdtype)

    def fft(self, x, n, axis):
        return np.fft.fft(x, n=n, axis=axis)

    def ifft(self, x, n, axis):
        return np.fft.ifft(x, n=n, axis=axis)

    def einsum(self, s, *ops):
        return np.einsum(s, *ops, optimize=True)

    def stack(self, xs, axis=0):
        return np.stack(xs, axis=axis)

    def cat(self, xs, axis):
        return np.concatenate(xs, axis=axis)

    def zeros(self, shape, complex_=False):
        return np.zeros(shape, dtype=self.cdtype if complex_ else self.fdtype)

    def where(self, c, a, b):
        return np.where(c, a, b)

    def sqrt(self, x):
        return np.sqrt(x)

    def exp(self, x):
        return np.exp(x)

    def clamp0(self, x):
        return np.maximum(x, 0.0)

    def abs(self, x):
        return np.abs(x)

    def real(self, x):
        return np.real(x)

    def conj(self, x):
        return np.conj(x)

    def flip_last(self, x):
        return x[..., ::-1]

    def minimum_all(self, x):
        return np.min(x, axis=(-2, -1))

    def maximum_all(self, x):
        return np.max(x, axis=(-2, -1))

    def sum_all(self, x):
        return np.sum(x, axis=(-2, -1))

    def to_numpy(self, x):
        return np.asarray(x)


class _TorchBackend(_NumpyBackend):
    name = "torch"

    def __init__(self):
        import torch

        self.t = torch
        self.fdtype = torch.float64
        self.cdtype = torch.complex128

    def asarray(self, x, complex_=False):
        t = self.t
        dt = self.cdtype if complex_ else self.fdtype
        if isinstance(x, t.Tensor):
            return x.to(dt)
        return t.as_tensor(np.asarray(x), dtype=dt)

    def fft(self, x, n, axis):
        return self.t.fft.fft(x, n=n, dim=axis)

    def ifft(self, x, n, axis):
        return self.t.fft.ifft(x, n=n, dim=axis)

    def einsum(self, s, *ops):
        cplx = any(o.is_complex() for o in ops)
        dt = self.cdtype if cplx else self.fdtype
        return self.t.einsum(s, *[o.to(dt) for o in ops])

    def stack(self, xs, axis=0):
        return self.t.stack(xs, dim=axis)

    def cat(self, xs, axis):
        return self.t.cat(xs, dim=axis)

    def zeros(self, shape, complex_=False):
        return self.t.zeros(shape, dtype=self.cdtype if complex_ else self.fdtype)

    def where(self, c, a, b):
        t = self.t
        a = a if isinstance(a, t.Tensor) else t.as_tensor(a, dtype=self.fdtype)
        b = b if isinstance(b, t.Tensor) else t.as_tensor(b, dtype=self.fdtype)
        return t.where(c, a, b)

    def sqrt(self, x):
        return self.t.sqrt(x) if isinstance(x, self.t.Tensor) else math.sqrt(x)

    def exp(self, x):
        return self.t.exp(x)

    def clamp0(self, x):
        return self.t.clamp_min(x, 0.0)

    def abs(self, x):
        return self.t.abs(x)

    def real(self, x):
        return self.t.real(x)

    def conj(self, x):
        return self.t.conj(x)

    def flip_last(self, x):
        return self.t.flip(x, dims=(-1,))

    def minimum_all(self, x):
        return self.t.amin(x, dim=(-2, -1))

    def maximum_all(self, x):
        return self.t.amax(x, dim=(-2, -1))

    def sum_all(self, x):
        return self.t.sum(x, dim=(-2, -1))

    def to_numpy(self, x):
        return x.detach().numpy()


NUMPY = _NumpyBackend()
_TORCH = None


def torch_backend():
    """Return the torch-CPU-float64 backend (created lazily)."""
    global _TORCH
    if _TORCH is None:
        _TORCH = _TorchBackend()
    return _TORCH


# --------------------------------------------------------------------------
# static geometry  (spectral_transform.py, initial_conditions.py)
# --------------------------------------------------------------------------
def spectral_params(M: int):
    """Resolution table.  Follows ``initial_conditions.py:50-85``."""
    M = int(M)
    table = {42: (64, 128, 1200), 63: (96, 192, 900), 106: (160, 320, 600)}
    if M not in table:
        raise ValueError(f"Unsupported value of M={M}. Only 42, 63, and 106 are supported.")
    J, I, dt = table[M]
    return M, I, J, dt


def build_lambdas(I: int) -> np.ndarray:
    """Uniform longitudes in [-pi, pi).  ``spectral_transform.py:54-77``."""
    return np.linspace(-np.pi, np.pi, num=int(I), endpoint=False)


# Quadrature override: J -> (mus, w).  Empty means SciPy's roots_legendre, as
# the reference.  The GPU path builds its nodes and weights by Newton's method
# to ~1e-15 (SciPy's weights err by up to ~3e-11 near the poles), so the
# parity tests of the GPU path load the same exact values here: both sides
# then see identical quadrature and differ only by FP64 round-off.
_QUADRATURE: Dict[int, Any] = {}


def set_quadrature(table=None) -> None:
    """Use ``table[J] = (mus, w)`` as the Gauss-Legendre nodes and weights
    (``None`` restores SciPy's ``roots_legendre``).  Clears the geometry cache."""
    _QUADRATURE.clear()
    if table:
        for J, (mus, w) in table.items():
            _QUADRATURE[int(J)] = (np.asarray(mus, np.float64).copy(), np.asarray(w, np.float64).copy())
    cached_geometry.cache_clear()


def gauss_legendre(J: int):
    """Gauss-Legendre nodes/weights.  ``spectral_transform.py:80-114``."""
    import scipy.special as sp

    if int(J) in _QUADRATURE:
        mus, w = _QUADRATURE[int(J)]
        return mus.copy(), w.copy()
    mus, w = sp.roots_legendre(int(J))
    return np.asarray(mus, np.float64), np.asarray(w, np.float64)


def _scaling_table(M: int, N: int) -> np.ndarray:
    """Factorial normalisation.  ``spectral_transform.py:117-146``."""
    scale = np.zeros((M + 1, N + 1))
    for m in range(M + 1):
        for n in range(m, N + 1):
            scale[m, n] = math.sqrt(((2 * n) + 1) * math.factorial(n - m) / (2 * math.factorial(n + m)))
    return scale


def _lpmn_recurrence(M: int, N: int, x: float):
    """Unnormalised P_n^m(x) with Condon-Shortley phase and dP/dx.

    Same recurrences as ``spectral_transform.py:149-216``; used only when
    SciPy lacks ``assoc_legendre_p_all``.
    """
    P = np.zeros((M + 1, N + 1))
    dP = np.zeros((M + 1, N + 1))
    P[0, 0] = 1.0
    s = math.sqrt(max(0.0, 1.0 - x * x))
    for m in range(1, M + 1):
        if m <= N:
            P[m, m] = -(2 * m - 1) * s * P[m - 1, m - 1]
    for m in range(0, min(M, N - 1) + 1):
        P[m, m + 1] = (2 * m + 1) * x * P[m, m]
    for m in range(M + 1):
        for n in range(m + 2, N + 1):
            P[m, n] = ((2 * n - 1) * x * P[m, n - 1] - (n + m - 1) * P[m, n - 2]) / (n - m)
    denom = x * x - 1.0
    for m in range(M + 1):
        if 0 < m <= N:
            dP[m, m] = m * x * P[m, m] / denom
        for n in range(m + 1, N + 1):
            dP[m, n] = (n * x * P[m, n] - (n + m) * P[m, n - 1]) / denom
    return P, dP


def PmnHmn(J: int, M: int, N: int, mus: np.ndarray):
    """Normalised associated Legendre basis and H = (1-mu^2) dP/dmu.

    Follows ``spectral_transform.py:219-287``: SciPy ``assoc_legendre_p_all``
    (``:263-267``), H from the derivative (``:276``), factorial scaling
    (``:278-280``) and the odd-m sign flip (``:282-285``).
    """
    import scipy.special as sp

    Pt = np.zeros((J, M + 1, N + 1))
    Ht = np.zeros((J, M + 1, N + 1))
    have_all = hasattr(sp, "assoc_legendre_p_all")
    for j in range(J):
        mu = float(mus[j])
        if have_all:
            assoc = np.asarray(sp.assoc_legendre_p_all(N, M, mu, diff_n=1), dtype=np.float64)
            P_j = np.swapaxes(assoc[0, : N + 1, : M + 1], 0, 1)
            dP_j = np.swapaxes(assoc[1, : N + 1, : M + 1], 0, 1)
        else:  # pragma: no cover
            P_j, dP_j = _lpmn_recurrence(M, N, mu)
        Pt[j] = P_j
        Ht[j] = (1.0 - mu * mu) * dP_j
    scale = _scaling_table(M, N)
    Pmn = Pt * scale[None]
    Hmn = Ht * scale[None]
    odd = (np.arange(M + 1) % 2) == 1
    Pmn[:, odd, 1:] *= -1.0
    Hmn[:, odd, 1:] *= -1.0
    return Pmn, Hmn


@lru_cache(maxsize=None)
def cached_geometry(M: int):
    """Geometry cache.  ``model.py:62-86``."""
    M, I, J, _ = spectral_params(M)
    N = M
    lambdas = build_lambdas(I)
    mus, w = gauss_legendre(J)
    Pmn, Hmn = PmnHmn(J, M, N, mus)
    return dict(M=M, N=N, I=I, J=J, lambdas=lambdas, mus=mus, w=w, Pmn=Pmn, Hmn=Hmn)


# --------------------------------------------------------------------------
# transforms  (spectral_transform.py)
# --------------------------------------------------------------------------
def fwd_fft_trunc(xp, data, I, M):
    """``fft(data/I)[..., :M+1]``.  ``spectral_transform.py:309-328``."""
    return xp.fft(data / I, n=I, axis=-1)[..., : M + 1]


def invrs_fft(xp, approxXim, I):
    """``ifft(I * X)``.  ``spectral_transform.py:331-348``."""
    return xp.ifft(I * approxXim, n=I, axis=-1)


def fwd_leg_w(xp, data, Pmnw):
    """``einsum('...jm,jmn->...mn')``.  ``spectral_transform.py:370-402``."""
    return xp.einsum("...jm,jmn->...mn", data, Pmnw)


def invrs_leg(xp, legcoeff, I, M, Pmn):
    """Inverse Legendre with the negative-m layout.  ``spectral_transform.py:438-481``.

    The negative-m einsum (``:478``) is ``conj`` of the positive one because
    the basis is real; it fills the last M columns in reversed order.
    """
    pos = xp.einsum("jmn,...mn->...jm", Pmn, legcoeff)
    J = pos.shape[-2]
    lead = tuple(pos.shape[:-1])
    neg = xp.einsum("jmn,...mn->...jm", Pmn[:, 1:, :], xp.conj(legcoeff[..., 1:, :]))
    mid = xp.zeros(lead + (I - 2 * M - 1,), complex_=True)
    return xp.cat([pos, mid, xp.flip_last(neg)], axis=-1)


def invrsUV_with_coeffs(xp, deltamn, etamn, fmn, I, M, Pmn, Hmn, tstepcoeffmn, marray):
    """Wind inversion.  ``spectral_transform.py:535-596`` (and ``invrsUV:484-532``)."""
    Np1 = deltamn.shape[-1]
    keep = np.ones(Np1)
    keep[0] = 0.0
    keep = xp.asarray(keep)
    deltamn = deltamn * keep
    etamn = etamn * keep
    eta_minus_f = etamn - fmn
    delta_scaled = deltamn * tstepcoeffmn
    eta_scaled = eta_minus_f * tstepcoeffmn
    newUm1 = invrs_leg(xp, 1j * (marray * delta_scaled), I, M, Pmn)
    newUm2 = invrs_leg(xp, eta_scaled, I, M, Hmn)
    Um_full = -(newUm1 - newUm2)
    Unew = invrs_fft(xp, Um_full, I)
    newVm1 = invrs_leg(xp, 1j * (marray * eta_scaled), I, M, Pmn)
    newVm2 = invrs_leg(xp, delta_scaled, I, M, Hmn)
    Vm_full = -(newVm1 + newVm2)
    Vnew = invrs_fft(xp, Vm_full, I)
    return Unew, Vnew, Um_full[..., : M + 1], Vm_full[..., : M + 1]


# --------------------------------------------------------------------------
# forcing / filters / nonlinear products
# --------------------------------------------------------------------------
def Phieqfun(xp, Phibar, DPhieq, lambdas, mus):
    """Equilibrium geopotential, strict dayside mask.  ``forcing.py:14-62``."""
    lam = np.asarray(lambdas)[None, :]
    mu = np.asarray(mus)[:, None]
    day = xp.asarray(((lam > -np.pi / 2) & (lam < np.pi / 2)).astype(np.float64))
    term = xp.asarray(np.cos(lam) * np.sqrt(1 - mu**2))
    return Phibar + day * (DPhieq * term)


def Qfun(Phieq, Phi, Phibar, taurad):
    """``forcing.py:65-95``."""
    return (1 / taurad) * (Phieq - (Phi + Phibar))


def Rfun(xp, U, V, Q, Phi, Phibar, taudrag):
    """Velocity forcing: Q clamp, denominator guard, taudrag=-1 branch.  ``forcing.py:98-155``."""
    Qc = xp.where(Q < 0, 0.0, Q)
    pt = Phi + Phibar
    tiny = np.finfo(np.float64).tiny
    pts = xp.where(xp.abs(pt) > 0, pt, tiny)
    Ru = -U * Qc / pts
    Rv = -V * Qc / pts
    no_drag = _is_minus_one(taudrag)
    if isinstance(no_drag, bool):
        if no_drag:
            return Ru, Rv
        return Ru - U / taudrag, Rv - V / taudrag
    tde = xp.where(no_drag, 1.0, taudrag)
    F = xp.where(no_drag, Ru, Ru - U / tde)
    G = xp.where(no_drag, Rv, Rv - V / tde)
    return F, G


def _is_minus_one(x):
    if isinstance(x, (int, float)):
        return float(x) == -1.0
    return x == -1


def sigma6(xp, N, K6, a, dt):
    """``filters.py:95-123`` (row vector over n, broadcast over m)."""
    n = xp.asarray(np.arange(N + 1, dtype=np.float64))
    ncoeff = ((n * n * n) / a**3) * (((n + 1) * (n + 1) * (n + 1)) / a**3)
    return 1 / (1 + 2 * dt * K6 * (ncoeff - 8 / a**6))


def sigma6Phi(xp, N, K6, a, dt):
    """``filters.py:126-151``."""
    n = xp.asarray(np.arange(N + 1, dtype=np.float64))
    ncoeff = ((n * n * n) / a**3) * (((n + 1) * (n + 1) * (n + 1)) / a**3)
    return 1 / (1 + 2 * dt * K6 * ncoeff)


def sigma6_exponential(xp, N, K6, a, dt):
    """Integrating-factor hyperdiffusion of eta, delta for the semi-implicit
    scheme, clamped at zero below n = 1.  ``filters.py:154-185``."""
    n = xp.asarray(np.arange(N + 1, dtype=np.float64))
    ncoeff = ((n * n * n) / a**3) * (((n + 1) * (n + 1) * (n + 1)) / a**3)
    return xp.exp(-(2 * dt * K6) * xp.clamp0(ncoeff - 8 / a**6))


def sigma6Phi_exponential(xp, N, K6, a, dt):
    """Same without the ``8/a^6`` offset.  ``filters.py:188-213``."""
    n = xp.asarray(np.arange(N + 1, dtype=np.float64))
    ncoeff = ((n * n * n) / a**3) * (((n + 1) * (n + 1) * (n + 1)) / a**3)
    return xp.exp(-(2 * dt * K6) * ncoeff)


def ABCDE(xp, U, V, eta, Phi, mus):
    """``initial_conditions.py:242-292``."""
    mu = np.asarray(mus)[:, None]
    den = xp.asarray(2.0 * (1.0 - mu**2))
    return U * eta, V * eta, U * Phi, V * Phi, (U * U + V * V) / den


# --------------------------------------------------------------------------
# static build  (model.py:457-557, time_stepping.py:491-534)
# --------------------------------------------------------------------------
@dataclass
class Static:
    M: int
    N: int
    I: int
    J: int
    dt: Any
    a: Any
    omega: Any
    g: Any
    Phibar: Any
    taurad: Any
    taudrag: Any
    DPhieq: Any
    lambdas: np.ndarray
    mus: np.ndarray
    w: np.ndarray
    Pmn: Any
    Hmn: Any
    Pmnw: Any
    Hmnw: Any
    fmn: Any
    tstepcoeff: Any
    tstepcoeff2: Any
    tstepcoeffmn: Any
    marray: Any
    mJarray: Any
    narray: Any
    sigma: Any
    sigmaPhi: Any
    sigma_exp: Any
    sigmaPhi_exp: Any
    Phieq: Any


def build_static(xp, *, M, dt, a, omega, g, Phibar, taurad, taudrag, DPhieq, K6, K6Phi, test):
    """``model.py:457-557``.  Scalars may be per-member arrays (..., 1, 1)."""
    geo = cached_geometry(int(M))
    N, I, J = geo["N"], geo["I"], geo["J"]
    mus, w = geo["mus"], geo["w"]
    Pmn = xp.asarray(geo["Pmn"])
    Hmn = xp.asarray(geo["Hmn"])
    Pmnw = xp.asarray(w[:, None, None] * geo["Pmn"])
    Hmnw = xp.asarray(w[:, None, None] * geo["Hmn"])
    # coriolismn (initial_conditions.py:295-316): only (m=0, n=1) is non-zero.
    e01 = np.zeros((M + 1, N + 1))
    e01[0, 1] = 1.0
    fmn = xp.asarray(e01) * (omega / math.sqrt(0.375))
    n = np.arange(N + 1, dtype=np.float64)
    nn1 = n * (n + 1)
    tcmn_den = nn1.copy()
    tcmn_den[0] = 1.0
    tcmn_mask = np.ones(N + 1)
    tcmn_mask[0] = 0.0
    tstepcoeffmn = xp.asarray(tcmn_mask / tcmn_den) * a  # time_stepping.py:491-501
    mu = mus[:, None]
    tstepcoeff = (2.0 * dt) / (a * xp.asarray(np.broadcast_to(1.0 - mu**2, (J, M + 1)).copy()))  # :516-522
    tstepcoeff2 = xp.asarray(np.ones((J, M + 1))) * (2.0 * dt / (a**2))  # :504-506
    marray = xp.asarray(np.broadcast_to(np.arange(M + 1, dtype=np.float64)[:, None], (M + 1, N + 1)).copy())
    mJarray = xp.asarray(np.broadcast_to(np.arange(M + 1, dtype=np.float64)[None, :], (J, M + 1)).copy())
    narray = xp.asarray(np.broadcast_to(nn1[None, :], (M + 1, N + 1)).copy())
    K6Phi_eff = K6 if K6Phi is None else K6Phi
    sig = sigma6(xp, N, K6, a, dt)
    sigP = sigma6Phi(xp, N, K6Phi_eff, a, dt)
    sigX = sigma6_exponential(xp, N, K6, a, dt)          # model.py:517-518
    sigPX = sigma6Phi_exponential(xp, N, K6Phi_eff, a, dt)
    if test is None:
        Phieq = Phieqfun(xp, Phibar, DPhieq, geo["lambdas"], mus)
    else:
        Phieq = xp.zeros((J, I))
    return Static(
        M=M, N=N, I=I, J=J, dt=dt, a=a, omega=omega, g=g, Phibar=Phibar, taurad=taurad,
        taudrag=taudrag, DPhieq=DPhieq, lambdas=geo["lambdas"], mus=mus, w=w, Pmn=Pmn, Hmn=Hmn,
        Pmnw=Pmnw, Hmnw=Hmnw, fmn=fmn, tstepcoeff=tstepcoeff, tstepcoeff2=tstepcoeff2,
        tstepcoeffmn=tstepcoeffmn, marray=marray, mJarray=mJarray, narray=narray, sigma=sig,
        sigmaPhi=sigP, sigma_exp=sigX, sigmaPhi_exp=sigPX, Phieq=Phieq,
    )


def _is_array(x):
    return hasattr(x, "shape") and len(getattr(x, "shape")) > 0


# --------------------------------------------------------------------------
# tendencies  (modEuler_tdiff.py, explicit_tdiff.py)
# --------------------------------------------------------------------------
def modeuler_phi(xp, s: Static, X, forcflag, diffflag):
    """``modEuler_tdiff.py:30-117``."""
    t1 = s.tstepcoeff / 4.0
    t2 = s.tstepcoeff2 / 4.0
    Beff = X["Bm"] + X["Fm"] if forcflag else X["Bm"]
    Aeff = X["Am"] - X["Gm"] if forcflag else X["Am"]
    mJ = s.mJarray
    c1 = fwd_leg_w(xp, X["Phim1"], s.Pmnw)
    c2 = fwd_leg_w(xp, t1 * (1j) * mJ * X["Cm"], s.Pmnw)
    dleg = fwd_leg_w(xp, X["deltam1"], s.Pmnw)
    d2 = fwd_leg_w(xp, t1 * (1j) * mJ * Beff, s.Pmnw)
    d5 = fwd_leg_w(xp, t2 * X["Em"], s.Pmnw)
    c3 = fwd_leg_w(xp, t1 * X["Dm"], s.Hmnw)
    d3 = fwd_leg_w(xp, t1 * Aeff, s.Hmnw)
    c4 = s.dt * s.Phibar * dleg
    d5 = s.narray * d5
    out = c1 - c2 + c3 - c4 - s.Phibar * 0.5 * (d2 + d3 + d5 + (1.0 / (s.a**2)) * (s.narray * c1))
    if forcflag:
        out = out + fwd_leg_w(xp, s.dt * X["PhiFm"], s.Pmnw)
    if diffflag:
        out = out * s.sigmaPhi
    return out


def modeuler_delta(xp, s: Static, X, forcflag, diffflag):
    """``modEuler_tdiff.py:120-208`` (forced A,B terms always used: ``:166-168``)."""
    t1 = s.tstepcoeff / 4.0
    t2 = s.tstepcoeff2 / 4.0
    Bf = X["Bm"] + X["Fm"]
    Af = X["Am"] - X["Gm"]
    mJ = s.mJarray
    d1 = fwd_leg_w(xp, X["deltam1"], s.Pmnw)
    d2 = fwd_leg_w(xp, t1 * (1j) * mJ * Bf, s.Pmnw)
    d4 = fwd_leg_w(xp, t2 * X["Phim1"], s.Pmnw)
    d5 = fwd_leg_w(xp, t2 * X["Em"], s.Pmnw)
    p2 = fwd_leg_w(xp, t1 * (1j) * mJ * X["Cm"], s.Pmnw)
    d3 = fwd_leg_w(xp, t1 * Af, s.Hmnw)
    p3 = fwd_leg_w(xp, t1 * X["Dm"], s.Hmnw)
    nn = s.narray
    d4 = nn * d4
    d5 = nn * d5
    out = d1 + d2 + d3 + d4 + d5 + (nn * (p2 + p3)) / (2.0 * (s.a**2)) - s.Phibar * (nn * d1) / (s.a**2)
    if forcflag:
        out = out + (nn * fwd_leg_w(xp, (s.dt / 2.0) * X["PhiFm"], s.Pmnw)) / (s.a**2)
    if diffflag:
        out = out * s.sigma
    return out


def modeuler_eta(xp, s: Static, X, forcflag, diffflag):
    """``modEuler_tdiff.py:211-268`` (forced/unforced coefficient asymmetry ``:254``)."""
    t = s.tstepcoeff if forcflag else s.tstepcoeff / 2.0
    Aeff = X["Am"] - X["Gm"] if forcflag else X["Am"]
    Beff = X["Bm"] + X["Fm"] if forcflag else X["Bm"]
    e1 = fwd_leg_w(xp, X["etam1"], s.Pmnw)
    e2 = fwd_leg_w(xp, t * (1j) * s.mJarray * Aeff, s.Pmnw)
    e3 = fwd_leg_w(xp, t * Beff, s.Hmnw)
    out = e1 - e2 + e3
    if diffflag:
        out = out * s.sigma
    return out


def explicit_phi(xp, s: Static, X, forcflag, diffflag):
    """``explicit_tdiff.py:20-85``."""
    t1 = s.tstepcoeff
    c1 = fwd_leg_w(xp, X["Phim0"], s.Pmnw)
    c2 = fwd_leg_w(xp, t1 * (1j) * s.mJarray * X["Cm"], s.Pmnw)
    dleg = fwd_leg_w(xp, X["deltam1"], s.Pmnw)
    c3 = fwd_leg_w(xp, t1 * X["Dm"], s.Hmnw)
    out = c1 - c2 + c3 - 2.0 * s.dt * s.Phibar * dleg
    if forcflag:
        out = out + fwd_leg_w(xp, 2.0 * s.dt * X["PhiFm"], s.Pmnw)
    if diffflag:
        out = out * s.sigmaPhi
    return out


def explicit_delta(xp, s: Static, X, forcflag, diffflag):
    """``explicit_tdiff.py:88-162`` (carry-only quirk ``:134-138``, drag terms ``:145-153``)."""
    t1 = s.tstepcoeff
    out = fwd_leg_w(xp, X["deltam0"], s.Pmnw)
    if forcflag:
        f1 = fwd_leg_w(xp, (t1 * (1j) * s.mJarray * X["Um"]) / s.taudrag, s.Pmnw)
        f3 = fwd_leg_w(xp, t1 * (1j) * s.mJarray * X["Fm"], s.Pmnw)
        f2 = fwd_leg_w(xp, (t1 * X["Vm"]) / s.taudrag, s.Hmnw)
        f4 = fwd_leg_w(xp, t1 * X["Gm"], s.Hmnw)
        out = out + (-f1 + f2 + f3 - f4)
    if diffflag:
        out = out * s.sigma
    return out


def explicit_eta(xp, s: Static, X, forcflag, diffflag):
    """``explicit_tdiff.py:165-233``."""
    t1 = s.tstepcoeff
    e1 = fwd_leg_w(xp, X["etam0"], s.Pmnw)
    e2 = fwd_leg_w(xp, t1 * (1j) * s.mJarray * X["Am"], s.Pmnw)
    e3 = fwd_leg_w(xp, t1 * X["Bm"], s.Hmnw)
    out = e1 - e2 + e3
    if forcflag:
        f1 = fwd_leg_w(xp, (t1 * (1j) * s.mJarray * X["Vm"]) / s.taudrag, s.Pmnw)
        f3 = fwd_leg_w(xp, t1 * (1j) * s.mJarray * X["Gm"], s.Pmnw)
        f2 = fwd_leg_w(xp, (t1 * X["Um"]) / s.taudrag, s.Hmnw)
        f4 = fwd_leg_w(xp, t1 * X["Fm"], s.Hmnw)
        out = out + (-f1 + f2 + f3 + f4)
    if diffflag:
        out = out * s.sigma
    return out


def _inv_taudrag(xp, taudrag):
    """``1/taudrag`` with the ``taudrag == -1`` "no drag" sentinel mapped to 0
    (``model.py:775-792``, ``semi_implicit_tdiff.py`` relax branch)."""
    no_drag = _is_minus_one(taudrag)
    if isinstance(no_drag, bool):
        return 0.0 if no_drag else 1.0 / taudrag
    return xp.where(no_drag, 0.0, 1.0 / xp.where(no_drag, 1.0, taudrag))


def semi_implicit_step(xp, s: Static, X, forcflag, diffflag, relax, si_alpha, Rum_lag, Rvm_lag):
    """Semi-implicit leapfrog: gravity waves (and, when ``relax``, Newtonian
    relaxation and Rayleigh drag) weighted by ``si_alpha`` at the new level,
    the rest explicit, then the exponential hyperdiffusion.  Returns the new
    spectral (eta, delta, Phi).  ``semi_implicit_tdiff.py`` si_timestep
    (dispatch ``time_stepping.py:387-488``, ``model.py:871-918``).

    ``X["etam0"]`` etc. are the n-1 base: the Robert-Asselin-filtered Fourier
    lineage (``model.py:1089-1106``)."""
    two_dt = 2.0 * s.dt
    if relax:
        itd = _inv_taudrag(xp, s.taudrag)
        itr = 1.0 / s.taurad
        Fx, Gx = Rum_lag, Rvm_lag
        PhiFx = X["PhiFm"] + X["Phim1"] * itr
    else:
        itd = itr = 0.0
        Fx, Gx, PhiFx = X["Fm"], X["Gm"], X["PhiFm"]
    Aeff = X["Am"] - Gx if forcflag else X["Am"]
    Beff = X["Bm"] + Fx if forcflag else X["Bm"]
    tc, mJ = s.tstepcoeff, s.mJarray
    eta0 = fwd_leg_w(xp, X["etam0"], s.Pmnw)
    del0 = fwd_leg_w(xp, X["deltam0"], s.Pmnw)
    phi0 = fwd_leg_w(xp, X["Phim0"], s.Pmnw)
    iA = fwd_leg_w(xp, tc * (1j) * mJ * Aeff, s.Pmnw)
    iB = fwd_leg_w(xp, tc * (1j) * mJ * Beff, s.Pmnw)
    iC = fwd_leg_w(xp, tc * (1j) * mJ * X["Cm"], s.Pmnw)
    Emn = fwd_leg_w(xp, X["Em"], s.Pmnw)
    hA = fwd_leg_w(xp, tc * Aeff, s.Hmnw)
    hB = fwd_leg_w(xp, tc * Beff, s.Hmnw)
    hD = fwd_leg_w(xp, tc * X["Dm"], s.Hmnw)
    lam = s.narray / (s.a**2)  # -del^2 eigenvalue n(n+1)/a^2
    xi = two_dt * si_alpha
    ex = two_dt * (1.0 - si_alpha)
    kd, kr = xi * itd, xi * itr
    gd, gr = ex * itd, ex * itr
    eta_s = eta0 - iA + hB - gd * (eta0 - s.fmn)
    delta_s = del0 + iB + hA + two_dt * lam * Emn + ex * lam * phi0 - gd * del0
    phi_s = phi0 - iC + hD - ex * s.Phibar * del0 - gr * phi0
    if forcflag:
        phi_s = phi_s + fwd_leg_w(xp, two_dt * PhiFx, s.Pmnw)
    # the 2x2 (delta, Phi) system per degree, eliminated for delta
    eta_n = (eta_s + kd * s.fmn) / (1.0 + kd)
    bq, cq = xi * lam, xi * s.Phibar
    delta_n = (delta_s + bq * phi_s / (1.0 + kr)) / ((1.0 + kd) + bq * cq / (1.0 + kr))
    phi_n = (phi_s - cq * delta_n) / (1.0 + kr)
    if diffflag:
        eta_n, delta_n, phi_n = eta_n * s.sigma_exp, delta_n * s.sigma_exp, phi_n * s.sigmaPhi_exp
    return eta_n, delta_n, phi_n


# --------------------------------------------------------------------------
# state
# --------------------------------------------------------------------------
STATE_FIELDS = (
    "etam_prev", "etam_curr", "deltam_prev", "deltam_curr", "Phim_prev", "Phim_curr",
    "eta_prev", "eta_curr", "delta_prev", "delta_curr", "Phi_prev", "Phi_curr",
    "U_curr", "V_curr", "Um_curr", "Vm_curr",
    "Am_curr", "Bm_curr", "Cm_curr", "Dm_curr", "Em_curr",
    "PhiFm_curr", "Fm_curr", "Gm_curr", "Rum_lag", "Rvm_lag", "dead",
)


@dataclass
class Flags:
    """``model.py:156-226`` (booleans are static, scalars traced)."""

    forcflag: bool = True
    diffflag: bool = True
    expflag: bool = False
    modalflag: bool = True
    diagnostics: bool = True
    alpha: Any = 0.01
    blowup_rms: float = 8000.0
    semi_implicit: bool = False
    raw_filter: bool = False
    williams_alpha: Any = 0.53
    si_alpha: Any = 0.5


def forcing_phys(xp, s: Static, test, Phi, U, V):
    """Forcing computed whenever ``test is None`` (quirk).  ``model.py:560-603``."""
    if test is None:
        Q = Qfun(s.Phieq, Phi, s.Phibar, s.taurad)
        F, G = Rfun(xp, U, V, Q, Phi, s.Phibar, s.taudrag)
        return Q, F, G
    z = 0.0 * Phi
    return z, z, z


def nonlinear_spectral(xp, s: Static, eta, Phi, U, V):
    """``model.py:606-641``."""
    A, B, C, D, E = ABCDE(xp, U, V, eta, Phi, s.mus)
    return tuple(fwd_fft_trunc(xp, f, s.I, s.M) for f in (A, B, C, D, E))


def diagnose_winds(xp, s: Static, eta, delta):
    """``model.py:644-666``: FFT + fwd_leg (unweighted P times w) + invrsUV."""
    etam = fwd_fft_trunc(xp, eta, s.I, s.M)
    deltam = fwd_fft_trunc(xp, delta, s.I, s.M)
    etamn = fwd_leg_w(xp, etam, s.Pmnw)
    deltamn = fwd_leg_w(xp, deltam, s.Pmnw)
    Uc, Vc, _, _ = invrsUV_with_coeffs(xp, deltamn, etamn, s.fmn, s.I, s.M, s.Pmn, s.Hmn, s.tstepcoeffmn, s.marray)
    return xp.real(Uc), xp.real(Vc)


def analytic_ic(xp, s: Static, test, a1):
    """``model.py:669-691`` with ``initial_conditions.py:18-47,88-239``."""
    a, omega, Phibar = s.a, s.omega, s.Phibar
    SU0 = 2.0 * np.pi * a / (3600.0 * 24.0 * 12.0)
    sina, cosa = math.sin(a1), math.cos(a1)
    etaamp = 2.0 * ((SU0 / a) + omega)
    Phiamp = SU0 * a * omega + 0.5 * SU0**2
    mu = np.asarray(s.mus)[:, None]
    lam = np.asarray(s.lambdas)[None, :]
    sq = np.sqrt(1.0 - mu**2)
    J, I = s.J, s.I
    delta0 = np.zeros((J, I))
    Phi0 = np.zeros((J, I))
    if test == 1:
        arg = -np.cos(lam) * sq * sina + mu * cosa
        eta0 = etaamp * arg
        bumpr = a / 3.0
        dist_arg = 0.0 * mu + np.cos(np.arcsin(0.0)) * np.cos(np.arcsin(mu)) * np.cos(lam - 3.0 * np.pi / 2.0)
        dist = a * np.arccos(np.clip(dist_arg, -1.0, 1.0))
        bump = (Phibar / 2.0) * (1.0 + np.cos(np.pi * dist / bumpr))
        Phi0 = np.where(dist < bumpr, bump, 0.0)
        U0 = SU0 * (sq * cosa + mu * np.cos(lam) * sina) * sq
        V0 = -SU0 * np.sin(lam) * sina * sq
    elif test == 2:
        arg = -np.cos(lam) * sq * sina + mu * cosa
        eta0 = etaamp * arg
        Phi0 = (Phibar - Phiamp) * (arg**2)
        U0 = SU0 * (sq * cosa + np.cos(lam) * mu * sina)
        V0 = np.broadcast_to(-SU0 * (np.sin(lam) * sina), (J, I)).copy()
    else:
        eta0 = etaamp * np.broadcast_to(mu, (J, I)).copy()
        U0 = np.zeros((J, I))
        V0 = np.zeros((J, I))
    return tuple(xp.asarray(f) for f in (eta0, delta0, Phi0, U0, V0))


def init_state(xp, s: Static, test, eta0, delta0, Phi0, U0, V0):
    """Two-level start, prev == curr.  ``model.py:694-772``."""
    PhiF0, F0, G0 = forcing_phys(xp, s, test, Phi0, U0, V0)
    etam0, deltam0, Phim0, Um0, Vm0 = (fwd_fft_trunc(xp, f, s.I, s.M) for f in (eta0, delta0, Phi0, U0, V0))
    PhiFm0, Fm0, Gm0 = (fwd_fft_trunc(xp, f, s.I, s.M) for f in (PhiF0, F0, G0))
    Am0, Bm0, Cm0, Dm0, Em0 = nonlinear_spectral(xp, s, eta0, Phi0, U0, V0)
    # _momentum_forcing_remainder (model.py:775-792)
    inv_td = _inv_taudrag(xp, s.taudrag)
    Rum0 = Fm0 + Um0 * inv_td
    Rvm0 = Gm0 + Vm0 * inv_td
    return dict(
        etam_prev=etam0, etam_curr=etam0, deltam_prev=deltam0, deltam_curr=deltam0,
        Phim_prev=Phim0, Phim_curr=Phim0, eta_prev=eta0, eta_curr=eta0, delta_prev=delta0,
        delta_curr=delta0, Phi_prev=Phi0, Phi_curr=Phi0, U_curr=U0, V_curr=V0, Um_curr=Um0,
        Vm_curr=Vm0, Am_curr=Am0, Bm_curr=Bm0, Cm_curr=Cm0, Dm_curr=Dm0, Em_curr=Em0,
        PhiFm_curr=PhiFm0, Fm_curr=Fm0, Gm_curr=Gm0, Rum_lag=Rum0, Rvm_lag=Rvm0,
        dead=np.zeros(np.shape(eta0)[:-2], dtype=bool),
    )


def rms_winds(xp, s: Static, U, V):
    """Area-weighted RMS wind.  ``time_stepping.py:537-576``."""
    phis = np.arcsin(np.asarray(s.mus))[:, None]
    dlam = s.lambdas[2] - s.lambdas[1]
    dphi = phis[2, 0] - phis[1, 0]
    area = 4.0 * np.pi * s.a**2
    comp = (s.a**2) * (np.sin(phis + np.pi / 2.0) ** 2) * dphi * dlam
    cphi = np.cos(phis)
    integ = (U / cphi) ** 2 + (V / cphi) ** 2
    return xp.sqrt(xp.sum_all(comp * integ / area))


def step_once(xp, state, t, s: Static, flags: Flags, test, Uic, Vic):
    """One step of the scan body.  ``model.py:795-1194``: modEuler, explicit or
    semi-implicit tendency; classic RA filter on the physical prev carry, or
    the RAW filter (``:1007-1087``) on both the physical and the Fourier
    lineage.  The Fourier prev carry is the unfiltered curr (``:1107-1110``)
    for classic RA without the semi-implicit scheme, the filtered Fourier
    lineage otherwise (``:1089-1106``)."""
    X = dict(
        etam0=state["etam_prev"], etam1=state["etam_curr"], deltam0=state["deltam_prev"],
        deltam1=state["deltam_curr"], Phim0=state["Phim_prev"], Phim1=state["Phim_curr"],
        Am=state["Am_curr"], Bm=state["Bm_curr"], Cm=state["Cm_curr"], Dm=state["Dm_curr"],
        Em=state["Em_curr"], Fm=state["Fm_curr"], Gm=state["Gm_curr"], Um=state["Um_curr"],
        Vm=state["Vm_curr"], PhiFm=state["PhiFm_curr"],
    )
    if flags.diagnostics:
        rms = rms_winds(xp, s, state["U_curr"], state["V_curr"])
        spin_min = xp.minimum_all(xp.sqrt(state["U_curr"] ** 2 + state["V_curr"] ** 2))
        dead_next = np.logical_or(state["dead"], xp.to_numpy(rms) > flags.blowup_rms)
    else:
        rms = spin_min = 0.0
        dead_next = state["dead"]

    if flags.semi_implicit:
        etamn, deltamn, Phimn = semi_implicit_step(
            xp, s, X, flags.forcflag, flags.diffflag, bool(flags.forcflag) and test is None, flags.si_alpha,
            state["Rum_lag"], state["Rvm_lag"])
    elif flags.expflag:
        Phimn = explicit_phi(xp, s, X, flags.forcflag, flags.diffflag)
        deltamn = explicit_delta(xp, s, X, flags.forcflag, flags.diffflag)
        etamn = explicit_eta(xp, s, X, flags.forcflag, flags.diffflag)
    else:
        Phimn = modeuler_phi(xp, s, X, flags.forcflag, flags.diffflag)
        deltamn = modeuler_delta(xp, s, X, flags.forcflag, flags.diffflag)
        etamn = modeuler_eta(xp, s, X, flags.forcflag, flags.diffflag)
    full = [invrs_leg(xp, c, s.I, s.M, s.Pmn) for c in (etamn, deltamn, Phimn)]
    neweta, newdelta, newPhi = (xp.real(invrs_fft(xp, f, s.I)) for f in full)
    newetam, newdeltam, newPhim = (f[..., : s.M + 1] for f in full)
    Uc, Vc, newUm, newVm = invrsUV_with_coeffs(
        xp, deltamn, etamn, s.fmn, s.I, s.M, s.Pmn, s.Hmn, s.tstepcoeffmn, s.marray
    )
    newU, newV = xp.real(Uc), xp.real(Vc)
    if test == 1:
        newU, newV = Uic, Vic
        newUm, newVm = state["Um_curr"], state["Vm_curr"]

    do_ra = bool(flags.modalflag) and int(t) > 2
    al = flags.alpha
    # filter weights: classic RA moves the mid level by al * d; RAW (Williams
    # 2009) moves it by al * w * d and the new level by -al * (1 - w) * d
    wa = flags.williams_alpha if flags.raw_filter else 1.0
    lev = (("eta", neweta, "etam", newetam), ("delta", newdelta, "deltam", newdeltam),
           ("Phi", newPhi, "Phim", newPhim))
    mids, news, mmids, mnews = [], [], [], []
    for name, nw, mname, mnw in lev:
        prev, curr = state[name + "_prev"], state[name + "_curr"]
        mprev, mcurr = state[mname + "_prev"], state[mname + "_curr"]
        if do_ra:
            d = prev - 2.0 * curr + nw
            dm = mprev - 2.0 * mcurr + mnw
            if flags.raw_filter:
                mids.append(curr + al * wa * d)
                news.append(nw - al * (1.0 - wa) * d)
                mmids.append(mcurr + al * wa * dm)
                mnews.append(mnw - al * (1.0 - wa) * dm)
            else:
                mids.append(curr + al * d)
                news.append(nw)
                mmids.append(mcurr + al * dm)
                mnews.append(mnw)
        else:
            mids.append(curr)
            news.append(nw)
            mmids.append(mcurr)
            mnews.append(mnw)
    eta_mid, delta_mid, Phi_mid = mids
    neweta, newdelta, newPhi = news
    newetam, newdeltam, newPhim = mnews
    if flags.semi_implicit or flags.raw_filter:
        etam_mid, deltam_mid, Phim_mid = mmids
    else:  # unfiltered Fourier prev carry of the classic path
        etam_mid, deltam_mid, Phim_mid = state["etam_curr"], state["deltam_curr"], state["Phim_curr"]

    PhiF2, F2, G2 = forcing_phys(xp, s, test, newPhi, newU, newV)
    PhiFm2, Fm2, Gm2 = (fwd_fft_trunc(xp, f, s.I, s.M) for f in (PhiF2, F2, G2))
    Am2, Bm2, Cm2, Dm2, Em2 = nonlinear_spectral(xp, s, neweta, newPhi, newU, newV)
    if flags.semi_implicit:  # lagged momentum-forcing remainder (model.py:1135-1143)
        itd = _inv_taudrag(xp, s.taudrag)
        Rum_n = state["Fm_curr"] + state["Um_curr"] * itd
        Rvm_n = state["Gm_curr"] + state["Vm_curr"] * itd
    else:
        Rum_n, Rvm_n = state["Rum_lag"], state["Rvm_lag"]

    new = dict(
        etam_prev=etam_mid, etam_curr=newetam, deltam_prev=deltam_mid,
        deltam_curr=newdeltam, Phim_prev=Phim_mid, Phim_curr=newPhim,
        eta_prev=eta_mid, eta_curr=neweta, delta_prev=delta_mid, delta_curr=newdelta,
        Phi_prev=Phi_mid, Phi_curr=newPhi, U_curr=newU, V_curr=newV, Um_curr=newUm, Vm_curr=newVm,
        Am_curr=Am2, Bm_curr=Bm2, Cm_curr=Cm2, Dm_curr=Dm2, Em_curr=Em2, PhiFm_curr=PhiFm2,
        Fm_curr=Fm2, Gm_curr=Gm2, Rum_lag=Rum_n, Rvm_lag=Rvm_n, dead=dead_next,
    )
    out = dict(
        eta=neweta, delta=newdelta, Phi=newPhi, U=newU, V=newV, rms=rms, spin_min=spin_min,
        phi_min=xp.minimum_all(Phi_mid) if flags.diagnostics else 0.0,
        phi_max=xp.maximum_all(Phi_mid) if flags.diagnostics else 0.0, dead=dead_next,
    )
    if flags.diagnostics and np.any(dead_next):
        # skip_update (model.py:847-864): dead members keep their state.
        if np.ndim(dead_next) == 0:
            out = dict(
                eta=state["eta_curr"], delta=state["delta_curr"], Phi=state["Phi_curr"],
                U=state["U_curr"], V=state["V_curr"], rms=rms, spin_min=spin_min,
                phi_min=xp.minimum_all(state["Phi_curr"]), phi_max=xp.maximum_all(state["Phi_curr"]),
                dead=dead_next,
            )
            st = dict(state)
            st["dead"] = dead_next
            return st, out
        raise NotImplementedError("per-member blow-up gating in the batched oracle")
    return new, out


def run_model_scan(xp=NUMPY, *, M, dt, tmax, Phibar, omega, a, test=None, g=9.8, forcflag=True,
                   taurad=86400.0, taudrag=86400.0, DPhieq=4.0e6, a1=0.05, diffflag=True,
                   modalflag=True, alpha=0.01, expflag=False, K6=1.24e33, K6Phi=None,
                   starttime=None, eta0_init=None, delta0_init=None, Phi0_init=None,
                   U0_init=None, V0_init=None, diagnostics=True, return_history=True,
                   record=None, semi_implicit=False, si_alpha=0.5, raw_filter=False,
                   williams_alpha=0.53) -> Dict[str, Any]:
    """Driver.  ``model.py:1345-1765`` (validation, IC selection, ``t_seq = arange(starttime, tmax)``).

    ``record`` optionally lists history fields to keep (default: all five
    physical fields).  Continuation from pickles is not part of the oracle.
    """
    if tmax < 2:
        raise ValueError("tmax must be >= 2 (SWAMPE uses a 2-level initialization).")
    if isinstance(dt, (int, float)) and float(dt) <= 0.0:
        raise ValueError("dt must be positive.")
    if semi_implicit and expflag:  # model.py:1531-1537
        raise ValueError("semi_implicit=True is incompatible with expflag=True (pick one scheme).")
    if raw_filter and expflag:
        raise ValueError("raw_filter=True is incompatible with expflag=True.")
    s = build_static(xp, M=M, dt=dt, a=a, omega=omega, g=g, Phibar=Phibar, taurad=taurad,
                     taudrag=taudrag, DPhieq=DPhieq, K6=K6, K6Phi=K6Phi, test=test)
    st0 = 2 if starttime is None else int(starttime)
    if st0 > tmax:
        raise ValueError(f"starttime={st0} must be <= tmax={tmax}.")
    flags = Flags(forcflag=forcflag, diffflag=diffflag, expflag=expflag, modalflag=modalflag,
                  diagnostics=diagnostics, alpha=alpha, semi_implicit=bool(semi_implicit),
                  raw_filter=bool(raw_filter), williams_alpha=williams_alpha, si_alpha=si_alpha)
    if eta0_init is not None or delta0_init is not None or Phi0_init is not None:
        if eta0_init is None or delta0_init is None or Phi0_init is None:
            raise ValueError("If providing explicit ICs, eta0_init, delta0_init, and Phi0_init must all be provided.")
        eta0, delta0, Phi0 = (xp.asarray(f) for f in (eta0_init, delta0_init, Phi0_init))
        if (U0_init is None) != (V0_init is None):
            raise ValueError("Provide both U0_init and V0_init, or neither.")
        if U0_init is not None:
            U0, V0 = xp.asarray(U0_init), xp.asarray(V0_init)
        else:
            U0, V0 = diagnose_winds(xp, s, eta0, delta0)
    else:
        eta0, delta0, Phi0, U0, V0 = analytic_ic(xp, s, test, a1)
    state = init_state(xp, s, test, eta0, delta0, Phi0, U0, V0)
    t_seq = np.arange(st0, tmax, dtype=np.int32)
    hist = {k: [] for k in (record or ("eta", "delta", "Phi", "U", "V"))}
    diag = {k: [] for k in ("rms", "spin_min", "phi_min", "phi_max", "dead")}
    for t in t_seq:
        state, out = step_once(xp, state, int(t), s, flags, test, U0, V0)
        if return_history:
            for k in hist:
                hist[k].append(out[k])
            for k in diag:
                diag[k].append(out[k])
    res = dict(static=s, t_seq=t_seq, last_state=state, starttime=st0)
    if return_history:
        outs = {k: (xp.stack(v, 0) if len(v) else None) for k, v in hist.items()}
        for k, v in diag.items():
            outs[k] = np.asarray([float(xp.to_numpy(x)) if not isinstance(x, float) else x for x in v])
        res["outs"] = outs
        dead = outs["dead"].astype(bool)
        res["dead_first_idx"] = int(np.argmax(dead)) if dead.any() else -1
    return res


def run_model_scan_final(xp=NUMPY, **kw):
    """``model.py:1844-1951``: same as run_model_scan without history, diagnostics off."""
    kw.setdefault("diagnostics", False)
    return run_model_scan(xp, return_history=False, **kw)


def legacy_diagnostics(xp, res, tmax: int, test, a1: float = 0.05, contflag: bool = False):
    """``run_model``'s ``(tmax, 2)`` spinup / geopot arrays.  ``model.py:2106-2158``:
    row t-1 of each step t in t_seq holds (min wind speed, RMS wind) and
    (min Phi, max Phi); without continuation row 0 comes from the analytic
    initial condition."""
    spin = np.zeros((int(tmax), 2))
    geop = np.zeros((int(tmax), 2))
    outs = res["outs"]
    for k, t in enumerate(res["t_seq"]):
        i = int(t) - 1
        if 0 <= i < tmax:
            spin[i] = (outs["spin_min"][k], outs["rms"][k])
            geop[i] = (outs["phi_min"][k], outs["phi_max"][k])
    if not contflag:
        s = res["static"]
        _, _, Phi0, U0, V0 = (xp.to_numpy(f) for f in analytic_ic(xp, s, test, a1))
        spin[0] = (np.min(np.sqrt(U0 * U0 + V0 * V0)), float(xp.to_numpy(rms_winds(xp, s, U0, V0))))
        geop[0] = (np.min(Phi0), np.max(Phi0))
    return spin, geop
