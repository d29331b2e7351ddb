"""Drop-in replacement for the time-stepping core of ``my_swampe.model``.

Keeps the signatures of ``run_model_scan`` (reference ``model.py:1345-1765``),
``run_model_scan_final`` (``:1844-1951``), ``run_model`` (``:1954-2219``) and
``run_model_gpu`` (``:2222-2251``), the ``(eta, delta, Phi, U, V)`` history
layout ``(T, J, I)`` and the 27-field ``State`` (``:380-425``).  The scan body
runs in the CUDA kernels of ``libswampe_gb300``; arrays are torch tensors on
the GPU.

Two extensions: ``precision="fp64" | "fast"`` selects the FP64 kernels (the
parity path) or the FP32 / split-precision kernels, and every scalar
parameter may be a length-B sequence, which runs B ensemble members in one
launch (leading member axis on every output).
"""
from __future__ import annotations

import math
import warnings
from dataclasses import dataclass
from typing import Any, Dict, NamedTuple, Optional

import numpy as np
import torch
import torch.autograd.forward_ad as fwAD

from . import _lib, continuation
from .engine import Engine, RunFlagsC

_SUPPORTED_M = {42: (64, 128, 1200), 63: (96, 192, 900), 106: (160, 320, 600)}


def spectral_params(M: int):
    """(N, I, J, dt, lambdas, mus, w) -- ``initial_conditions.py:50-85``.

    mus and w come from the GPU Gauss-Legendre kernel (FP64)."""
    M = int(M)
    if M not in _SUPPORTED_M:
        raise ValueError(f"Unsupported value of M={M}. Only 42, 63, and 106 are supported.")
    J, I, dt = _SUPPORTED_M[M]
    eng = _geometry_engine(M)
    geo = eng.geometry(0)
    lambdas = torch.linspace(-math.pi, math.pi, I + 1, dtype=torch.float64, device=eng.device)[:-1]
    return M, I, J, dt, lambdas, geo["mus"], geo["w"]


_GEO_ENGINES: Dict[int, Engine] = {}


def _geometry_engine(M: int) -> Engine:
    if M not in _GEO_ENGINES:
        _GEO_ENGINES[M] = Engine([(M, 1)], "fp64")
    return _GEO_ENGINES[M]


@dataclass(frozen=True)
class RunFlags:
    """``model.py:156-226``."""

    forcflag: bool = True
    diffflag: bool = True
    expflag: bool = False
    modalflag: bool = True
    diagnostics: bool = True
    semi_implicit: bool = False
    raw_filter: bool = False
    alpha: Any = 0.01
    blowup_rms: Any = 8000.0
    williams_alpha: Any = 0.53
    si_alpha: Any = 0.5


@dataclass(frozen=True)
class Static:
    """Geometry, operators and constants (``model.py:228-378``), as FP64 GPU tensors."""

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
    lambdas: torch.Tensor
    mus: torch.Tensor
    w: torch.Tensor
    Pmn: torch.Tensor
    Hmn: torch.Tensor
    Pmnw: torch.Tensor
    Hmnw: torch.Tensor
    fmn: torch.Tensor
    tstepcoeff: torch.Tensor
    tstepcoeff2: torch.Tensor
    tstepcoeffmn: torch.Tensor
    marray: torch.Tensor
    mJarray: torch.Tensor
    narray: torch.Tensor
    sigma: torch.Tensor
    sigmaPhi: torch.Tensor
    sigma_exp: torch.Tensor
    sigmaPhi_exp: torch.Tensor
    Phieq: torch.Tensor


class State(NamedTuple):
    """Scan carry with the reference's 27 fields (``model.py:380-425``)."""

    etam_prev: torch.Tensor
    etam_curr: torch.Tensor
    deltam_prev: torch.Tensor
    deltam_curr: torch.Tensor
    Phim_prev: torch.Tensor
    Phim_curr: torch.Tensor
    eta_prev: torch.Tensor
    eta_curr: torch.Tensor
    delta_prev: torch.Tensor
    delta_curr: torch.Tensor
    Phi_prev: torch.Tensor
    Phi_curr: torch.Tensor
    U_curr: torch.Tensor
    V_curr: torch.Tensor
    Um_curr: torch.Tensor
    Vm_curr: torch.Tensor
    Am_curr: torch.Tensor
    Bm_curr: torch.Tensor
    Cm_curr: torch.Tensor
    Dm_curr: torch.Tensor
    Em_curr: torch.Tensor
    PhiFm_curr: torch.Tensor
    Fm_curr: torch.Tensor
    Gm_curr: torch.Tensor
    Rum_lag: torch.Tensor
    Rvm_lag: torch.Tensor
    dead: torch.Tensor


def _scalar_tensor(x, dev):
    return torch.as_tensor(x, dtype=torch.float64, device=dev)


def build_static(*, M, dt, a, omega, g, Phibar, taurad, taudrag, DPhieq, K6, K6Phi, test, engine: Optional[Engine] = None) -> Static:
    """``model.py:457-557`` on the GPU (FP64).  Scalars may be per-member vectors."""
    eng = engine if engine is not None else _geometry_engine(int(M))
    geo = eng.geometry(0)
    dev = eng.device
    M = int(M)
    N = M
    J, I, _ = _SUPPORTED_M[M]
    mus, w, Pmn, Hmn = geo["mus"], geo["w"], geo["Pmn"], geo["Hmn"]
    lambdas = torch.linspace(-math.pi, math.pi, I + 1, dtype=torch.float64, device=dev)[:-1]
    vals = [_scalar_tensor(v, dev) for v in (dt, a, omega, g, Phibar, taurad, taudrag, DPhieq, K6,
                                             K6 if K6Phi is None else K6Phi)]
    if any(v.dim() for v in vals):  # ensemble: broadcast every scalar to the member axis
        Bn = max(v.shape[0] for v in vals if v.dim())
        vals = [v.expand(Bn) if v.dim() == 0 else v for v in vals]
    dt_, a_, om_, g_, Pb_, tr_, td_, DP, K6_, K6P = vals
    n = torch.arange(N + 1, dtype=torch.float64, device=dev)
    mm = torch.arange(M + 1, dtype=torch.float64, device=dev)
    nn1 = n * (n + 1)
    den = nn1.clone()
    den[0] = 1.0
    tcmn = a_[..., None, None] / den if a_.dim() else a_ / den
    tcmn = tcmn * (n > 0)
    tcmn = torch.broadcast_to(tcmn, tcmn.shape[:-1] + (M + 1, N + 1)) if tcmn.dim() == 1 else tcmn.expand(*tcmn.shape[:-2], M + 1, N + 1)
    fmn = torch.zeros(a_.shape + (M + 1, N + 1), dtype=torch.float64, device=dev)
    fmn[..., 0, 1] = om_ / math.sqrt(0.375)
    onem = (1.0 - mus**2)[:, None]
    if dt_.dim():
        tsc = (2.0 * dt_[:, None, None]) / (a_[:, None, None] * onem)
        tsc = tsc.expand(-1, J, M + 1)
        tsc2 = (2.0 * dt_ / a_**2)[:, None, None].expand(-1, J, M + 1)
    else:
        tsc = ((2.0 * dt_) / (a_ * onem)).expand(J, M + 1)
        tsc2 = torch.full((J, M + 1), float(2.0 * dt_ / a_**2), dtype=torch.float64, device=dev)

    def _sig(K, off, expo):
        aa = a_[..., None] if a_.dim() else a_
        tt = dt_[..., None] if dt_.dim() else dt_
        KK = K[..., None] if K.dim() else K
        nc = ((n * n * n) / aa**3) * (((n + 1) * (n + 1) * (n + 1)) / aa**3)
        f1 = 8 / aa**6 if off else 0.0
        if expo:
            out = torch.exp(-2 * tt * KK * torch.clamp(nc - f1, min=0.0)) if off else torch.exp(-2 * tt * KK * nc)
        else:
            out = 1 / (1 + 2 * tt * KK * (nc - f1))
        return out[..., None, :].expand(*out.shape[:-1], M + 1, N + 1)

    if test is None:
        lam = lambdas[None, :]
        day = ((lambdas > -math.pi / 2) & (lambdas < math.pi / 2))[None, :]
        term_shape = torch.cos(lam) * torch.sqrt(1 - mus[:, None] ** 2)
        if DP.dim():
            Phieq = Pb_[:, None, None] + torch.where(day, DP[:, None, None] * term_shape, 0.0)
        else:
            Phieq = Pb_ + torch.where(day, DP * term_shape, 0.0)
    else:
        Phieq = torch.zeros((J, I), dtype=torch.float64, device=dev)
    return Static(
        M=M, N=N, I=I, J=J, dt=dt_, a=a_, omega=om_, g=g_, Phibar=Pb_, taurad=tr_, taudrag=td_,
        lambdas=lambdas, mus=mus, w=w, Pmn=Pmn, Hmn=Hmn, Pmnw=w[:, None, None] * Pmn, Hmnw=w[:, None, None] * Hmn,
        fmn=fmn, tstepcoeff=tsc, tstepcoeff2=tsc2, tstepcoeffmn=tcmn,
        marray=mm[:, None].expand(M + 1, N + 1), mJarray=mm[None, :].expand(J, M + 1), narray=nn1[None, :].expand(M + 1, N + 1),
        sigma=_sig(K6_, True, False), sigmaPhi=_sig(K6P, False, False), sigma_exp=_sig(K6_, True, True),
        sigmaPhi_exp=_sig(K6P, False, True), Phieq=Phieq,
    )


def _analytic_ic(M, a, omega, Phibar, test, a1, dev):
    """``model.py:669-691`` / ``initial_conditions.py:18-239`` in FP64 on the GPU."""
    J, I, _ = _SUPPORTED_M[M]
    eng = _geometry_engine(M)
    mus = eng.geometry(0)["mus"].to(dev)
    lam = torch.linspace(-math.pi, math.pi, I + 1, dtype=torch.float64, device=dev)[:-1][None, :]
    mu = mus[:, None]
    sq = torch.sqrt(1.0 - mu**2)
    SU0 = 2.0 * math.pi * a / (3600.0 * 24.0 * 12.0)
    sina, cosa = math.sin(a1), math.cos(a1)
    etaamp = 2.0 * ((SU0 / a) + omega)
    Phiamp = SU0 * a * omega + 0.5 * SU0**2
    z = torch.zeros((J, I), dtype=torch.float64, device=dev)
    if test == 1:
        arg = -torch.cos(lam) * sq * sina + mu * cosa
        eta0 = etaamp * arg
        bumpr = a / 3.0
        dist_arg = 0.0 * mu + math.cos(math.asin(0.0)) * torch.cos(torch.asin(mu)) * torch.cos(lam - 3.0 * math.pi / 2.0)
        dist = a * torch.arccos(torch.clamp(dist_arg, -1.0, 1.0))
        bump = (Phibar / 2.0) * (1.0 + torch.cos(math.pi * dist / bumpr))
        Phi0 = torch.where(dist < bumpr, bump, 0.0)
        U0 = SU0 * (sq * cosa + mu * torch.cos(lam) * sina) * sq
        V0 = -SU0 * torch.sin(lam) * sina * sq
    elif test == 2:
        arg = -torch.cos(lam) * sq * sina + mu * cosa
        eta0 = etaamp * arg
        Phi0 = (Phibar - Phiamp) * (arg**2)
        U0 = SU0 * (sq * cosa + torch.cos(lam) * mu * sina)
        V0 = (-SU0 * (torch.sin(lam) * sina)).expand(J, I)
    else:
        eta0 = (etaamp * mu).expand(J, I)
        Phi0 = z
        U0 = z
        V0 = z
    return [t.expand(J, I).contiguous() for t in (eta0, z, Phi0, U0, V0)]


def _first_dead_index(dead: torch.Tensor) -> torch.Tensor:
    """``model.py:1768-1795`` (per member along the last axis)."""
    d = dead.bool()
    if d.shape[-1] == 0:
        return torch.full(d.shape[:-1], -1, dtype=torch.int32, device=d.device)
    first = torch.argmax(d.to(torch.int32), dim=-1).to(torch.int32)
    return torch.where(d.any(dim=-1), first, torch.full_like(first, -1))


def assert_finite_state(last_state: State, *, raise_on_nan: bool = True) -> bool:
    """``model.py:1798-1841``."""
    bad = [n for n in ("eta_curr", "delta_curr", "Phi_curr", "U_curr", "V_curr")
           if not bool(torch.isfinite(getattr(last_state, n)).all())]
    if bad:
        if raise_on_nan:
            raise RuntimeError(
                "Final state contains non-finite values in fields: " + ", ".join(bad)
                + ". This usually indicates the integration blew up. Consider enabling diagnostics=True "
                "to gate on RMS-wind blowup, or reducing dt / increasing K6."
            )
        return False
    return True


def _is_python_scalar(x) -> bool:
    return isinstance(x, (int, float, np.floating))


def _member_count(*vals) -> Optional[int]:
    B = None
    for v in vals:
        if v is None or _is_python_scalar(v):
            continue
        t = torch.as_tensor(v)
        if t.dim() == 0:
            continue
        if t.dim() != 1:
            raise ValueError("per-member parameters must be scalars or 1-D sequences")
        if B is None:
            B = t.shape[0]
        elif t.shape[0] != B:
            raise ValueError("per-member parameter sequences must all have the same length")
    return B


def _prepare_ic(x, J, I, B, batched, name, dev):
    t = torch.as_tensor(x, dtype=torch.float64, device=dev)
    if t.shape == (J, I):
        return t.expand(B, J, I)
    if batched and t.shape == (B, J, I):
        return t
    raise ValueError(f"{name} must have shape {(J, I)}, got {tuple(t.shape)}.")


def _tracked(x) -> bool:
    """True for a tensor that carries a reverse-mode graph or a forward-mode tangent."""
    if not torch.is_tensor(x):
        return False
    if x.requires_grad and torch.is_grad_enabled():
        return True
    return fwAD.unpack_dual(x).tangent is not None


def _per_member(x, B: int, dev) -> torch.Tensor:
    t = x if torch.is_tensor(x) else torch.as_tensor(x, dtype=torch.float64)
    t = t.to(device=dev, dtype=torch.float64)
    return t.expand(B) if t.dim() == 0 else t.reshape(B)


def run_model_scan(
    *, M: int, dt, tmax: int, Phibar, omega, a, test: Optional[int] = None, g=9.8, forcflag: bool = True,
    taurad=86400.0, taudrag=86400.0, DPhieq=4 * (10**6), a1=0.05, diffflag: bool = True, modalflag: bool = True,
    alpha=0.01, expflag: bool = False, K6=1.24 * (10**33), K6Phi=None, contflag: bool = False,
    custompath: Optional[str] = None, contTime=None, timeunits: str = "hours", starttime: Optional[int] = None,
    eta0_init=None, delta0_init=None, Phi0_init=None, U0_init=None, V0_init=None,
    semi_implicit: bool = False, si_alpha=0.5, raw_filter: bool = False, williams_alpha=0.53,
    diagnostics: bool = True, return_history: bool = True, remat_step: bool = False, jit_scan: bool = True,
    donate_state: bool = False, precision: str = "fp64", device=None,
) -> Dict[str, Any]:
    """Full run with time histories.  Same keywords and validation as the
    reference (``model.py:1345-1765``); ``remat_step``, ``jit_scan`` and
    ``donate_state`` are accepted for compatibility and have no effect (the
    scan body is always a compiled kernel pair and the state is updated in
    place).  Tensors among taurad, taudrag, DPhieq, Phibar, a, dt, K6, K6Phi,
    omega, alpha, g and the ``*_init`` fields that require grad (or carry
    forward-mode tangents) make the
    ``last_state`` curr fields (eta, delta, Phi, U, V) differentiable through
    the hand-written adjoint and tangent-linear kernels, the counterpart of
    ``jax.grad`` / ``jax.jvp`` through the reference's scan.  ``semi_implicit`` selects the semi-implicit leapfrog
    (``semi_implicit_tdiff.py``) and ``raw_filter`` the Robert-Asselin-Williams
    filter (``model.py:1007-1087``); both run forward only (the hand-written
    adjoint covers the modified-Euler scheme with the classic filter).
    """
    if tmax < 2:
        raise ValueError("tmax must be >= 2 (SWAMPE uses a 2-level initialization).")
    if _is_python_scalar(dt) and float(dt) <= 0.0:
        raise ValueError("dt must be positive.")
    if test is not None:
        test = int(test)
    if semi_implicit and expflag:
        raise ValueError("semi_implicit=True is incompatible with expflag=True (pick one scheme).")
    if raw_filter and expflag:
        raise ValueError(
            "raw_filter=True is incompatible with expflag=True (the explicit scheme reads the "
            "unfiltered spectral prev carry, so the RAW lineage change would alter its parity behavior)."
        )
    if test not in (None, 1, 2):
        raise NotImplementedError(f"test={test} is not implemented (use None, 1 or 2)")
    M = int(M)
    if M not in _SUPPORTED_M:
        raise ValueError(f"Unsupported value of M={M}. Only 42, 63, and 106 are supported.")
    J, I, _ = _SUPPORTED_M[M]

    # start time (model.py:1574-1613)
    timestamp_val = None
    cont_key = None
    if contflag:
        if contTime is None:
            raise ValueError("contflag=True requires contTime.")
        try:
            timestamp_val = float(contTime)
        except (TypeError, ValueError) as e:
            raise ValueError(f"contTime must be numeric (int/float or numeric string), got {contTime!r}.") from e
        ts_round = round(timestamp_val)
        cont_key = str(int(ts_round)) if abs(timestamp_val - ts_round) < 1e-12 else str(contTime)
    if starttime is None:
        starttime_eff = 2 if not contflag else continuation.compute_t_from_timestamp(timeunits, timestamp_val, float(dt))
    else:
        starttime_eff = int(starttime)
    if starttime_eff > tmax:
        raise ValueError(f"starttime={starttime_eff} must be <= tmax={tmax}.")

    have_ic = (eta0_init is not None) or (delta0_init is not None) or (Phi0_init is not None)
    ic_derivs: Dict[str, torch.Tensor] = {}  # d(analytic initial fields) / d(parameter), semi-implicit runs
    if have_ic and (eta0_init is None or delta0_init is None or Phi0_init is None):
        raise ValueError("If providing explicit ICs, eta0_init, delta0_init, and Phi0_init must all be provided.")
    if have_ic and ((U0_init is None) != (V0_init is None)):
        raise ValueError("Provide both U0_init and V0_init, or neither.")

    Bm = _member_count(dt, a, omega, Phibar, taurad, taudrag, DPhieq, K6, K6Phi, alpha,
                       si_alpha if semi_implicit else None, williams_alpha if raw_filter else None)
    for x in (eta0_init, delta0_init, Phi0_init, U0_init, V0_init):
        if x is not None and torch.as_tensor(x).dim() == 3:
            b = torch.as_tensor(x).shape[0]
            if Bm is not None and b != Bm:
                raise ValueError("member axis of the initial fields does not match the parameters")
            Bm = b
    batched = Bm is not None
    B = Bm if batched else 1
    # shapes of the explicit initial fields, checked at entry like the reference
    # (before any device work)
    for name, x in (("eta0_init", eta0_init), ("delta0_init", delta0_init), ("Phi0_init", Phi0_init),
                    ("U0_init", U0_init), ("V0_init", V0_init)):
        if x is not None:
            shp = tuple(torch.as_tensor(x).shape)
            if shp != (J, I) and not (batched and shp == (B, J, I)):
                raise ValueError(f"{name} must have shape {(J, I)}, got {shp}.")

    # differentiable inputs: the per-member parameters the adjoint and the tangent
    # model cover, the initial fields, and alpha and g, which the curr fields of
    # the modified-Euler scheme do not depend on (their derivative is zero)
    # K6Phi=None means K6Phi = K6 (model.py:512): then K6 drives both
    coef_inputs = dict(a=a, dt=dt, K6=K6, K6Phi=K6 if K6Phi is None else K6Phi, omega=omega, si_alpha=si_alpha)
    ic_inputs = (eta0_init, delta0_init, Phi0_init, U0_init, V0_init)
    diff_inputs = (taurad, taudrag, DPhieq, Phibar, *ic_inputs, alpha, g, *coef_inputs.values())
    needs_grad = any(_tracked(x) for x in diff_inputs)
    if _tracked(williams_alpha):
        raise NotImplementedError("derivatives through the RAW filter are not implemented")
    tangent_only = bool(semi_implicit or expflag)  # schemes differentiated by tangent runs (no adjoint)
    if needs_grad:
        if raw_filter or test == 1:
            raise NotImplementedError("derivatives are implemented with the classic filter and test None or 2")
        if U0_init is None and (_tracked(eta0_init) or _tracked(delta0_init)):
            raise NotImplementedError("derivatives with respect to eta0_init / delta0_init need U0_init and V0_init")
        if tangent_only and torch.is_grad_enabled() and any(torch.is_tensor(x) and x.requires_grad for x in ic_inputs):
            raise NotImplementedError("reverse-mode gradients with respect to the initial fields need the adjoint, "
                                      "which the explicit and semi-implicit schemes do not have (forward mode works)")

    eng = Engine([(M, B)], precision, device)
    dev = eng.device
    K6Phi_eff = K6 if K6Phi is None else K6Phi
    eng.set_params(0, dt=dt, a=a, omega=omega, Phibar=Phibar, taurad=taurad, taudrag=taudrag,
                   DPhieq=DPhieq if test is None else 0.0, K6=K6, K6Phi=K6Phi_eff, alpha=alpha,
                   si_alpha=si_alpha, williams_alpha=williams_alpha)
    nd = lambda x: x.detach() if torch.is_tensor(x) else x  # noqa: E731  (the Static record holds values)
    static = build_static(M=M, dt=nd(dt), a=nd(a), omega=nd(omega), g=nd(g), Phibar=nd(Phibar), taurad=nd(taurad),
                          taudrag=nd(taudrag), DPhieq=nd(DPhieq), K6=nd(K6), K6Phi=nd(K6Phi), test=test, engine=eng)

    if have_ic:
        eta0 = _prepare_ic(eta0_init, J, I, B, batched, "eta0_init", dev)
        delta0 = _prepare_ic(delta0_init, J, I, B, batched, "delta0_init", dev)
        Phi0 = _prepare_ic(Phi0_init, J, I, B, batched, "Phi0_init", dev)
        if U0_init is not None:
            U0 = _prepare_ic(U0_init, J, I, B, batched, "U0_init", dev)
            V0 = _prepare_ic(V0_init, J, I, B, batched, "V0_init", dev)
        else:
            U0, V0 = eng.diagnose_winds([torch.stack((eta0, delta0), 0).to(eng.rdtype)])[0].to(torch.float64)
    elif not contflag:
        if batched and not all(_is_python_scalar(v) for v in (a, omega, Phibar)):
            raise ValueError("analytic initial conditions need scalar a, omega and Phibar; pass *_init fields instead")
        val = lambda x: float(x.detach()) if torch.is_tensor(x) else float(x)  # noqa: E731
        av, omv, pb = val(a), val(omega), val(Phibar)
        fields = _analytic_ic(M, av, omv, pb, test, float(a1), dev)
        eta0, delta0, Phi0, U0, V0 = (f.expand(B, J, I) for f in fields)
        # the analytic fields are polynomials of degree <= 2 in a, omega, Phibar
        # (initial_conditions.py:18-47, 88-239), so a centred difference is their
        # exact derivative: carry it into the differentiable run
        # (the explicit and semi-implicit schemes, which differentiate by tangent
        # runs, take them as initial-field tangents of the parameter directions)
        for x, i, name in ((a, 0, "a"), (omega, 1, "omega"), (Phibar, 2, "Phibar")):
            if _tracked(x):
                h = 1e-3 * abs((av, omv, pb)[i]) or 1e-3
                arg = [av, omv, pb]
                arg[i] += h
                fp = _analytic_ic(M, *arg, test, float(a1), dev)
                arg[i] -= 2 * h
                fm = _analytic_ic(M, *arg, test, float(a1), dev)
                d = [(u - v) / (2 * h) for u, v in zip(fp, fm)]
                if semi_implicit or expflag:
                    ic_derivs[name] = torch.stack([dd.expand(B, J, I) for dd in d], 0)
                    continue
                dx = x - x.detach()
                eta0, delta0, Phi0, U0, V0 = (f + dx * dd.expand(B, J, I)
                                              for f, dd in zip((eta0, delta0, Phi0, U0, V0), d))
    else:
        fields = []
        for name in ("eta", "delta", "Phi"):
            try:
                arr = continuation.read_pickle(f"{name}-{cont_key}", custompath=custompath)
            except FileNotFoundError:
                if str(contTime) == cont_key:
                    raise
                arr = continuation.read_pickle(f"{name}-{contTime}", custompath=custompath)
            fields.append(_prepare_ic(arr, J, I, B, False, name, dev))
        eta0, delta0, Phi0 = fields
        U0, V0 = eng.diagnose_winds([torch.stack((eta0, delta0), 0).to(eng.rdtype)])[0].to(torch.float64)

    flags = RunFlagsC(scheme=2 if semi_implicit else (1 if expflag else 0), forcflag=forcflag, diffflag=diffflag,
                      modalflag=modalflag, test=test, diagnostics=diagnostics, blowup_rms=8000.0,
                      t_start=starttime_eff, raw_filter=bool(raw_filter))
    T = tmax - starttime_eff
    diag = eng.new_diag(T) if diagnostics else None
    gd = eng.groups[0]
    hist = [torch.empty((max(T, 0), 5, B, J, I), dtype=eng.rdtype, device=dev)] if return_history else None
    ics = torch.stack((eta0, delta0, Phi0, U0, V0), 0)
    eng.init_state([ics.detach()], flags, diag=diag)
    four = gd["fourier"]
    # Rum_lag/Rvm_lag: pass-through carries of the semi-implicit scheme (model.py:734-739, 775-792)
    td = gd["params"][_lib.P_TAUDRAG]
    inv_td = torch.where(td == -1.0, torch.zeros_like(td), 1.0 / td).to(eng.rdtype)
    Rum = four[_lib.F_F] + four[_lib.F_U] * inv_td[None, :, None]
    Rvm = four[_lib.F_G] + four[_lib.F_V] * inv_td[None, :, None]
    dcurr = None
    if needs_grad and T > 0:
        # the differentiable final curr fields; with neither history nor
        # diagnostics asked for, this run is the run (the engine holds its final state)
        from . import adjoint

        if return_history or diagnostics:
            eng.forward(flags, t0=starttime_eff, nsteps=T, row0=0, diag=diag, hist=hist, write_prev_last=True)
            saved = (four.clone(), gd["member"].clone())
        dflags = RunFlagsC(scheme=2 if semi_implicit else (1 if expflag else 0), forcflag=forcflag, diffflag=diffflag,
                           modalflag=modalflag, test=test, diagnostics=False, t_start=starttime_eff)
        dpar = dict(taurad=_per_member(taurad, B, dev), taudrag=_per_member(taudrag, B, dev),
                    DPhieq=_per_member(DPhieq if test is None else 0.0, B, dev), Phibar=_per_member(Phibar, B, dev))
        for k, x in coef_inputs.items():
            if _tracked(x):
                dpar[k] = _per_member(x, B, dev)
        dcurr = adjoint.integrate(eng, dflags, starttime_eff, T, [dpar], [ics], ic_derivs=[ic_derivs])[0]
        for x in (alpha, g):  # zero derivative, but part of the graph
            if _tracked(x):
                dcurr = dcurr + 0.0 * x.to(dcurr.dtype).sum()
        if return_history or diagnostics:  # the gated run's state (dead flags included)
            four.copy_(saved[0])
            gd["member"].copy_(saved[1])
    elif T > 0:
        eng.forward(flags, t0=starttime_eff, nsteps=T, row0=0, diag=diag, hist=hist, write_prev_last=True)
    phys = eng.output_physical(flags)[0]
    eng.check_device_status()
    if semi_implicit and T > 0:  # the lagged remainders the steps advanced
        Rum, Rvm = four[_lib.F_RU_LAG].clone(), four[_lib.F_RV_LAG].clone()
    # the Fourier prev carry follows the filtered lineage with the semi-implicit
    # scheme or the RAW filter, the unfiltered curr otherwise (model.py:1089-1110)
    last = _assemble_state(eng, phys, Rum, Rvm, batched, filtered_prev=bool(semi_implicit or raw_filter))
    if dcurr is not None:
        pick = (lambda v: v) if batched else (lambda v: v[0])
        last = last._replace(eta_curr=pick(dcurr[0]), delta_curr=pick(dcurr[1]), Phi_curr=pick(dcurr[2]),
                             U_curr=pick(dcurr[3]), V_curr=pick(dcurr[4]))
    res: Dict[str, Any] = dict(static=static, t_seq=torch.arange(starttime_eff, tmax, dtype=torch.int32, device=dev),
                               last_state=last, starttime=starttime_eff)
    if return_history:
        h = hist[0]
        outs = {}
        for k, name in enumerate(("eta", "delta", "Phi", "U", "V")):
            v = h[:, k]  # (T, B, J, I)
            outs[name] = v.permute(1, 0, 2, 3) if batched else v[:, 0]
        if diagnostics:
            d = diag[0][:T]  # (T, 5, B)
            vals = dict(rms=torch.sqrt(d[:, _lib.D_RMS2]), spin_min=d[:, _lib.D_SPIN], phi_min=d[:, _lib.D_PHIMIN],
                        phi_max=d[:, _lib.D_PHIMAX], dead=d[:, _lib.D_DEAD] != 0)
        else:
            z = torch.zeros((T, B), dtype=torch.float64, device=dev)
            vals = dict(rms=z, spin_min=z, phi_min=z, phi_max=z, dead=torch.zeros((T, B), dtype=torch.bool, device=dev))
        for k, v in vals.items():
            outs[k] = v.t() if batched else v[:, 0]
        res["outs"] = outs
        res["dead_first_idx"] = _first_dead_index(outs["dead"])
    return res


def _assemble_state(eng: Engine, phys: torch.Tensor, Rum, Rvm, batched: bool, filtered_prev: bool = False) -> State:
    gd = eng.groups[0]
    four = gd["fourier"]

    def fo(k):  # (M+1, B, J) -> (B, J, M+1)
        v = four[k].permute(1, 2, 0)
        return v if batched else v[0]

    def fr(t):
        v = t.permute(1, 2, 0)
        return v if batched else v[0]

    def ph(k):
        return phys[k] if batched else phys[k, 0]

    dead = gd["member"][_lib.MS_DEAD] != 0
    if filtered_prev:
        pe, pd, pp = _lib.F_ETA_MID, _lib.F_DELTA_MID, _lib.F_PHI_MID
    else:
        pe, pd, pp = _lib.F_ETA_PREV, _lib.F_DELTA_PREV, _lib.F_PHI_PREV
    return State(
        etam_prev=fo(pe), etam_curr=fo(_lib.F_ETA), deltam_prev=fo(pd),
        deltam_curr=fo(_lib.F_DELTA), Phim_prev=fo(pp), Phim_curr=fo(_lib.F_PHI),
        eta_prev=ph(5), eta_curr=ph(0), delta_prev=ph(6), delta_curr=ph(1), Phi_prev=ph(7), Phi_curr=ph(2),
        U_curr=ph(3), V_curr=ph(4), Um_curr=fo(_lib.F_U), Vm_curr=fo(_lib.F_V), Am_curr=fo(_lib.F_A),
        Bm_curr=fo(_lib.F_B), Cm_curr=fo(_lib.F_C), Dm_curr=fo(_lib.F_D), Em_curr=fo(_lib.F_E),
        PhiFm_curr=fo(_lib.F_PHIF), Fm_curr=fo(_lib.F_F), Gm_curr=fo(_lib.F_G), Rum_lag=fr(Rum), Rvm_lag=fr(Rvm),
        dead=dead if batched else dead[0],
    )


def run_model_scan_final(**kw) -> Dict[str, Any]:
    """``model.py:1844-1951``: terminal state only; diagnostics off by default."""
    if "return_history" in kw:
        raise TypeError("run_model_scan_final() got an unexpected keyword argument 'return_history'")
    kw.setdefault("diagnostics", False)
    return run_model_scan(return_history=False, **kw)


def run_model(M, dt, tmax, Phibar, omega, a, test=None, g=9.8, forcflag=True, taurad=86400, taudrag=86400,
              DPhieq=4 * (10**6), a1=0.05, plotflag=True, plotfreq=5, minlevel=None, maxlevel=None,
              diffflag=True, modalflag=True, alpha=0.01, contflag=False, saveflag=True, expflag=False,
              savefreq=150, K6=1.24 * 10**33, custompath=None, contTime=None, timeunits="hours", verbose=True,
              *, K6Phi=None, semi_implicit=False, si_alpha=0.5, raw_filter=False, williams_alpha=0.53,
              jit_scan=True, as_numpy=True, precision="fp64", device=None) -> Dict[str, Any]:
    """SWAMPE-compatible wrapper (``model.py:1954-2219``): history on the host,
    legacy ``(tmax, 2)`` spinup/geopot arrays (``:2106-2158``) and optional
    pickle saving every savefreq steps.  ``plotflag`` only warns: host plotting
    (``plotting.py``) is not part of this package."""
    result = run_model_scan(M=M, dt=dt, tmax=tmax, Phibar=Phibar, omega=omega, a=a, test=test, g=g,
                            forcflag=forcflag, taurad=taurad, taudrag=taudrag, DPhieq=DPhieq, a1=a1,
                            diffflag=diffflag, modalflag=modalflag, alpha=alpha, expflag=expflag, K6=K6,
                            K6Phi=K6Phi, contflag=contflag, custompath=custompath, contTime=contTime,
                            timeunits=timeunits, semi_implicit=semi_implicit, si_alpha=si_alpha,
                            raw_filter=raw_filter, williams_alpha=williams_alpha, jit_scan=jit_scan,
                            precision=precision, device=device)
    static = result["static"]
    outs = result["outs"]
    need_host = bool(as_numpy or saveflag or plotflag)
    conv = (lambda x: x.detach().cpu().numpy()) if need_host else (lambda x: x)
    t_seq = conv(result["t_seq"])
    hist = {k: conv(outs[k]) for k in ("eta", "delta", "Phi", "U", "V", "rms", "spin_min", "phi_min", "phi_max")}
    lib = np if need_host else torch
    dev = result["t_seq"].device
    spin = np.zeros((tmax, 2)) if need_host else torch.zeros((tmax, 2), dtype=torch.float64, device=dev)
    geop = np.zeros((tmax, 2)) if need_host else torch.zeros((tmax, 2), dtype=torch.float64, device=dev)
    idx = (t_seq.astype(np.int64) - 1) if need_host else (t_seq.long() - 1)
    ok = (idx >= 0) & (idx < tmax)
    spin[idx[ok], 0] = hist["spin_min"][ok]
    spin[idx[ok], 1] = hist["rms"][ok]
    geop[idx[ok], 0] = hist["phi_min"][ok]
    geop[idx[ok], 1] = hist["phi_max"][ok]
    if not contflag:  # model.py:2132-2158: index 0 from the analytic initial condition
        fields = _analytic_ic(int(M), float(a), float(omega), float(Phibar), test, float(a1), dev)
        _, _, P0, U0, V0 = fields
        mus = static.mus
        phis = torch.arcsin(mus)[:, None]
        dlam = static.lambdas[2] - static.lambdas[1]
        dphi = phis[2, 0] - phis[1, 0]
        comp = (a**2) * (torch.sin(phis + math.pi / 2.0) ** 2) * dphi * dlam
        rms0 = torch.sqrt(torch.sum(comp * ((U0 / torch.cos(phis)) ** 2 + (V0 / torch.cos(phis)) ** 2) / (4.0 * math.pi * a**2)))
        vals = (torch.min(torch.sqrt(U0 * U0 + V0 * V0)), rms0, torch.min(P0), torch.max(P0))
        vals = [float(v) for v in vals] if need_host else vals
        spin[0, 0], spin[0, 1], geop[0, 0], geop[0, 1] = vals
    if saveflag:
        for k, t in enumerate(t_seq):
            if int(t) % int(savefreq) == 0:
                ts = continuation.compute_timestamp(timeunits, int(t), dt)
                continuation.save_data(ts, hist["eta"][k], hist["delta"][k], hist["Phi"][k], hist["U"][k],
                                       hist["V"][k], spin, geop, custompath=custompath)
    if plotflag:
        # model.py:2180-2203 draws matplotlib figures on the host; plotting is not
        # part of this package (the histories it would draw are returned)
        warnings.warn("run_model(plotflag=True): plotting is not part of my_swampe_gb300; plot the returned "
                      "fields with the reference's my_swampe.plotting", stacklevel=2)
    if verbose:
        print("GCM run completed!")
    T = hist["eta"].shape[0]
    return dict(
        eta=hist["eta"][-1] if T else None, delta=hist["delta"][-1] if T else None, Phi=hist["Phi"][-1] if T else None,
        U=hist["U"][-1] if T else None, V=hist["V"][-1] if T else None, spinup=spin, geopot=geop,
        lambdas=conv(static.lambdas), mus=conv(static.mus), t_seq=t_seq,
    )


def run_model_gpu(*args, **kwargs) -> Dict[str, Any]:
    """``model.py:2222-2251``: run_model with GPU-friendly defaults."""
    kwargs = dict(kwargs)
    kwargs.setdefault("plotflag", False)
    kwargs.setdefault("saveflag", False)
    kwargs.setdefault("as_numpy", False)
    kwargs.setdefault("jit_scan", True)
    return run_model(*args, **kwargs)
