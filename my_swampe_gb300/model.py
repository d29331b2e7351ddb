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
from collections import OrderedDict
from dataclasses import dataclass, replace as _dc_replace
from typing import Any, Dict, NamedTuple, Optional, Tuple

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


# Engines (plan, geometry, packed bases, device state, captured step graphs)
# reused across calls, keyed on (M, B, precision, device): the counterpart of
# the reference's lru_cache'd geometry and per-key compiled scans
# (model.py:62-153).  A call never returns views of an engine's buffers.
_ENGINE_CACHE: "OrderedDict[tuple, Engine]" = OrderedDict()
_ENGINE_CACHE_SIZE = 8


def _engine_for(M: int, B: int, precision: str, device=None, steps: bool = True) -> Engine:
    """The cached one-group engine of (M, B, precision).  steps=False: an engine
    that only prepares geometry and initial fields (its ensemble steps on a
    split engine), so the Legendre kernels are not autotuned for it."""
    dev = torch.device(device) if device is not None else (
        torch.device("cuda", torch.cuda.current_device()) if torch.cuda.is_available() else torch.device("cuda"))
    tune = bool(steps) and int(B) >= 32
    key = (int(M), int(B), precision, dev.type, dev.index, tune)
    eng = _ENGINE_CACHE.pop(key, None)
    if eng is None:
        # ensembles of 32 members or more: the autotuner picks the Legendre kernel
        # (tensor cores or a SIMT member tile) once per (M, B, precision) in the
        # process; smaller ones keep the default (tensor cores where available)
        eng = Engine([(int(M), int(B))], precision, device, autotune=tune)
    _ENGINE_CACHE[key] = eng
    while len(_ENGINE_CACHE) > _ENGINE_CACHE_SIZE:
        _ENGINE_CACHE.popitem(last=False)
    return eng


# Ensembles of this many members or more run, on the plain paths (no history,
# diagnostics, semi-implicit scheme or RAW filter), as two halves of one
# concurrent plan: each half's step chain on its own stream, so that the
# kernels of one half fill the SMs the other half's leave idle.  Members are
# independent: each half's results are those of the same members run alone.
# (Forward only, M = 42, fast, 7,199 steps: 1.70M -> 2.09M member-steps/s at
# B = 64, 2.16M -> 2.47M at B = 128.)
_SPLIT_MIN_B = 64


def _split_engine_for(M: int, sizes: Tuple[int, int], precision: str, device=None) -> Engine:
    dev = torch.device(device) if device is not None else (
        torch.device("cuda", torch.cuda.current_device()) if torch.cuda.is_available() else torch.device("cuda"))
    key = (int(M), tuple(int(b) for b in sizes), precision, "split", dev.type, dev.index)
    eng = _ENGINE_CACHE.pop(key, None)
    if eng is None:
        eng = Engine([(int(M), int(b)) for b in sizes], precision, device, concurrent=True, autotune=True)
    _ENGINE_CACHE[key] = eng
    while len(_ENGINE_CACHE) > _ENGINE_CACHE_SIZE:
        _ENGINE_CACHE.popitem(last=False)
    return eng


def clear_engine_cache() -> None:
    """Release the cached engines (their plans and device buffers)."""
    _ENGINE_CACHE.clear()


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
    # scalars the tables above were built from: the kernels rebuild their
    # coefficient tables and Phieq from these (dataclasses.replace of taurad,
    # taudrag, ... takes effect, as in the retrieval's fast path)
    DPhieq: Any = None
    K6: Any = None
    K6Phi: Any = None
    test: Optional[int] = None


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
        sigmaPhi_exp=_sig(K6P, False, True), Phieq=Phieq, DPhieq=DP, K6=K6_, K6Phi=K6P, test=test,
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
    omega, si_alpha, alpha, williams_alpha, g and the ``*_init`` fields that require grad (or carry
    forward-mode tangents) make the
    ``last_state`` curr fields (eta, delta, Phi, U, V) differentiable through
    the hand-written adjoint and tangent-linear kernels, the counterpart of
    ``jax.grad`` / ``jax.jvp`` through the reference's scan.  ``semi_implicit`` selects the semi-implicit leapfrog
    (``semi_implicit_tdiff.py``) and ``raw_filter`` the Robert-Asselin-Williams
    filter (``model.py:1007-1087``).  Their parameter gradients (si_alpha,
    alpha and williams_alpha among them) are tangent-linear runs; the
    semi-implicit scheme's initial-field gradients come from its adjoint, and
    the RAW filter has forward-mode initial-field derivatives only.
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
    # model cover, the initial fields, and g.  alpha moves the curr fields only
    # where the filtered level feeds the trajectory (the semi-implicit scheme's
    # n-1 base, the RAW filter's new level), williams_alpha only with the RAW
    # filter; elsewhere their derivative (and that of g) is zero.
    # K6Phi=None means K6Phi = K6 (model.py:512): then K6 drives both
    coef_inputs = dict(a=a, dt=dt, K6=K6, K6Phi=K6 if K6Phi is None else K6Phi, omega=omega, si_alpha=si_alpha)
    zero_deriv = [g]
    if semi_implicit or raw_filter:
        coef_inputs["alpha"] = alpha
    else:
        zero_deriv.append(alpha)
    if raw_filter:
        coef_inputs["williams_alpha"] = williams_alpha
    else:
        zero_deriv.append(williams_alpha)
    ic_inputs = (eta0_init, delta0_init, Phi0_init, U0_init, V0_init)
    diff_inputs = (taurad, taudrag, DPhieq, Phibar, *ic_inputs, *zero_deriv, *coef_inputs.values())
    needs_grad = any(_tracked(x) for x in diff_inputs)
    if needs_grad:
        if test == 1:
            raise NotImplementedError("derivatives are implemented for test None or 2")
        if U0_init is None and (_tracked(eta0_init) or _tracked(delta0_init)):
            raise NotImplementedError("derivatives with respect to eta0_init / delta0_init need U0_init and V0_init")
        if raw_filter and any(torch.is_tensor(x) and x.requires_grad for x in ic_inputs):
            raise NotImplementedError("reverse-mode initial-field gradients through the RAW filter are not "
                                      "implemented (forward mode and parameter gradients are)")

    split = (batched and B >= _SPLIT_MIN_B and tmax > starttime_eff and test != 1
             and not (return_history or diagnostics or semi_implicit or raw_filter))
    eng = _engine_for(M, B, precision, device, steps=not split)
    dev = eng.device
    K6Phi_eff = K6 if K6Phi is None else K6Phi
    eng.set_params(0, dt=dt, a=a, omega=omega, Phibar=Phibar, taurad=taurad, taudrag=taudrag,
                   DPhieq=DPhieq if test is None else 0.0, K6=K6, K6Phi=K6Phi_eff, alpha=alpha,
                   si_alpha=si_alpha, williams_alpha=williams_alpha)
    nd = lambda x: x.detach() if torch.is_tensor(x) else x  # noqa: E731  (the Static record holds values)
    static = build_static(M=M, dt=nd(dt), a=nd(a), omega=nd(omega), g=nd(g), Phibar=nd(Phibar), taurad=nd(taurad),
                          taudrag=nd(taudrag), DPhieq=nd(DPhieq), K6=nd(K6), K6Phi=nd(K6Phi), test=test, engine=eng)

    ic_derivs: Dict[str, torch.Tensor] = {}  # d(initial fields) / d(parameter), outside the autograd graph
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
        # exact derivative: carry it into the differentiable run (with the RAW
        # filter, which has no adjoint, as initial-field tangents of the
        # parameter's tangent runs)
        for x, i, name in ((a, 0, "a"), (omega, 1, "omega"), (Phibar, 2, "Phibar")):
            if _tracked(x):
                h = 1e-3 * abs((av, omv, pb)[i]) or 1e-3
                arg = [av, omv, pb]
                arg[i] += h
                fp = _analytic_ic(M, *arg, test, float(a1), dev)
                arg[i] -= 2 * h
                fm = _analytic_ic(M, *arg, test, float(a1), dev)
                d = [(u - v) / (2 * h) for u, v in zip(fp, fm)]
                if raw_filter:
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
    if split:
        phys, dcurr, last = _run_split(
            M, B, precision, device, flags, starttime_eff, T, ics=torch.stack((eta0, delta0, Phi0, U0, V0), 0),
            pvals=dict(dt=dt, a=a, omega=omega, Phibar=Phibar, taurad=taurad, taudrag=taudrag,
                       DPhieq=DPhieq if test is None else 0.0, K6=K6, K6Phi=K6Phi_eff, alpha=alpha),
            needs_grad=needs_grad, coef_inputs=coef_inputs, zero_deriv=tuple(zero_deriv), batched=batched)
        return dict(static=static, t_seq=torch.arange(starttime_eff, tmax, dtype=torch.int32, device=dev),
                    last_state=last, starttime=starttime_eff)
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
                           modalflag=modalflag, test=test, diagnostics=False, t_start=starttime_eff,
                           raw_filter=bool(raw_filter))
        dpar = dict(taurad=_per_member(taurad, B, dev), taudrag=_per_member(taudrag, B, dev),
                    DPhieq=_per_member(DPhieq if test is None else 0.0, B, dev), Phibar=_per_member(Phibar, B, dev))
        for k, x in coef_inputs.items():
            if _tracked(x):
                dpar[k] = _per_member(x, B, dev)
        dcurr = adjoint.integrate(eng, dflags, starttime_eff, T, [dpar], [ics], ic_derivs=[ic_derivs])[0]
        for x in zero_deriv:  # zero derivative, but part of the graph
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


def _run_split(M, B, precision, device, flags: RunFlagsC, t0: int, T: int, ics: torch.Tensor, pvals: Dict[str, Any],
               needs_grad: bool, coef_inputs: Dict[str, Any], zero_deriv, batched: bool):
    """run_model_scan's stepping for a large ensemble as two concurrent halves
    (one plan of two groups, each chain on its own stream).  ics: (5, B, J, I);
    parameters are scalars or per-member tensors, sliced per half.  Returns the
    physical final fields (5, B, J, I), the differentiable final curr fields
    (or None) and the final State, all joined along the member axis."""
    sizes = (B // 2, B - B // 2)
    eng = _split_engine_for(M, sizes, precision, device)
    dev = eng.device
    sls = (slice(0, sizes[0]), slice(sizes[0], B))

    def part(x, sl):
        if torch.is_tensor(x) and x.dim() == 1:
            return x[sl]
        if not torch.is_tensor(x) and not _is_python_scalar(x) and np.ndim(x) == 1:
            return torch.as_tensor(x, dtype=torch.float64)[sl]
        return x

    for g, sl in enumerate(sls):
        eng.set_params(g, **{k: part(v, sl) for k, v in pvals.items()})
    ics_g = [ics[:, sl] for sl in sls]
    eng.init_state([x.detach() for x in ics_g], flags)
    # pass-through carries of the semi-implicit scheme's State fields: F + U / taudrag of the initial state
    Rum, Rvm = [], []
    for gd in eng.groups:
        four = gd["fourier"]
        td = gd["params"][_lib.P_TAUDRAG]
        inv_td = torch.where(td == -1.0, torch.zeros_like(td), 1.0 / td).to(eng.rdtype)
        Rum.append(four[_lib.F_F] + four[_lib.F_U] * inv_td[None, :, None])
        Rvm.append(four[_lib.F_G] + four[_lib.F_V] * inv_td[None, :, None])
    Rum, Rvm = torch.cat(Rum, dim=1), torch.cat(Rvm, dim=1)
    dcurr = None
    if needs_grad:
        from . import adjoint

        dflags = RunFlagsC(scheme=flags.scheme, forcflag=flags.forcflag, diffflag=flags.diffflag,
                           modalflag=flags.modalflag, test=flags.test, diagnostics=False, t_start=t0)
        dpar = dict(taurad=_per_member(pvals["taurad"], B, dev), taudrag=_per_member(pvals["taudrag"], B, dev),
                    DPhieq=_per_member(pvals["DPhieq"], B, dev), Phibar=_per_member(pvals["Phibar"], B, dev))
        for k, x in coef_inputs.items():
            if _tracked(x):
                dpar[k] = _per_member(x, B, dev)
        outs = adjoint.integrate(eng, dflags, t0, T, [{k: v[sl] for k, v in dpar.items()} for sl in sls], ics_g)
        dcurr = torch.cat(outs, dim=1)
        for x in zero_deriv:  # zero derivative, but part of the graph
            if _tracked(x):
                dcurr = dcurr + 0.0 * x.to(dcurr.dtype).sum()
    else:
        eng.forward(flags, t0=t0, nsteps=T, row0=0, write_prev_last=True)
    phys = torch.cat(eng.output_physical(flags), dim=1)
    eng.check_device_status()
    last = _assemble_state(eng, phys, Rum, Rvm, batched)
    if dcurr is not None:
        last = last._replace(eta_curr=dcurr[0], delta_curr=dcurr[1], Phi_curr=dcurr[2], U_curr=dcurr[3],
                             V_curr=dcurr[4])
    return phys, dcurr, last


def _assemble_state(eng: Engine, phys: torch.Tensor, Rum, Rvm, batched: bool, filtered_prev: bool = False) -> State:
    """The State of the engine's groups, joined along the member axis in group
    order (one group, or the two halves of a split ensemble)."""

    def fo(k):  # (M+1, B, J) -> (B, J, M+1), a copy (the engine's buffers are reused)
        f = torch.cat([gd["fourier"][k] for gd in eng.groups], dim=1)
        v = f.permute(1, 2, 0).clone(memory_format=torch.contiguous_format)
        return v if batched else v[0]

    def fr(t):
        v = t.permute(1, 2, 0).clone(memory_format=torch.contiguous_format)
        return v if batched else v[0]

    def ph(k):
        return phys[k] if batched else phys[k, 0]

    dead = torch.cat([gd["member"][_lib.MS_DEAD] for gd in eng.groups]) != 0
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


# ---------------------------------------------------------------------------
# The scan core's own entry points (model.py:694-772, 1197-1342), which the
# retrieval calls directly (retrieval/scripts/pipeline.py:646-688, 870-927):
# build_static + _init_state_from_fields once, then simulate_scan_last (or a
# loop of _step_once_state_only) per parameter sample, with
# dataclasses.replace(static, taurad=..., taudrag=...) and optional FP32 casts
# of static and state (which select the fast precision here).
# ---------------------------------------------------------------------------
# State Fourier field -> Fourier slot of the engine
_STATE_SLOTS = (("etam_curr", _lib.F_ETA), ("deltam_curr", _lib.F_DELTA), ("Phim_curr", _lib.F_PHI),
                ("Um_curr", _lib.F_U), ("Vm_curr", _lib.F_V), ("Am_curr", _lib.F_A), ("Bm_curr", _lib.F_B),
                ("Cm_curr", _lib.F_C), ("Dm_curr", _lib.F_D), ("Em_curr", _lib.F_E), ("PhiFm_curr", _lib.F_PHIF),
                ("Fm_curr", _lib.F_F), ("Gm_curr", _lib.F_G))
_PREV_NAMES = ("etam_prev", "deltam_prev", "Phim_prev")
_PREV_SLOTS = (_lib.F_ETA_PREV, _lib.F_DELTA_PREV, _lib.F_PHI_PREV)
_MID_SLOTS = (_lib.F_ETA_MID, _lib.F_DELTA_MID, _lib.F_PHI_MID)
_STATIC_PARAMS = ("dt", "a", "omega", "Phibar", "taurad", "taudrag", "DPhieq", "K6", "K6Phi")


def _state_precision(x) -> str:
    dt = x.dtype if torch.is_tensor(x) else np.asarray(x).dtype
    return "fast" if dt in (torch.float32, torch.complex64, np.float32, np.complex64) else "fp64"


def _flags_c(flags: "RunFlags", test, t_start: int, diagnostics: Optional[bool] = None) -> RunFlagsC:
    return RunFlagsC(scheme=2 if flags.semi_implicit else (1 if flags.expflag else 0), forcflag=flags.forcflag,
                     diffflag=flags.diffflag, modalflag=flags.modalflag, test=test,
                     diagnostics=flags.diagnostics if diagnostics is None else diagnostics,
                     blowup_rms=float(flags.blowup_rms), t_start=int(t_start), raw_filter=bool(flags.raw_filter))


def _static_values(static: Static, flags: "RunFlags", test) -> Dict[str, Any]:
    """Per-member parameter values of a Static (tensors keep their autograd
    graph and forward-mode tangents)."""
    if static.K6 is None or static.DPhieq is None:
        raise ValueError("this Static carries no K6 / DPhieq: build it with my_swampe_gb300.model.build_static")
    vals = {k: getattr(static, k) for k in _STATIC_PARAMS}
    if vals["K6Phi"] is None:
        vals["K6Phi"] = vals["K6"]
    if test is not None:
        vals["DPhieq"] = 0.0
    vals.update(alpha=flags.alpha, si_alpha=flags.si_alpha, williams_alpha=flags.williams_alpha)
    return vals


def _set_static_params(eng: Engine, vals: Dict[str, Any]) -> None:
    nd = {k: (v.detach() if torch.is_tensor(v) else v) for k, v in vals.items()}
    eng.set_params(0, **nd)


def _init_state_from_fields(*, static: Static, flags: "RunFlags", test: Optional[int], eta0, delta0, Phi0, U0,
                            V0) -> State:
    """Two-level initial state, prev == curr == the given physical fields
    (model.py:694-772): forcing at the initial step, truncated Fourier
    coefficients of the eight fields, the nonlinear terms and the lagged
    momentum-forcing remainder, computed by the library's INIT kernel.  The
    fields are (J, I) or (B, J, I); float32 fields build the state in the
    fast precision."""
    prec = _state_precision(eta0)
    dev = static.mus.device
    rdt = torch.float64 if prec == "fp64" else torch.float32
    f0 = [torch.as_tensor(x, device=dev).to(rdt) for x in (eta0, delta0, Phi0, U0, V0)]
    batched = f0[0].dim() == 3
    B = f0[0].shape[0] if batched else 1
    eng = _engine_for(static.M, B, prec, dev)
    J, I = eng.groups[0]["J"], eng.groups[0]["I"]
    for name, x in zip(("eta0", "delta0", "Phi0", "U0", "V0"), f0):
        if tuple(x.shape[-2:]) != (J, I) or (batched and x.shape != f0[0].shape):
            raise ValueError(f"{name} must have shape {(J, I)} (or (B, J, I)), got {tuple(x.shape)}")
    _set_static_params(eng, _static_values(static, flags, test))
    ics = torch.stack([x if batched else x[None] for x in f0], 0)
    eng.init_state([ics], _flags_c(flags, test, 2, diagnostics=False))
    gd = eng.groups[0]
    four = gd["fourier"]
    td = gd["params"][_lib.P_TAUDRAG]
    inv_td = torch.where(td == -1.0, torch.zeros_like(td), 1.0 / td).to(eng.rdtype)
    Rum = four[_lib.F_F] + four[_lib.F_U] * inv_td[None, :, None]
    Rvm = four[_lib.F_G] + four[_lib.F_V] * inv_td[None, :, None]
    phys = torch.stack([ics[k] for k in (0, 1, 2, 3, 4, 0, 1, 2)], 0)
    st = _assemble_state(eng, phys, Rum, Rvm, batched)
    # physical members are the given fields themselves, as in the reference
    return st._replace(eta_prev=f0[0], eta_curr=f0[0], delta_prev=f0[1], delta_curr=f0[1], Phi_prev=f0[2],
                       Phi_curr=f0[2], U_curr=f0[3], V_curr=f0[4],
                       dead=torch.zeros(st.dead.shape, dtype=torch.bool, device=dev))


def _load_state(eng: Engine, flags: "RunFlags", state0: State, test, t0: int, diag=None) -> int:
    """Put a reference-layout State into the engine; returns the t_start the
    steps must use.

    The Fourier carries are taken as given.  The physical fields enter as the
    synthesis of their truncated Fourier coefficients plus their part beyond
    the truncation, carried as the engine's residual with per-member weights:
    a two-level state (prev == curr, e.g. from _init_state_from_fields) keeps
    the residual on both levels; a stepped state (band-limited curr, e.g. a
    previous run's last_state) keeps the prev level's.  A member whose prev and
    curr levels both carry different content beyond the truncation is refused."""
    gd = eng.groups[0]
    four, resid, member = gd["fourier"], gd["resid"], gd["member"]
    dev, rdt, cdt = eng.device, eng.rdtype, eng.cdtype
    batched = torch.as_tensor(state0.eta_curr).dim() == 3

    def ph(x):
        t = torch.as_tensor(x, device=dev).detach().to(rdt)
        return t if batched else t[None]

    def fo(x):  # (B, J, M+1) -> (M+1, B, J)
        t = torch.as_tensor(x, device=dev).detach().to(cdt)
        return (t if batched else t[None]).permute(2, 0, 1)

    pc = torch.stack([ph(getattr(state0, n)) for n in ("eta_curr", "delta_curr", "Phi_curr", "U_curr", "V_curr")])
    pp = torch.stack([ph(getattr(state0, n)) for n in ("eta_prev", "delta_prev", "Phi_prev")])
    fresh = (pp == pc[:3]).flatten(2).all(dim=2).all(dim=0)  # (B,): prev == curr
    mid = r_p = None
    if not bool(fresh.all()):
        eng.init_state([torch.cat([pp, pc[3:]], 0)], _flags_c(flags, test, t0, diagnostics=False))
        mid = four[[_lib.F_ETA, _lib.F_DELTA, _lib.F_PHI]].clone()
        r_p = resid[:3].clone()
    eng.init_state([pc], _flags_c(flags, test, t0), diag=diag)
    for name, slot in _STATE_SLOTS:
        four[slot].copy_(fo(getattr(state0, name)))
    filtered = bool(flags.semi_implicit or flags.raw_filter)
    for name, ps, ms in zip(_PREV_NAMES, _PREV_SLOTS, _MID_SLOTS):
        v = fo(getattr(state0, name))
        if filtered:
            four[ms].copy_(v)   # the Fourier prev carry is the filtered lineage
            four[ps].copy_(v)
        else:
            four[ps].copy_(v)
            if mid is not None:
                four[ms].copy_(mid[_MID_SLOTS.index(ms)])
    if flags.semi_implicit:  # the lagged remainders live in the unfiltered prev slots
        four[_lib.F_RU_LAG].copy_(fo(state0.Rum_lag))
        four[_lib.F_RV_LAG].copy_(fo(state0.Rvm_lag))
    stepped = torch.zeros_like(fresh)
    if r_p is not None:
        tol = 1e-9 if eng.precision == "fp64" else 1e-5
        scale = pc.abs().flatten(2).amax(dim=2).clamp_min(1e-300)[..., None, None]  # (5, B, 1, 1)
        r_c = resid.clone()
        rc_small = ((r_c.abs() <= tol * scale).flatten(2).all(dim=2)).all(dim=0)
        same = ((r_p - r_c[:3]).abs() <= tol * scale[:3]).flatten(2).all(dim=2).all(dim=0)
        stepped = ~fresh & rc_small
        bad = ~fresh & ~stepped & ~same
        if bool(bad.any()):
            raise NotImplementedError(
                "state0 members " + str(torch.nonzero(bad).flatten().tolist()) + " carry different content beyond "
                "the truncation on their prev and curr levels; only two-level states (prev == curr) and stepped "
                "states (band-limited curr) are supported")
        sel = stepped[None, :, None, None]
        resid[:3].copy_(torch.where(sel, r_p, r_c[:3]))
        w1 = torch.ones_like(member[_lib.MS_WCURR])
        member[_lib.MS_WCURR].copy_(torch.where(stepped, torch.zeros_like(w1), w1))
        member[_lib.MS_WMID].copy_(w1)
        member[_lib.MS_UPDATED].copy_(stepped.to(member.dtype))
    dead = torch.as_tensor(state0.dead, device=dev).reshape(-1).to(member.dtype)
    member[_lib.MS_DEAD].copy_(dead.expand(member.shape[1]))
    # stepped members advance by increments from the first step (fast precision);
    # the semi-implicit scheme takes its lagged remainders from the state
    return t0 - 1 if (flags.semi_implicit or bool(stepped.all())) else t0


def _t_window(t_seq):
    t = torch.as_tensor(t_seq).reshape(-1).to("cpu", torch.int64)
    n = int(t.numel())
    if n and not torch.equal(t, torch.arange(int(t[0]), int(t[0]) + n)):
        raise ValueError("t_seq must be consecutive time indices (arange(t0, t0 + n))")
    return (int(t[0]) if n else 2), n


def _uv_matches_state(Uic, Vic, state0) -> bool:
    return all(x is None or torch.equal(torch.as_tensor(x).to(torch.as_tensor(y).device, torch.as_tensor(y).dtype),
                                        torch.as_tensor(y))
               for x, y in ((Uic, state0.U_curr), (Vic, state0.V_curr)))


def _scan_checks(static: Static, flags: "RunFlags", state0: State, test, Uic, Vic):
    if test not in (None, 1, 2):
        raise NotImplementedError(f"test={test} is not implemented (use None, 1 or 2)")
    if flags.semi_implicit and flags.expflag:
        raise ValueError("semi_implicit=True is incompatible with expflag=True (pick one scheme).")
    if flags.raw_filter and flags.expflag:
        raise ValueError("raw_filter=True is incompatible with expflag=True.")
    if test == 1 and not _uv_matches_state(Uic, Vic, state0):
        raise NotImplementedError("test=1 pins the winds to the state's own U_curr, V_curr: Uic, Vic must equal them")


def _run_loaded(static: Static, flags: "RunFlags", state0: State, test, t0: int, n: int, hist: bool):
    """Load state0, step n times from t0; returns (engine, physical outputs,
    diagnostics rows or None, history or None, batched)."""
    prec = _state_precision(state0.etam_curr)
    batched = torch.as_tensor(state0.eta_curr).dim() == 3
    B = torch.as_tensor(state0.eta_curr).shape[0] if batched else 1
    dev = static.mus.device
    eng = _engine_for(static.M, B, prec, dev)
    _set_static_params(eng, _static_values(static, flags, test))
    diag = eng.new_diag(n) if flags.diagnostics else None
    t_start = _load_state(eng, flags, state0, test, t0, diag=diag)
    fc = _flags_c(flags, test, t_start)
    gd = eng.groups[0]
    h = [torch.empty((n, 5, B, gd["J"], gd["I"]), dtype=eng.rdtype, device=eng.device)] if hist else None
    if n > 0:
        eng.forward(fc, t0=t0, nsteps=n, row0=0, diag=diag, hist=h, write_prev_last=True)
    phys = eng.output_physical(fc)[0]
    eng.check_device_status()
    return eng, fc, phys, diag, h, batched


def _state_after(eng: Engine, flags: "RunFlags", phys, batched: bool, state0: State) -> State:
    four = eng.groups[0]["fourier"]
    if flags.semi_implicit:
        Rum, Rvm = four[_lib.F_RU_LAG], four[_lib.F_RV_LAG]
        st = _assemble_state(eng, phys, Rum, Rvm, batched, filtered_prev=True)
    else:  # pass-through carries (model.py:1144-1145)
        st = _assemble_state(eng, phys, four[_lib.F_F], four[_lib.F_G], batched,
                             filtered_prev=bool(flags.raw_filter))
        st = st._replace(Rum_lag=state0.Rum_lag, Rvm_lag=state0.Rvm_lag)
    return st


class _ScanLastFn(torch.autograd.Function):
    """Derivatives of simulate_scan_last's curr fields (eta, delta, Phi, U, V)
    in the Static's scalar parameters, with state0 held fixed (as the
    retrieval's fast path does: its state0 is built once from the base
    parameters).  Forward mode: the tangent-linear model from a zero initial
    tangent.  Reverse mode: one tangent run per parameter that needs a
    gradient (members are independent: one run serves every member)."""

    @staticmethod
    def forward(ctx, ctl, *params):
        ctx.ctl = ctl
        ctx.save_for_forward(*params)
        ctx.save_for_backward(*params)
        return ctl["out"]

    @staticmethod
    def _tangent(ctx, dpar_rows):
        ctl = ctx.ctl
        eng, flags, state0, test, t0, n = ctl["eng"], ctl["flags"], ctl["state0"], ctl["test"], ctl["t0"], ctl["n"]
        _set_static_params(eng, ctl["vals"])
        t_start = _load_state(eng, flags, state0, test, t0)
        fc = _flags_c(flags, test, t_start, diagnostics=False)
        tfour, tresid, _ = eng.new_tangent_buffers()
        eng.tangent_forward(fc, t0, n, tfour, tresid, [dpar_rows])
        out = eng.tangent_output(fc, tfour, tresid, [dpar_rows])[0][:5]
        eng.check_device_status()
        return out

    @staticmethod
    def jvp(ctx, _ctl_t, *params_t):
        B = ctx.ctl["B"]
        dev = ctx.ctl["eng"].device
        rows = torch.zeros((_lib.NTANGENT, B), dtype=torch.float64, device=dev)
        for k, t in enumerate(params_t):
            if t is not None:
                rows[k] = torch.as_tensor(t, device=dev).to(torch.float64).expand(B)
        out = _ScanLastFn._tangent(ctx, rows)
        return out.to(ctx.ctl["out"].dtype)

    @staticmethod
    def backward(ctx, gout):
        B = ctx.ctl["B"]
        dev = ctx.ctl["eng"].device
        params = ctx.saved_tensors
        res = [None] * (1 + len(params))
        w = gout.to(torch.float64)
        for k in range(len(params)):
            if not ctx.needs_input_grad[1 + k]:
                continue
            rows = torch.zeros((_lib.NTANGENT, B), dtype=torch.float64, device=dev)
            rows[k] = 1.0
            jk = _ScanLastFn._tangent(ctx, rows).to(torch.float64)
            g = (w * jk).sum(dim=(0, 2, 3))
            res[1 + k] = g.sum().reshape(params[k].shape).to(params[k].dtype) if params[k].dim() == 0 else \
                g.reshape(params[k].shape).to(params[k].dtype)
        return tuple(res)


def simulate_scan_last(*, static: Static, flags: "RunFlags", state0: State, t_seq, test: Optional[int], Uic, Vic,
                       remat_step: bool = False) -> State:
    """Advance state0 along t_seq without a time history (model.py:1281-1342);
    returns the final State.  ``remat_step`` is accepted for compatibility (the
    kernels keep no per-step residuals).  float32 state fields select the fast
    precision.  The scalar parameters of ``static`` (dt, a, omega, Phibar,
    taurad, taudrag, DPhieq, K6, K6Phi) rebuild the coefficient tables, so a
    ``dataclasses.replace(static, taurad=..., taudrag=...)`` takes effect; as
    tensors that require grad or carry forward-mode tangents they make the
    curr fields of the result differentiable, with state0 held fixed."""
    _scan_checks(static, flags, state0, test, Uic, Vic)
    t0, n = _t_window(t_seq)
    vals = _static_values(static, flags, test)
    eng, fc, phys, _, _, batched = _run_loaded(static, flags, state0, test, t0, n, hist=False)
    st = _state_after(eng, flags, phys, batched, state0)
    tracked = [k for k in _lib.TANGENT_PARAMS if k in vals and _tracked(vals[k])]
    if tracked and n > 0:
        if test == 1:
            raise NotImplementedError("derivatives are implemented for test None or 2")
        B = eng.groups[0]["B"]
        dev = eng.device
        params = [torch.as_tensor(vals[k], dtype=torch.float64, device=dev) if k in vals else
                  torch.zeros((), dtype=torch.float64, device=dev) for k in _lib.TANGENT_PARAMS]
        out = torch.stack([phys[k] for k in range(5)], 0)
        ctl = dict(eng=eng, flags=flags, state0=state0, test=test, t0=t0, n=n, B=B, vals=vals, out=out)
        dcurr = _ScanLastFn.apply(ctl, *params)
        pick = (lambda v: v) if batched else (lambda v: v[0])
        st = st._replace(eta_curr=pick(dcurr[0]), delta_curr=pick(dcurr[1]), Phi_curr=pick(dcurr[2]),
                         U_curr=pick(dcurr[3]), V_curr=pick(dcurr[4]))
    return st


def simulate_scan(*, static: Static, flags: "RunFlags", state0: State, t_seq, test: Optional[int], Uic, Vic):
    """Advance state0 along t_seq keeping the per-step outputs
    (model.py:1237-1278): returns (last_state, outs) with outs["eta" | "delta"
    | "Phi" | "U" | "V"] of shape (T, J, I) (member axis first for ensembles)
    and, with flags.diagnostics, "rms", "spin_min", "phi_min", "phi_max",
    "dead" of shape (T,)."""
    _scan_checks(static, flags, state0, test, Uic, Vic)
    t0, n = _t_window(t_seq)
    eng, fc, phys, diag, h, batched = _run_loaded(static, flags, state0, test, t0, n, hist=True)
    st = _state_after(eng, flags, phys, batched, state0)
    outs: Dict[str, Any] = {}
    for k, name in enumerate(("eta", "delta", "Phi", "U", "V")):
        v = h[0][:, k]
        outs[name] = v.permute(1, 0, 2, 3) if batched else v[:, 0]
    B = eng.groups[0]["B"]
    if diag is not None:
        d = diag[0][:n]
        vals = dict(rms=torch.sqrt(d[:, _lib.D_RMS2]), spin_min=d[:, _lib.D_SPIN], phi_min=d[:, _lib.D_PHIMIN],
                    phi_max=d[:, _lib.D_PHIMAX], dead=d[:, _lib.D_DEAD] != 0)
    else:
        z = torch.zeros((n, B), dtype=torch.float64, device=eng.device)
        vals = dict(rms=z, spin_min=z, phi_min=z, phi_max=z, dead=torch.zeros((n, B), dtype=torch.bool,
                                                                                device=eng.device))
    for k, v in vals.items():
        outs[k] = v.t() if batched else v[:, 0]
    return st, outs


def _step_once_state_only(state: State, t, static: Static, flags: "RunFlags", test: Optional[int], Uic, Vic) -> State:
    """One step returning only the new State (model.py:1197-1235)."""
    t = int(torch.as_tensor(t).reshape(()).item())
    return simulate_scan_last(static=static, flags=flags, state0=state, t_seq=[t], test=test, Uic=Uic, Vic=Vic)


def run_model_scan_final(
    *, M: int, dt, tmax: int, Phibar, omega, a, test: Optional[int] = None, g=9.8, forcflag: bool = True,
    taurad=86400.0, taudrag=86400.0, DPhieq=4 * (10**6), a1=0.05, diffflag: bool = True, modalflag: bool = True,
    alpha=0.01, expflag: bool = False, K6=1.24 * (10**33), K6Phi=None, contflag: bool = False,
    custompath: Optional[str] = None, contTime=None, timeunits: str = "hours", starttime: Optional[int] = None,
    eta0_init=None, delta0_init=None, Phi0_init=None, U0_init=None, V0_init=None,
    semi_implicit: bool = False, si_alpha=0.5, raw_filter: bool = False, williams_alpha=0.53,
    diagnostics: bool = False, remat_step: bool = False, jit_scan: bool = True, donate_state: bool = False,
    precision: str = "fp64", device=None,
) -> Dict[str, Any]:
    """``model.py:1844-1951``: terminal state only (``static``, ``t_seq``,
    ``last_state``, ``starttime``); the same keywords as :func:`run_model_scan`
    without ``return_history``, diagnostics off by default."""
    return run_model_scan(
        M=M, dt=dt, tmax=tmax, Phibar=Phibar, omega=omega, a=a, test=test, g=g, forcflag=forcflag, taurad=taurad,
        taudrag=taudrag, DPhieq=DPhieq, a1=a1, diffflag=diffflag, modalflag=modalflag, alpha=alpha, expflag=expflag,
        K6=K6, K6Phi=K6Phi, contflag=contflag, custompath=custompath, contTime=contTime, timeunits=timeunits,
        starttime=starttime, eta0_init=eta0_init, delta0_init=delta0_init, Phi0_init=Phi0_init, U0_init=U0_init,
        V0_init=V0_init, semi_implicit=semi_implicit, si_alpha=si_alpha, raw_filter=raw_filter,
        williams_alpha=williams_alpha, diagnostics=diagnostics, return_history=False, remat_step=remat_step,
        jit_scan=jit_scan, donate_state=donate_state, precision=precision, device=device)


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
