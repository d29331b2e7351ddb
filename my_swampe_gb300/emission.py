"""The retrieval's emission stage on the GPU, batched over ensemble members.

The reference builds it inside its retrieval pipeline
(``retrieval/scripts/pipeline.py:690-1000``): the terminal Phi of a run goes to
a temperature map, an emission (intensity) map, the spherical-harmonic
coefficients of that map (a weighted ridge least-squares projection, normalised
by the first coefficient), and the planet's phase curve, which is linear in
those coefficients.  This module keeps the reference's function names and
configuration field names; every function takes one field (J, I) or an
ensemble (B, J, I) and runs hand-written FP64 CUDA kernels
(``csrc/emission.cu``), FP64 like the reference's emission stage.

Two matrices come from the third-party spherical-harmonic model the reference
uses (jaxoplanet 0.1.0, ``starry`` ``Surface.intensity`` and ``light_curve``),
which the caller evaluates once per retrieval, as the reference does:

* the Ylm design matrix ``design`` (n_pix, n_coeff), the intensity of each unit
  coefficient vector at the model's pixels, from which :func:`build_projector`
  forms the projector (``pipeline.py:808-819``);
* the light-curve design matrix (n_times, n_coeff), the planet's flux at each
  observation time for each unit coefficient vector at amplitude 1, which
  :func:`phase_curve` multiplies (``pipeline.py:983-994``).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Optional, Sequence, Tuple

import numpy as np
import torch

from . import _lib

__all__ = ["EmissionConfig", "phi_to_temperature", "temperature_to_intensity", "build_projector",
           "intensity_map_to_y_dense", "emission_coefficients", "phase_curve", "simple_phase_curve"]


@dataclass
class EmissionConfig:
    """The emission fields of the reference's pipeline config (``pipeline.py:160-188``)."""

    emission_temp_mode: str = "geopotential"  # T = (Phibar + Phi) / R_d, or "linear": T_ref + Phi / phi_to_T_scale
    R_d: float = 3.78e3
    T_ref: float = 1000.0
    phi_to_T_scale: float = 600.0
    Tmin_K: float = 1.0
    emission_model: str = "bolometric"  # T^4, or "planck"
    planck_wavelength_m: float = 4.5e-6
    planck_x_clip: float = 80.0
    planck_band_wavelengths_m: Optional[Sequence[float]] = None
    planck_band_weights: Optional[Sequence[float]] = None

    def c(self) -> _lib.EmissionCfg:
        """The C struct, with the checks of the reference's validate_config (``pipeline.py:344-409``)."""
        mode = str(self.emission_temp_mode).strip().lower()
        model = str(self.emission_model).strip().lower()
        if mode not in ("geopotential", "linear"):
            raise ValueError(f"emission_temp_mode must be 'geopotential' or 'linear', got {self.emission_temp_mode!r}")
        if model not in ("bolometric", "planck"):
            raise ValueError(f"Unknown emission_model={self.emission_model!r}.")
        if not float(self.Tmin_K) > 0.0:
            raise ValueError(f"Tmin_K must be > 0, got {self.Tmin_K!r}")
        if (self.planck_band_wavelengths_m is None) != (self.planck_band_weights is None):
            raise ValueError("planck_band_wavelengths_m and planck_band_weights must be set together.")
        if self.planck_band_wavelengths_m is not None:
            if model != "planck":
                raise ValueError("planck_band_* requires emission_model='planck'.")
            wl = np.asarray(self.planck_band_wavelengths_m, dtype=np.float64).reshape(-1)
            w = np.asarray(self.planck_band_weights, dtype=np.float64).reshape(-1)
            if wl.size == 0 or wl.size != w.size:
                raise ValueError("planck_band_wavelengths_m and planck_band_weights must be equal-length and non-empty.")
            if wl.size > _lib.EMISSION_MAX_BANDS:
                raise ValueError(f"at most {_lib.EMISSION_MAX_BANDS} Planck bands")
            if not (np.all(np.isfinite(wl)) and np.all(wl > 0)):
                raise ValueError("planck_band_wavelengths_m must be finite and positive (meters).")
            if not (np.all(np.isfinite(w)) and np.all(w > 0.0)):
                raise ValueError("planck_band_weights must be finite and positive.")
            w = w / np.sum(w)
        else:
            wl = np.asarray([self.planck_wavelength_m], dtype=np.float64)
            w = np.ones(1)
        c = _lib.EmissionCfg()
        c.temp_mode = 0 if mode == "geopotential" else 1
        c.R_d, c.T_ref, c.phi_to_T_scale, c.Tmin = (float(self.R_d), float(self.T_ref), float(self.phi_to_T_scale),
                                                    float(self.Tmin_K))
        c.model = 0 if model == "bolometric" else 1
        c.nbands = int(wl.size)
        for k in range(wl.size):
            c.wavelengths[k] = float(wl[k])
            c.band_weights[k] = float(w[k])
        c.x_clip = float(self.planck_x_clip)
        return c


def _ensemble(x, name: str) -> Tuple[torch.Tensor, bool]:
    t = torch.as_tensor(x)
    if t.dim() not in (2, 3):
        raise ValueError(f"{name} must be (J, I) or (B, J, I), got shape {tuple(t.shape)}")
    if not torch.cuda.is_available():
        raise RuntimeError("my_swampe_gb300.emission needs a CUDA GPU: there is no CPU fallback")
    dev = t.device if t.is_cuda else torch.device("cuda", torch.cuda.current_device())
    batched = t.dim() == 3
    t = t.to(device=dev, dtype=torch.float64)
    return (t if batched else t[None]).contiguous(), batched


def _per_member(x, B: int, dev) -> torch.Tensor:
    return torch.as_tensor(x, dtype=torch.float64, device=dev).reshape(-1).expand(B).contiguous()


def _stream(dev) -> int:
    return torch.cuda.current_stream(dev).cuda_stream


def _check(rc: int, what: str) -> None:
    if rc != _lib.SWP_OK:
        raise RuntimeError(f"libswampe_gb300 {what} failed ({_lib.ERRORS.get(rc, rc)})")


def _map(x, Phibar, cfg: EmissionConfig, input_kind: int, stage: int, w_lat=None):
    xs, batched = _ensemble(x, "field")
    B, J, I = xs.shape
    dev = xs.device
    pb = _per_member(0.0 if Phibar is None else Phibar, B, dev)
    w = None if w_lat is None else torch.as_tensor(w_lat, dtype=torch.float64, device=dev).reshape(-1).contiguous()
    if w is not None and w.numel() != J:
        raise ValueError(f"w_lat must have {J} latitude weights, got {w.numel()}")
    out = torch.empty_like(xs)
    ok = torch.zeros(B, dtype=torch.int32, device=dev)
    c = cfg.c()
    _check(_lib.load().swp_emission_map(xs.data_ptr(), pb.data_ptr(), B, J, I, None if w is None else w.data_ptr(),
                                        ctypes.byref(c), input_kind, stage, out.data_ptr(), ok.data_ptr(),
                                        _stream(dev)), "swp_emission_map")
    return out, ok, batched


def phi_to_temperature(phi, Phibar, cfg: EmissionConfig = EmissionConfig()) -> torch.Tensor:
    """T = max((Phibar + Phi) / R_d, Tmin) (geopotential mode; Phibar per member,
    the value the dynamics ran with) or max(T_ref + Phi / phi_to_T_scale, Tmin)
    (linear); all NaN for a member whose Phi is not finite (``pipeline.py:696-714``)."""
    out, _, batched = _map(phi, Phibar, cfg, 0, 0)
    return out if batched else out[0]


def temperature_to_intensity(T, cfg: EmissionConfig = EmissionConfig()) -> torch.Tensor:
    """T^4 (bolometric) or the relative Planck intensity 1 / (expm1(x) + 1e-30),
    band-averaged with the normalised band weights (``pipeline.py:716-754``)."""
    out, _, batched = _map(T, None, cfg, 1, 1)
    return out if batched else out[0]


def build_projector(design, w_lat, ridge: float = 1.0e-6) -> torch.Tensor:
    """Projector (n_coeff, n_pix) = (Bw^T Bw + ridge I)^-1 Bw^T with Bw = sqrt(w)
    design, w the latitude weights repeated over longitude (``pipeline.py:808-819``;
    set-up, once per retrieval).  design: (n_pix, n_coeff), latitude-major pixels."""
    Bm = torch.as_tensor(design, dtype=torch.float64)
    w = torch.as_tensor(w_lat, dtype=torch.float64, device=Bm.device).reshape(-1)
    npix, ncoef = Bm.shape
    if npix % w.numel():
        raise ValueError("design rows must be latitude-major pixels of the weights' grid")
    if not bool(torch.isfinite(Bm).all()):
        raise RuntimeError("Design matrix B contains NaNs/Infs.")
    if not bool(torch.isfinite(w).all()) or bool((w < 0).any()):
        raise RuntimeError("latitude weights must be finite and non-negative")
    w_sqrt = torch.sqrt(w.repeat_interleave(npix // w.numel()))
    Bw = w_sqrt[:, None] * Bm
    gram = Bw.T @ Bw + float(ridge) * torch.eye(ncoef, dtype=torch.float64, device=Bm.device)
    P = torch.linalg.solve(gram, Bw.T)
    if not bool(torch.isfinite(P).all()):
        raise RuntimeError("Projector contains NaNs/Infs.")
    return P


def _project(rhs: torch.Tensor, ok: torch.Tensor, projector) -> torch.Tensor:
    B, J, I = rhs.shape
    P = torch.as_tensor(projector, dtype=torch.float64, device=rhs.device).contiguous()
    if P.dim() != 2 or P.shape[1] != J * I:
        raise ValueError(f"projector must be (n_coeff, {J * I}), got {tuple(P.shape)}")
    y = torch.empty((B, P.shape[0]), dtype=torch.float64, device=rhs.device)
    _check(_lib.load().swp_emission_project(rhs.data_ptr(), ok.data_ptr(), B, J * I, P.data_ptr(), P.shape[0],
                                            y.data_ptr(), _stream(rhs.device)), "swp_emission_project")
    return y


def intensity_map_to_y_dense(I_map, projector, w_lat) -> torch.Tensor:
    """Coefficients of an intensity map (``pipeline.py:821-846``): the map over its
    w-weighted mean, times sqrt(w), through the projector, divided by the first
    coefficient; all NaN when the map, its mean or y0 fails the reference's guards."""
    rhs, ok, batched = _map(I_map, None, EmissionConfig(), 2, 2, w_lat)
    y = _project(rhs, ok, projector)
    return y if batched else y[0]


def emission_coefficients(phi, Phibar, projector, w_lat, cfg: EmissionConfig = EmissionConfig()) -> torch.Tensor:
    """phi_to_temperature, temperature_to_intensity and intensity_map_to_y_dense
    in one pass per member: the map coefficients (B, n_coeff) of each member's
    terminal Phi."""
    rhs, ok, batched = _map(phi, Phibar, cfg, 0, 2, w_lat)
    y = _project(rhs, ok, projector)
    return y if batched else y[0]


def phase_curve(y, design_lc, amplitude=1.0) -> torch.Tensor:
    """The planet's flux at the observation times, amplitude (planet_fpfs, per
    member) times design_lc (n_times, n_coeff) . y (``pipeline.py:983-994``)."""
    yv = torch.as_tensor(y, dtype=torch.float64)
    batched = yv.dim() == 2
    yv = (yv if batched else yv[None]).to("cuda" if not yv.is_cuda else yv.device).contiguous()
    B, ncoef = yv.shape
    A = torch.as_tensor(design_lc, dtype=torch.float64, device=yv.device).contiguous()
    if A.dim() != 2 or A.shape[1] != ncoef:
        raise ValueError(f"design_lc must be (n_times, {ncoef}), got {tuple(A.shape)}")
    amp = _per_member(amplitude, B, yv.device)
    lc = torch.empty((B, A.shape[0]), dtype=torch.float64, device=yv.device)
    _check(_lib.load().swp_phase_curve_linear(yv.data_ptr(), A.data_ptr(), amp.data_ptr(), B, ncoef, A.shape[0],
                                              lc.data_ptr(), _stream(yv.device)), "swp_phase_curve_linear")
    return lc if batched else lc[0]


def simple_phase_curve(phi, phase_angles, mus=None) -> torch.Tensor:
    """The simplified phase-curve projection of the reference's parity test
    (``unit_tests/test_parity_reference_regression.py:67-82``): per phase, the
    sum of Phi times the visible cosine max(cos(lambda - phase), 0) and
    sqrt(1 - mu^2), over mean |flux|.  mus defaults to the Gauss-Legendre nodes
    of the grid (numpy's leggauss, as the test)."""
    xs, batched = _ensemble(phi, "phi")
    B, J, I = xs.shape
    dev = xs.device
    mu = np.polynomial.legendre.leggauss(J)[0] if mus is None else mus
    mu = torch.as_tensor(mu, dtype=torch.float64, device=dev).reshape(-1).contiguous()
    ph = torch.as_tensor(phase_angles, dtype=torch.float64, device=dev).reshape(-1).contiguous()
    if mu.numel() != J:
        raise ValueError(f"mus must have {J} values")
    out = torch.empty((B, ph.numel()), dtype=torch.float64, device=dev)
    _check(_lib.load().swp_phase_curve_simple(xs.data_ptr(), B, J, I, mu.data_ptr(), ph.data_ptr(), ph.numel(),
                                              out.data_ptr(), _stream(dev)), "swp_phase_curve_simple")
    return out if batched else out[0]
