"""CPU FP64 oracle for the emission stage of the retrieval.

TEST INFRASTRUCTURE ONLY.  This module is an oracle: it may be imported by
``tests/`` and by ``__graft_entry__.smoke()``.  The GPU product path
(``my_swampe_gb300.emission``) never imports it.

It restates, in numpy float64, the reference's emission stage for one member
(one (J, I) field), with the reference's guards; paths are relative to the
reference project root:

* ``phi_to_temperature``          retrieval/scripts/pipeline.py:696-714
* ``planck_intensity_relative``   pipeline.py:716-735
* ``temperature_to_intensity``    pipeline.py:743-754
* ``build_projector``             pipeline.py:808-819
* ``intensity_map_to_y_dense``    pipeline.py:821-846
* ``phase_curve``                 pipeline.py:983-994 (the planet's flux is
  linear in the map coefficients with amplitude planet_fpfs; the light-curve
  design matrix is an input)
* ``simple_phase_curve``          unit_tests/test_parity_reference_regression.py:67-82

The Ylm and light-curve design matrices come from jaxoplanet 0.1.0 (starry
``Surface.intensity`` / ``light_curve``), which is not part of the reference
tree and is not installed here; tests give both sides the same matrices.
"""
from __future__ import annotations

import numpy as np

H_PLANCK = 6.62607015e-34
C_LIGHT = 299792458.0
K_BOLTZMANN = 1.380649e-23


def phi_to_temperature(phi, Phibar, *, temp_mode="geopotential", R_d=3.78e3, T_ref=1000.0, phi_to_T_scale=600.0,
                       Tmin_K=1.0):
    phi = np.asarray(phi, dtype=np.float64)
    if not np.all(np.isfinite(phi)):
        return np.full_like(phi, np.nan)
    if temp_mode == "geopotential":
        T = (Phibar + phi) / R_d
    else:
        T = T_ref + phi / phi_to_T_scale
    return np.maximum(T, Tmin_K)


def planck_intensity_relative(T, wavelength_m, x_clip=80.0):
    T = np.asarray(T, dtype=np.float64)
    if not np.all(np.isfinite(T)):
        return np.full_like(T, np.nan)
    x = (H_PLANCK * C_LIGHT) / (wavelength_m * K_BOLTZMANN * T)
    x = np.clip(x, 0.0, x_clip)
    return 1.0 / (np.expm1(x) + 1.0e-30)


def temperature_to_intensity(T, *, emission_model="bolometric", planck_wavelength_m=4.5e-6, planck_x_clip=80.0,
                             planck_band_wavelengths_m=None, planck_band_weights=None):
    T = np.asarray(T, dtype=np.float64)
    if emission_model == "bolometric":
        return T ** 4
    if planck_band_wavelengths_m is not None:
        w = np.asarray(planck_band_weights, dtype=np.float64)
        w = w / np.sum(w)
        out = np.zeros_like(T)
        for wgt, lam in zip(w, planck_band_wavelengths_m):
            out = out + wgt * planck_intensity_relative(T, lam, planck_x_clip)
        return out
    return planck_intensity_relative(T, planck_wavelength_m, planck_x_clip)


def build_projector(design, w_lat, ridge=1.0e-6):
    design = np.asarray(design, dtype=np.float64)
    npix, ncoef = design.shape
    w_pix = np.repeat(np.asarray(w_lat, dtype=np.float64), npix // len(w_lat))
    Bw = np.sqrt(w_pix)[:, None] * design
    gram = Bw.T @ Bw + ridge * np.eye(ncoef)
    return np.linalg.solve(gram, Bw.T)


def intensity_map_to_y_dense(I_map, projector, w_lat):
    I_flat = np.asarray(I_map, dtype=np.float64).reshape(-1)
    w_pix = np.repeat(np.asarray(w_lat, dtype=np.float64), I_flat.size // len(w_lat))
    finite = np.isfinite(I_flat)
    all_finite_in = bool(np.all(finite))
    w_eff = w_pix * finite
    w_sum = np.sum(w_eff)
    I_safe = np.where(finite, I_flat, 0.0)
    I_mean = np.sum(w_eff * I_safe) / w_sum if w_sum > 0.0 else np.nan
    eps = 1.0e-30
    mean_ok = bool(np.isfinite(I_mean) and abs(I_mean) > eps)
    I_rel = I_safe / I_mean if mean_ok else np.full_like(I_safe, np.nan)
    y = np.asarray(projector, dtype=np.float64) @ (np.sqrt(w_pix) * I_rel)
    y0 = y[0]
    y0_ok = bool(np.isfinite(y0) and abs(y0) > eps)
    y = y / y0 if y0_ok else np.full_like(y, np.nan)
    if not (all_finite_in and mean_ok and y0_ok and np.all(np.isfinite(y))):
        return np.full_like(y, np.nan)
    return y


def phase_curve(y, design_lc, amplitude=1.0):
    return amplitude * (np.asarray(design_lc, dtype=np.float64) @ np.asarray(y, dtype=np.float64))


def simple_phase_curve(phi, phase_angles, mus=None):
    phi = np.asarray(phi, dtype=np.float64)
    J, I = phi.shape
    lambdas = np.linspace(-np.pi, np.pi, I, endpoint=False)[None, :]
    mu = np.polynomial.legendre.leggauss(J)[0] if mus is None else np.asarray(mus, dtype=np.float64)
    area_weight = np.sqrt(np.clip(1.0 - mu[:, None] ** 2, 0.0, None))
    flux = np.empty(len(phase_angles), dtype=np.float64)
    for k, phase in enumerate(phase_angles):
        visible = np.maximum(np.cos(lambdas - phase), 0.0)
        flux[k] = float(np.sum(phi * visible * area_weight))
    norm = np.mean(np.abs(flux))
    if norm > 0:
        flux = flux / norm
    return flux


def real_ylm_design(ydeg, lat, lon):
    """A real spherical-harmonic basis (associated Legendre functions of
    sin(lat) times cos(m lon) / sin(|m| lon), scaled to unit RMS over the
    pixels, in the (l, m) order
    of the reference's lm_list, pipeline.py:783) at the pixels: a stand-in
    design matrix for tests.  It is not starry's normalisation or orientation,
    which the tests do not need: both sides are given the same matrix."""
    from scipy.special import lpmv

    x = np.sin(np.asarray(lat, dtype=np.float64))
    lon = np.asarray(lon, dtype=np.float64)
    cols = []
    for ell in range(ydeg + 1):
        for m in range(-ell, ell + 1):
            v = lpmv(abs(m), ell, x) * (np.cos(m * lon) if m >= 0 else np.sin(-m * lon))
            cols.append(v / np.sqrt(np.mean(v * v)))  # unit RMS columns
    return np.stack(cols, axis=1)
