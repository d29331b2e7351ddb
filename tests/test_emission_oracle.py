"""The emission-stage oracle against the reference's own tests and golden
vectors, and the emission C ABI's argument checks (no GPU needed).

Pinned: the simplified phase curve of the reference's parity test reproduces
the fixtures' phase_curve from their final Phi
(unit_tests/test_parity_reference_regression.py:67-82, 136-148).  The
temperature, intensity and projection restatements follow
retrieval/scripts/pipeline.py:696-846 and are checked by the properties the
reference's pipeline tests assert (retrieval/scripts/tests/test_pipeline.py:
88-110, 148-155, 301-308)."""
import ctypes

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import emission_oracle as eo

FIXTURES = ("reference_case_forced_default.npz", "reference_case_unforced_test1.npz")


def _grid(J=64, I=128):
    mu, w = np.polynomial.legendre.leggauss(J)
    lat = np.repeat(np.arcsin(mu), I)
    lon = np.tile(np.linspace(-np.pi, np.pi, I, endpoint=False), J)
    return mu, w, lat, lon


@pytest.mark.parametrize("name", FIXTURES)
def test_simple_phase_curve_reproduces_the_fixture(name):
    ref = np.load(GOLDEN / name)
    got = eo.simple_phase_curve(ref["final_Phi"], ref["phase_angles"])
    np.testing.assert_allclose(got, ref["phase_curve"], rtol=0, atol=1e-10)


def test_geopotential_temperature_is_phibar_over_R_d():
    """test_pipeline.py:301-308: Phi = 0 gives T = Phibar / R_d."""
    T = eo.phi_to_temperature(np.zeros((64, 128)), 3.0e5, R_d=3.78e3)
    np.testing.assert_allclose(T, 3.0e5 / 3.78e3, rtol=1e-14)
    T = eo.phi_to_temperature(np.full((4, 4), -1e9), 3.0e5)
    assert np.all(T == 1.0)  # the Tmin floor


def test_nan_guards():
    """test_pipeline.py:148-155: NaN in -> all NaN out."""
    bad = np.full((64, 128), np.nan)
    assert np.all(np.isnan(eo.phi_to_temperature(bad, 3e5)))
    _, w, lat, lon = _grid()
    P = eo.build_projector(eo.real_ylm_design(4, lat, lon), w)
    assert np.all(np.isnan(eo.intensity_map_to_y_dense(bad, P, w)))
    one_bad = np.ones((64, 128))
    one_bad[3, 5] = np.inf
    assert np.all(np.isnan(eo.intensity_map_to_y_dense(one_bad, P, w)))
    assert np.all(np.isnan(eo.planck_intensity_relative(np.array([1.0, np.nan]), 4.5e-6)))


def test_projector_is_left_inverse_of_weighted_design():
    """test_pipeline.py:88-94."""
    _, w, lat, lon = _grid()
    D = eo.real_ylm_design(10, lat, lon)
    P = eo.build_projector(D, w)
    Bw = np.sqrt(np.repeat(w, 128))[:, None] * D
    assert np.max(np.abs(P @ Bw - np.eye(D.shape[1]))) < 1e-2


def test_intensity_roundtrip_low_order():
    """test_pipeline.py:97-110: a map built from a known low-order y comes back."""
    _, w, lat, lon = _grid()
    D = eo.real_ylm_design(10, lat, lon)
    P = eo.build_projector(D, w)
    rng = np.random.default_rng(0)
    y_true = np.zeros(D.shape[1])
    y_true[0] = 1.0
    y_true[1:6] = 0.05 * rng.standard_normal(5)
    y_rec = eo.intensity_map_to_y_dense((D @ y_true).reshape(64, 128), P, w)
    assert abs(y_rec[0] - 1.0) < 1e-4
    assert np.corrcoef(y_true[1:6], y_rec[1:6])[0, 1] > 0.99


def test_planck_band_average_is_weighted_mean_of_bands():
    T = np.linspace(800.0, 2500.0, 17)
    one = eo.temperature_to_intensity(T, emission_model="planck", planck_wavelength_m=4.5e-6)
    band = eo.temperature_to_intensity(T, emission_model="planck", planck_band_wavelengths_m=[3.6e-6, 4.5e-6],
                                       planck_band_weights=[1.0, 3.0])
    np.testing.assert_allclose(band, 0.25 * eo.planck_intensity_relative(T, 3.6e-6) + 0.75 * one, rtol=1e-14)


def test_emission_config_validation():
    from my_swampe_gb300.emission import EmissionConfig

    EmissionConfig().c()
    c = EmissionConfig(emission_model="planck", planck_band_wavelengths_m=[3.6e-6, 4.5e-6],
                       planck_band_weights=[1.0, 3.0]).c()
    assert c.nbands == 2 and abs(c.band_weights[0] - 0.25) < 1e-15
    for bad in (dict(emission_temp_mode="x"), dict(emission_model="x"), dict(Tmin_K=0.0),
                dict(planck_band_wavelengths_m=[4e-6]),
                dict(emission_model="planck", planck_band_wavelengths_m=[4e-6], planck_band_weights=[0.0]),
                dict(emission_model="planck", planck_band_wavelengths_m=[-4e-6], planck_band_weights=[1.0]),
                dict(planck_band_wavelengths_m=[4e-6], planck_band_weights=[1.0])):
        with pytest.raises(ValueError):
            EmissionConfig(**bad).c()


def test_emission_entries_refuse_bad_arguments_without_gpu():
    from my_swampe_gb300 import _lib
    from my_swampe_gb300.emission import EmissionConfig

    lib = _lib.load()
    c = EmissionConfig().c()
    one = ctypes.c_void_p(16)  # never dereferenced: the checks fail first
    assert lib.swp_emission_map(None, one, 1, 4, 4, one, ctypes.byref(c), 0, 2, one, None, None) == 1
    assert lib.swp_emission_map(one, one, 0, 4, 4, one, ctypes.byref(c), 0, 2, one, None, None) == 1
    assert lib.swp_emission_map(one, one, 1, 4, 4, one, ctypes.byref(c), 2, 1, one, None, None) == 1
    assert lib.swp_emission_map(one, one, 1, 4, 4, None, ctypes.byref(c), 0, 2, one, None, None) == 1
    assert lib.swp_emission_project(one, None, 1, 16, None, 4, one, None) == 1
    assert lib.swp_phase_curve_linear(one, one, None, 1, 0, 3, one, None) == 1
    assert lib.swp_phase_curve_simple(one, 1, 4, 4, None, one, 3, one, None) == 1
