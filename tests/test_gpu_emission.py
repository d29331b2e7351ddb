"""The emission-stage kernels (my_swampe_gb300.emission, csrc/emission.cu)
against the CPU oracle (FP64 on both sides) and the reference fixtures'
golden phase curves.  Tolerances: 1e-12 relative for the maps and the
coefficients (the reductions differ from numpy's only in summation order),
1e-10 absolute for the golden phase curves (the reference test's own)."""
import numpy as np
import pytest
import torch

from conftest import FIXTURE_CASES, GOLDEN
from oracle import emission_oracle as eo

pytestmark = pytest.mark.gpu

FIXTURES = ("reference_case_forced_default.npz", "reference_case_unforced_test1.npz")
J, I = 64, 128


def _grid():
    mu, w = np.polynomial.legendre.leggauss(J)
    lat = np.repeat(np.arcsin(mu), I)
    lon = np.tile(np.linspace(-np.pi, np.pi, I, endpoint=False), J)
    return mu, w, lat, lon


def _ensemble(B=5, seed=3):
    """Terminal-Phi-like fields: a day-night pattern plus noise, per member."""
    rng = np.random.default_rng(seed)
    mu, _, _, _ = _grid()
    lam = np.linspace(-np.pi, np.pi, I, endpoint=False)[None, :]
    base = 4e4 * np.cos(lam) * np.sqrt(1 - mu[:, None] ** 2)
    return np.stack([base * (1 + 0.3 * k) + 2e3 * rng.standard_normal((J, I)) for k in range(B)])


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("name", FIXTURES)
def test_simple_phase_curve_matches_the_fixture(cuda, name):
    """unit_tests/test_parity_reference_regression.py:136-148 on the GPU kernel,
    from the fixture's final Phi and (ensemble of two) from a perturbed copy."""
    from my_swampe_gb300.emission import simple_phase_curve

    ref = np.load(GOLDEN / name)
    phi = ref["final_Phi"]
    got = simple_phase_curve(torch.tensor(phi, device="cuda"), ref["phase_angles"]).cpu().numpy()
    np.testing.assert_allclose(got, ref["phase_curve"], rtol=0, atol=1e-10)
    two = torch.tensor(np.stack([phi, 2.0 * phi + 1.0]), device="cuda")
    both = simple_phase_curve(two, ref["phase_angles"]).cpu().numpy()
    np.testing.assert_allclose(both[0], ref["phase_curve"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(both[1], eo.simple_phase_curve(2.0 * phi + 1.0, ref["phase_angles"]), rtol=0,
                               atol=1e-12)


@pytest.mark.parametrize("case", list(FIXTURE_CASES))
def test_simple_phase_curve_of_the_gpu_terminal_phi(cuda, case):
    """The fixture case run on the GPU FP64 path, then its phase curve on the GPU."""
    from my_swampe_gb300 import run_model_scan_final
    from my_swampe_gb300.emission import simple_phase_curve

    ref = np.load(GOLDEN / f"{case}.npz")
    phi = run_model_scan_final(**FIXTURE_CASES[case], diagnostics=False)["last_state"].Phi_curr
    got = simple_phase_curve(phi, ref["phase_angles"]).cpu().numpy()
    np.testing.assert_allclose(got, ref["phase_curve"], rtol=0, atol=1e-10)


@pytest.mark.parametrize("mode", ["geopotential", "linear"])
def test_temperature_matches_oracle(cuda, mode):
    from my_swampe_gb300.emission import EmissionConfig, phi_to_temperature

    phi = _ensemble()
    Pb = np.array([3e5, 4e5, 5e5, 6e5, 7e5])
    cfg = EmissionConfig(emission_temp_mode=mode)
    T = phi_to_temperature(torch.tensor(phi, device="cuda"), torch.tensor(Pb, device="cuda"), cfg).cpu().numpy()
    for b in range(len(Pb)):
        want = eo.phi_to_temperature(phi[b], Pb[b], temp_mode=mode)
        assert _rel(T[b], want) <= 1e-15
    # one field, scalar Phibar
    T1 = phi_to_temperature(torch.tensor(phi[0], device="cuda"), 3e5, cfg).cpu().numpy()
    np.testing.assert_array_equal(T1, T[0])


@pytest.mark.parametrize("model,bands", [("bolometric", None), ("planck", None),
                                         ("planck", ([3.6e-6, 4.5e-6, 8.0e-6], [1.0, 2.0, 1.0]))])
def test_intensity_matches_oracle(cuda, model, bands):
    from my_swampe_gb300.emission import EmissionConfig, temperature_to_intensity

    T = np.stack([eo.phi_to_temperature(p, 4e5) for p in _ensemble()])
    kw = dict(emission_model=model)
    if bands:
        kw.update(planck_band_wavelengths_m=bands[0], planck_band_weights=bands[1])
    got = temperature_to_intensity(torch.tensor(T, device="cuda"), EmissionConfig(**kw)).cpu().numpy()
    for b in range(T.shape[0]):
        assert _rel(got[b], eo.temperature_to_intensity(T[b], **kw)) <= 1e-14


@pytest.mark.parametrize("model", ["bolometric", "planck"])
def test_emission_coefficients_match_oracle(cuda, model):
    """Phi -> T -> intensity -> projection, fused, against the oracle's chain,
    with a ydeg = 10 design matrix (121 coefficients) on the M = 42 grid."""
    from my_swampe_gb300.emission import EmissionConfig, build_projector, emission_coefficients, \
        intensity_map_to_y_dense

    _, w, lat, lon = _grid()
    D = eo.real_ylm_design(10, lat, lon)
    P_np = eo.build_projector(D, w)
    P = build_projector(torch.tensor(D, device="cuda"), torch.tensor(w, device="cuda"))
    assert _rel(P.cpu().numpy(), P_np) <= 1e-9
    phi = _ensemble()
    Pb = np.full(phi.shape[0], 4e5)
    cfg = EmissionConfig(emission_model=model)
    y = emission_coefficients(torch.tensor(phi, device="cuda"), torch.tensor(Pb, device="cuda"),
                              torch.tensor(P_np, device="cuda"), torch.tensor(w, device="cuda"), cfg).cpu().numpy()
    for b in range(phi.shape[0]):
        T = eo.phi_to_temperature(phi[b], Pb[b])
        Imap = eo.temperature_to_intensity(T, emission_model=model)
        want = eo.intensity_map_to_y_dense(Imap, P_np, w)
        assert want[0] == 1.0 and y[b, 0] == 1.0
        assert _rel(y[b], want) <= 1e-12, b
        # the same from the intensity map itself
        yi = intensity_map_to_y_dense(torch.tensor(Imap, device="cuda"), torch.tensor(P_np, device="cuda"),
                                      torch.tensor(w, device="cuda")).cpu().numpy()
        assert _rel(yi, want) <= 1e-12


@pytest.mark.parametrize("JI", [(96, 192), (160, 320)])
def test_emission_coefficients_on_the_larger_grids(cuda, JI):
    """M = 63 and M = 106 grids, linear temperature mode, band-averaged Planck
    intensity, ydeg = 6 (49 coefficients)."""
    from my_swampe_gb300.emission import EmissionConfig, emission_coefficients

    Jg, Ig = JI
    mu, w = np.polynomial.legendre.leggauss(Jg)
    lat = np.repeat(np.arcsin(mu), Ig)
    lon = np.tile(np.linspace(-np.pi, np.pi, Ig, endpoint=False), Jg)
    P = eo.build_projector(eo.real_ylm_design(6, lat, lon), w)
    rng = np.random.default_rng(Jg)
    lam = np.linspace(-np.pi, np.pi, Ig, endpoint=False)[None, :]
    phi = np.stack([3e4 * k * np.cos(lam) * np.sqrt(1 - mu[:, None] ** 2) + 1e3 * rng.standard_normal((Jg, Ig))
                    for k in (1, 2, 3)])
    kw = dict(emission_temp_mode="linear", emission_model="planck", planck_band_wavelengths_m=[3.6e-6, 4.5e-6],
              planck_band_weights=[1.0, 1.0])
    y = emission_coefficients(torch.tensor(phi, device="cuda"), 0.0, torch.tensor(P, device="cuda"),
                              torch.tensor(w, device="cuda"), EmissionConfig(**kw)).cpu().numpy()
    for b in range(3):
        T = eo.phi_to_temperature(phi[b], 0.0, temp_mode="linear")
        Imap = eo.temperature_to_intensity(T, emission_model="planck", planck_band_wavelengths_m=[3.6e-6, 4.5e-6],
                                           planck_band_weights=[1.0, 1.0])
        assert _rel(y[b], eo.intensity_map_to_y_dense(Imap, P, w)) <= 1e-12, b


def test_non_finite_member_gives_nan_and_leaves_the_others(cuda):
    from my_swampe_gb300.emission import emission_coefficients, intensity_map_to_y_dense

    _, w, lat, lon = _grid()
    P = torch.tensor(eo.build_projector(eo.real_ylm_design(4, lat, lon), w), device="cuda")
    wt = torch.tensor(w, device="cuda")
    phi = _ensemble(B=3)
    clean = emission_coefficients(torch.tensor(phi, device="cuda"), 4e5, P, wt).cpu().numpy()
    phi[1, 10, 20] = np.nan
    got = emission_coefficients(torch.tensor(phi, device="cuda"), 4e5, P, wt).cpu().numpy()
    assert np.all(np.isnan(got[1]))
    np.testing.assert_array_equal(got[[0, 2]], clean[[0, 2]])
    # a zero intensity map has no usable mean: all NaN
    z = intensity_map_to_y_dense(torch.zeros((1, J, I), dtype=torch.float64, device="cuda"), P, wt).cpu().numpy()
    assert np.all(np.isnan(z))


def test_phase_curve_matches_oracle(cuda):
    from my_swampe_gb300.emission import phase_curve

    rng = np.random.default_rng(9)
    y = rng.standard_normal((4, 121))
    A = rng.standard_normal((200, 121))
    amp = np.array([1500e-6, 1e-3, 2e-3, 5e-4])
    got = phase_curve(torch.tensor(y, device="cuda"), torch.tensor(A, device="cuda"),
                      torch.tensor(amp, device="cuda")).cpu().numpy()
    for b in range(4):
        assert _rel(got[b], eo.phase_curve(y[b], A, amp[b])) <= 1e-13
    one = phase_curve(torch.tensor(y[0], device="cuda"), torch.tensor(A, device="cuda"), 1500e-6).cpu().numpy()
    np.testing.assert_array_equal(one, got[0])


def test_members_are_independent_bit_for_bit(cuda):
    """An ensemble's coefficients equal the single-member calls exactly."""
    from my_swampe_gb300.emission import emission_coefficients

    _, w, lat, lon = _grid()
    P = torch.tensor(eo.build_projector(eo.real_ylm_design(6, lat, lon), w), device="cuda")
    wt = torch.tensor(w, device="cuda")
    phi = torch.tensor(_ensemble(B=4, seed=8), device="cuda")
    Pb = torch.tensor([3e5, 4e5, 5e5, 6e5], dtype=torch.float64, device="cuda")
    ens = emission_coefficients(phi, Pb, P, wt)
    for b in range(4):
        assert torch.equal(ens[b], emission_coefficients(phi[b], Pb[b], P, wt))
