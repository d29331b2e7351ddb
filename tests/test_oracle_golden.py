"""The CPU oracle pinned against the reference's own golden fixtures, quirk
tests and transform known-answer tests (no GPU needed)."""
import numpy as np
import pytest

from conftest import ATOL, FIXTURE_CASES, GOLDEN
from oracle import swampe_oracle as o


def _phase_curve(phi, phase_angles):
    """Simplified retrieval projection (unit_tests/test_parity_reference_regression.py:67-82)."""
    J, I = phi.shape
    lam = np.linspace(-np.pi, np.pi, I, endpoint=False)[None, :]
    mus = np.polynomial.legendre.leggauss(J)[0][:, None]
    wgt = np.sqrt(np.clip(1.0 - mus * mus, 0.0, None))
    flux = np.array([np.sum(phi * np.maximum(np.cos(lam - p), 0.0) * wgt) for p in phase_angles])
    nrm = np.mean(np.abs(flux))
    return flux / nrm if nrm > 0 else flux


@pytest.mark.parametrize("case", list(FIXTURE_CASES))
def test_oracle_matches_reference_fixtures(case):
    ref = np.load(GOLDEN / f"{case}.npz")
    r = o.run_model_scan(**FIXTURE_CASES[case])
    ls = r["last_state"]
    for f in ("eta", "delta", "Phi", "U", "V"):
        np.testing.assert_allclose(np.asarray(ls[f + "_curr"]), ref["final_" + f], rtol=0, atol=ATOL[f])
    for i, st in enumerate(ref["snapshot_steps"]):
        k = int(np.where(r["t_seq"] == st)[0][0])
        for f in ("eta", "delta", "Phi", "U", "V"):
            np.testing.assert_allclose(r["outs"][f][k], ref["snapshot_" + f][i], rtol=0, atol=ATOL[f])
    got = _phase_curve(np.asarray(ls["Phi_curr"]), ref["phase_angles"])
    np.testing.assert_allclose(got, ref["phase_curve"], rtol=0, atol=1e-10)


@pytest.mark.parametrize("case", list(FIXTURE_CASES))
def test_oracle_legacy_spinup_geopot_match_fixtures(case):
    """run_model's (tmax, 2) spinup / geopot arrays (model.py:2106-2158) against
    the arrays the reference fixtures carry: wind diagnostics at the U/V
    tolerance, Phi extrema at the Phi tolerance."""
    ref = np.load(GOLDEN / f"{case}.npz")
    kw = FIXTURE_CASES[case]
    r = o.run_model_scan(**kw)
    spin, geop = o.legacy_diagnostics(o.NUMPY, r, kw["tmax"], kw["test"])
    np.testing.assert_allclose(spin, ref["spinup"], rtol=0, atol=ATOL["U"])
    np.testing.assert_allclose(geop, ref["geopot"], rtol=0, atol=ATOL["Phi"])


def test_oracle_transform_kats():
    """unit_tests/test_transform_stack.py:37-97."""
    geo = o.cached_geometry(42)
    mus = geo["mus"]
    np.testing.assert_allclose(geo["Pmn"][:, 2, 2], 0.25 * np.sqrt(15.0) * (1 - mus**2), atol=1e-10, rtol=1e-10)
    np.testing.assert_allclose(geo["Hmn"][:, 0, 1], 0.5 * np.sqrt(6.0) * (1 - mus**2), atol=1e-10, rtol=1e-10)
    g106 = o.cached_geometry(106)
    omega = 3.2e-5
    f = 2.0 * omega * g106["mus"][:, None] * np.ones((1, g106["I"]))
    fm = o.fwd_fft_trunc(o.NUMPY, f, g106["I"], 106)
    fmn = o.fwd_leg_w(o.NUMPY, fm, g106["w"][:, None, None] * g106["Pmn"])
    chk = np.zeros((107, 107), complex)
    chk[0, 1] = omega / np.sqrt(0.375)
    np.testing.assert_allclose(fmn, chk, atol=1e-10, rtol=1e-10)


def test_oracle_quirks():
    """Dayside strict mask and Rfun clamp (unit_tests/test_parity_quirks.py:52-82)."""
    lam = np.asarray([-np.pi / 2, 0.0, np.pi / 2])
    out = o.Phieqfun(o.NUMPY, 10.0, 4.0, lam, np.asarray([0.0]))
    assert out[0, 0] == 10.0 and out[0, 2] == 10.0 and out[0, 1] > 10.0
    U = np.asarray([[2.0, -3.0]]); V = np.asarray([[1.0, 5.0]]); Q = np.asarray([[-2.0, 4.0]])
    Phi = np.asarray([[10.0, 10.0]])
    F, G = o.Rfun(o.NUMPY, U, V, Q, Phi, 2.0, -1.0)
    np.testing.assert_allclose(F, [[0.0, -U[0, 1] * Q[0, 1] / 12.0]], atol=1e-12, rtol=0)
    np.testing.assert_allclose(G, [[0.0, -V[0, 1] * Q[0, 1] / 12.0]], atol=1e-12, rtol=0)


def test_oracle_torch_backend_matches_numpy():
    torch = pytest.importorskip("torch")
    kw = dict(FIXTURE_CASES["reference_case_forced_default"])
    kw["tmax"] = 4
    a = o.run_model_scan_final(**kw)["last_state"]["Phi_curr"]
    b = o.run_model_scan_final(o.torch_backend(), **kw)["last_state"]["Phi_curr"]
    np.testing.assert_allclose(np.asarray(a), b.detach().numpy(), rtol=0, atol=1e-9)


def test_reference_M106_basis_round_trip_amplifies_modes():
    """The reference's M=106 basis carries its scaling-table underflow
    (spectral_transform.py:117-146): for m >~ 80 the weighted forward-inverse
    Legendre round trip is no longer a projector.  Its largest eigenvalue is
    1.33 (at m = 83), so a scheme that re-projects the full state every step
    (the reference's FP64 steps) amplifies those modes; for m <= 79 it is the
    identity to 1e-10."""
    geo = o.cached_geometry(106)
    P, w = geo["Pmn"], geo["w"]
    worst = {}
    for m in range(107):
        Pm = P[:, m, m:]
        ev = np.abs(np.linalg.eigvals((w[:, None] * Pm).T @ Pm))
        worst[m] = (ev.max(), ev.min())
    assert all(abs(worst[m][0] - 1) < 1e-10 and abs(worst[m][1] - 1) < 1e-10 for m in range(80))
    top = max(range(107), key=lambda m: worst[m][0])
    assert top == 83 and 1.3 < worst[83][0] < 1.35
