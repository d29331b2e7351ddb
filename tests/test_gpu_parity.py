"""Parity of the CUDA path (through the C ABI) with the reference fixtures and
the CPU oracle.  Tolerances: the reference's own (eta/delta 1e-10, Phi 5e-8,
U/V 1e-9 absolute) against the golden fixtures; against the FP64 oracle on
identical inputs, 2e-9 of each field's maximum (observed: 1e-11 .. 3e-10,
from FP64 re-association and from the GPU's Gauss weights, which are ~10x
more accurate than SciPy's roots_legendre used by the reference)."""
import numpy as np
import pytest

from conftest import ATOL, FIXTURE_CASES, GOLDEN
from oracle import swampe_oracle as o

pytestmark = pytest.mark.gpu
FIELDS = ("eta", "delta", "Phi", "U", "V")


def _np(x):
    return x.detach().cpu().numpy()


def _close_rel(got, want, rel, what=""):
    scale = max(np.max(np.abs(want)), 1e-300)
    err = np.max(np.abs(got - want))
    assert err <= rel * scale, f"{what}: max err {err:.3e} > {rel:.1e} * {scale:.3e}"


@pytest.mark.parametrize("M", [42, 63, 106])
def test_geometry_matches_scipy(cuda, M):
    from my_swampe_gb300.engine import Engine

    eng = Engine([(M, 1)], "fp64")
    geo = eng.geometry(0)
    ref = o.cached_geometry(M)
    J = ref["J"]
    exact = np.load(GOLDEN / "gauss_legendre.npz")
    np.testing.assert_allclose(_np(geo["mus"]), exact[f"mu{J}"], rtol=0, atol=3e-16)
    np.testing.assert_allclose(_np(geo["w"]), exact[f"w{J}"], rtol=3e-13, atol=0)
    np.testing.assert_allclose(_np(geo["mus"]), ref["mus"], rtol=0, atol=1e-14)
    # SciPy's roots_legendre weights (used by the reference) carry up to ~3e-11
    # relative error near the poles; the GPU weights are exact to ~1e-15.
    np.testing.assert_allclose(_np(geo["w"]), ref["w"], rtol=5e-11, atol=0)
    # the basis includes the reference's scaling underflow at M=106 (m >~ 77)
    np.testing.assert_allclose(_np(geo["Pmn"]), ref["Pmn"], rtol=0, atol=2e-12)
    np.testing.assert_allclose(_np(geo["Hmn"]), ref["Hmn"], rtol=0, atol=2e-11)


@pytest.mark.parametrize("case", list(FIXTURE_CASES))
def test_fixture_parity(cuda, case):
    """unit_tests/test_parity_reference_regression.py:96-148 on the GPU FP64 path."""
    from my_swampe_gb300 import run_model_scan, run_model_scan_final

    ref = np.load(GOLDEN / f"{case}.npz")
    kw = FIXTURE_CASES[case]
    out = run_model_scan(**kw, diagnostics=True, jit_scan=False)
    last = out["last_state"]
    t_seq = _np(out["t_seq"])
    for f in FIELDS:
        np.testing.assert_allclose(_np(getattr(last, f + "_curr")), ref["final_" + f], rtol=0, atol=ATOL[f])
    for i, st in enumerate(ref["snapshot_steps"]):
        k = int(np.where(t_seq == st)[0][0])
        for f in FIELDS:
            np.testing.assert_allclose(_np(out["outs"][f][k]), ref["snapshot_" + f][i], rtol=0, atol=ATOL[f])
    fin = run_model_scan_final(**kw, diagnostics=False, jit_scan=False)
    from test_oracle_golden import _phase_curve

    got = _phase_curve(_np(fin["last_state"].Phi_curr), ref["phase_angles"])
    np.testing.assert_allclose(got, ref["phase_curve"], rtol=0, atol=1e-10)


def _compare_with_oracle(kw, rel=2e-9, fields=FIELDS, state_fields=True):
    from my_swampe_gb300 import run_model_scan

    g = run_model_scan(**kw)
    r = o.run_model_scan(**kw)
    gl, rl = g["last_state"], r["last_state"]
    for f in fields:
        _close_rel(_np(getattr(gl, f + "_curr")), np.asarray(rl[f + "_curr"]), rel, f + "_curr")
        if f in ("eta", "delta", "Phi"):
            _close_rel(_np(getattr(gl, f + "_prev")), np.asarray(rl[f + "_prev"]), rel, f + "_prev")
    if state_fields:
        for name in ("etam_curr", "deltam_curr", "Phim_curr", "etam_prev", "Phim_prev", "Um_curr", "Vm_curr",
                     "Am_curr", "Bm_curr", "Cm_curr", "Dm_curr", "Em_curr", "PhiFm_curr", "Fm_curr", "Gm_curr",
                     "Rum_lag", "Rvm_lag"):
            _close_rel(_np(getattr(gl, name)), np.asarray(rl[name]), rel, name)
    if kw.get("diagnostics", True) and kw.get("return_history", True):
        for f in FIELDS:
            _close_rel(_np(g["outs"][f]), np.asarray(r["outs"][f]), rel, "hist " + f)
        # reference tolerances are absolute (U/V 1e-9 m/s, Phi 5e-8); spin_min is a
        # minimum wind speed and can be near zero, so it gets the U/V bound
        for k, atol in (("rms", 1e-9), ("spin_min", 1e-9), ("phi_min", 5e-8), ("phi_max", 5e-8)):
            want = r["outs"][k]
            np.testing.assert_allclose(_np(g["outs"][k]), want, rtol=2e-9,
                                       atol=max(atol, 2e-9 * float(np.max(np.abs(want)))), err_msg=k)
    return g, r


@pytest.mark.parametrize("case", list(FIXTURE_CASES))
def test_fixture_cases_match_oracle_tightly(cuda, case):
    _compare_with_oracle(dict(FIXTURE_CASES[case]))


def test_forced_longer_run_and_modalflag_off(cuda):
    kw = dict(FIXTURE_CASES["reference_case_forced_default"])
    kw.update(tmax=14, dt=600.0)
    _compare_with_oracle(kw)
    kw.update(modalflag=False, forcflag=False)
    _compare_with_oracle(kw)


def test_explicit_scheme(cuda):
    kw = dict(FIXTURE_CASES["reference_case_forced_default"])
    kw.update(expflag=True, tmax=8, dt=300.0)
    _compare_with_oracle(kw)
    kw.update(taudrag=-1.0)
    _compare_with_oracle(kw)


def test_test2_unforced(cuda):
    kw = dict(M=42, dt=600.0, tmax=12, Phibar=3.0e3, omega=7.2921159e-5, a=6.37122e6, test=2, forcflag=False)
    _compare_with_oracle(kw)


@pytest.mark.parametrize("M", [63, 106])
def test_other_truncations(cuda, M):
    kw = dict(M=M, dt=300.0, tmax=6, Phibar=3.0e5, omega=3.2e-5, a=8.2e7, test=None, taurad=36000.0,
              taudrag=21600.0, DPhieq=1.0e6)
    _compare_with_oracle(kw)


def _spectral_noise(M, amp, nmax, seed):
    """Smooth random field: spectral coefficients with n <= nmax synthesised to the grid."""
    geo = o.cached_geometry(M)
    rng = np.random.default_rng(seed)
    c = np.zeros((M + 1, M + 1), complex)
    for m in range(nmax + 1):
        for n in range(m, nmax + 1):
            c[m, n] = rng.standard_normal() + (1j * rng.standard_normal() if m > 0 else 0.0)
    x = np.real(o.invrs_fft(o.NUMPY, o.invrs_leg(o.NUMPY, c, geo["I"], M, geo["Pmn"]), geo["I"]))
    return amp * x / np.max(np.abs(x))


def test_explicit_ics_with_diagnosed_winds(cuda):
    """model.py:1641-1643: U0/V0 absent -> winds diagnosed from eta0, delta0."""
    geo = o.cached_geometry(42)
    mu = geo["mus"][:, None]
    eta0 = 2 * 3.2e-5 * mu * np.ones((1, 128)) + _spectral_noise(42, 2e-6, 10, 3)
    delta0 = _spectral_noise(42, 2e-7, 10, 4)
    Phi0 = _spectral_noise(42, 3e3, 10, 5)
    kw = dict(M=42, dt=600.0, tmax=6, Phibar=3.0e5, omega=3.2e-5, a=8.2e7, test=None,
              eta0_init=eta0, delta0_init=delta0, Phi0_init=Phi0)
    _compare_with_oracle(kw)


def test_ensemble_members_match_direct_calls(cuda):
    """unit_tests/test_vmap_smoke.py:44-93: each member equals the direct call (atol 1e-10)."""
    from my_swampe_gb300 import run_model_scan_final

    base = dict(M=42, dt=600.0, tmax=5, Phibar=3.0e5, omega=7.292e-5, a=6.37122e6, test=None, forcflag=True,
                taurad=86400.0, taudrag=86400.0, diffflag=True, modalflag=True, alpha=0.01, expflag=False, K6=1.24e33)
    stack = [2.0e6, 4.0e6, 6.0e6]
    ens = _np(run_model_scan_final(**base, DPhieq=stack)["last_state"].Phi_curr)
    assert ens.shape == (3, 64, 128)
    for i, d in enumerate(stack):
        direct = _np(run_model_scan_final(**base, DPhieq=d)["last_state"].Phi_curr)
        np.testing.assert_allclose(ens[i], direct, rtol=0, atol=1e-10)
    assert min(np.max(np.abs(ens[i] - ens[j])) for i in range(3) for j in range(i + 1, 3)) > 0


def test_fast_precision_is_close(cuda):
    from my_swampe_gb300 import run_model_scan_final

    kw = dict(FIXTURE_CASES["reference_case_forced_default"])
    kw.update(tmax=12, dt=600.0)
    g = run_model_scan_final(**kw, precision="fast")["last_state"]
    r = o.run_model_scan_final(**kw)["last_state"]
    for f in FIELDS:
        got = _np(getattr(g, f + "_curr")).astype(np.float64)
        want = np.asarray(r[f + "_curr"])
        rel = np.linalg.norm(got - want) / np.linalg.norm(want)
        assert rel < 1e-5, (f, rel)


@pytest.mark.parametrize("kernel,tol", [("simt", 5e-6), ("tc", 2e-5)])
def test_fast_precision_long_forced_run_error(cuda, kernel, tol):
    """FP32 path (incremental steps) against the FP64 GPU path over 400 steps of
    the forced benchmark regime, relative L2 of Phi, eta, delta: <= 5e-6 with
    the SIMT FP32 Legendre kernel (24-bit operands), <= 2e-5 with the
    tensor-core kernel (3xTF32: 22-bit operands; observed 8.5e-6 for delta,
    the smallest field)."""
    import os

    import torch
    from my_swampe_gb300 import workloads
    from my_swampe_gb300.engine import Engine, RunFlagsC

    outs = {}
    for prec in ("fp64", "fast"):
        old = os.environ.pop("SWP_NO_TC", None)
        if kernel == "simt":
            os.environ["SWP_NO_TC"] = "1"
        try:
            eng = Engine([(42, 4)], prec)
        finally:
            os.environ.pop("SWP_NO_TC", None)
            if old is not None:
                os.environ["SWP_NO_TC"] = old
        if prec == "fast":
            assert eng.uses_tensor_cores == (kernel == "tc")
        wl = workloads.forced_ensemble(eng, seed=77)
        workloads.apply_params(eng, 0, wl["params"])
        flags = RunFlagsC()
        eng.init_state([wl["ics"]], flags)
        eng.forward(flags, t0=2, nsteps=400)
        outs[prec] = eng.output_physical(flags)[0].double()
    for k, name in enumerate(("eta", "delta", "Phi")):
        ref = outs["fp64"][k]
        rel = float(torch.linalg.vector_norm(outs["fast"][k] - ref) / torch.linalg.vector_norm(ref))
        assert rel < tol, (name, rel)
