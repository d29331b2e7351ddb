"""The opt-in schemes on the GPU: the semi-implicit leapfrog
(semi_implicit_tdiff.py) and the Robert-Asselin-Williams filter
(model.py:1007-1087), forward, against the FP64 oracle on identical inputs
(the reference's absolute tolerances, as the classic path) and against the
properties the reference's tests assert (unit_tests/test_semi_implicit.py,
unit_tests/test_raw_filter.py)."""
import numpy as np
import pytest

from oracle import swampe_oracle as o
from test_gpu_parity import FIELDS, _compare_with_oracle, _np

pytestmark = pytest.mark.gpu

SYNTH = dict(M=42, Phibar=3.0e5, omega=3.2e-5, a=8.2e7, taurad=36000.0, taudrag=21600.0, DPhieq=1.0e6, test=None)
WASP43B = dict(M=42, Phibar=4.0e6, omega=8.939689388812098e-05, a=71920952.0, taurad=36000.0, taudrag=21600.0,
               DPhieq=3.5e6, g=49.66, test=None)
EARTH = dict(M=42, Phibar=3.0e3, omega=7.2921159e-5, a=6.37122e6, forcflag=False)


def test_semi_implicit_forced_matches_oracle(cuda):
    # beyond t = 3 (filter on), with implicit relaxation and drag
    _compare_with_oracle(dict(SYNTH, dt=240.0, tmax=14, semi_implicit=True))


@pytest.mark.parametrize("variant", ["no_drag", "unforced", "no_modal", "no_diff", "alpha"])
def test_semi_implicit_variants_match_oracle(cuda, variant):
    kw = dict(SYNTH, dt=600.0, tmax=10, semi_implicit=True)
    if variant == "no_drag":
        kw.update(taudrag=-1.0)
    elif variant == "unforced":
        kw.update(forcflag=False)
    elif variant == "no_modal":
        kw.update(modalflag=False)
    elif variant == "no_diff":
        kw.update(diffflag=False)
    else:
        kw.update(si_alpha=0.7, K6Phi=2.0e33)
    _compare_with_oracle(kw)


@pytest.mark.parametrize("test", [1, 2])
def test_semi_implicit_test_cases_match_oracle(cuda, test):
    _compare_with_oracle(dict(EARTH, dt=600.0, tmax=10, test=test, semi_implicit=True))


@pytest.mark.parametrize("M", [63, 106])
def test_semi_implicit_other_truncations(cuda, M):
    _compare_with_oracle(dict(SYNTH, M=M, dt=600.0, tmax=6, semi_implicit=True))


def test_raw_filter_matches_oracle(cuda):
    _compare_with_oracle(dict(SYNTH, dt=240.0, tmax=14, raw_filter=True, williams_alpha=0.53))


def test_raw_filter_with_semi_implicit_matches_oracle(cuda):
    _compare_with_oracle(dict(SYNTH, dt=600.0, tmax=14, raw_filter=True, williams_alpha=0.53, semi_implicit=True))


def test_raw_filter_test1_matches_oracle(cuda):
    # the initial condition has content beyond the truncation: the RAW filter
    # moves its residual into the curr level as well
    _compare_with_oracle(dict(EARTH, dt=600.0, tmax=10, test=1, raw_filter=True, williams_alpha=0.53))


def test_raw_alpha_one_is_bit_identical_to_classic_ra(cuda):
    """test_raw_filter.py:37-44 on the GPU FP64 path."""
    from my_swampe_gb300 import run_model_scan

    kw = dict(SYNTH, dt=240.0, tmax=40)
    base = run_model_scan(**kw)
    raw = run_model_scan(**kw, raw_filter=True, williams_alpha=1.0)
    for k in FIELDS:
        np.testing.assert_array_equal(_np(base["outs"][k]), _np(raw["outs"][k]), err_msg=k)
    raw2 = run_model_scan(**kw, raw_filter=True, williams_alpha=0.53)
    assert float(np.max(np.abs(_np(base["outs"]["Phi"][-1]) - _np(raw2["outs"]["Phi"][-1])))) > 0.0


def test_semi_implicit_preserves_steady_advection(cuda):
    """test_semi_implicit.py:107-118"""
    from my_swampe_gb300 import run_model_scan

    out = run_model_scan(**EARTH, test=1, dt=600.0, tmax=2 + 36, semi_implicit=True)
    eta = _np(out["outs"]["eta"])
    drift = float(np.sqrt(np.mean((eta[-1] - eta[0]) ** 2))) / float(np.std(eta[0]))
    assert drift < 1e-8


def test_semi_implicit_stable_beyond_explicit_limit(cuda):
    """test_semi_implicit.py:60-71: one day of WASP-43b at dt = 1200 s."""
    from my_swampe_gb300 import run_model_scan_final

    last = run_model_scan_final(**WASP43B, dt=1200.0, tmax=74, semi_implicit=True)["last_state"]
    for f in ("eta_curr", "delta_curr", "Phi_curr", "U_curr", "V_curr", "etam_curr", "Rum_lag"):
        assert np.all(np.isfinite(_np(getattr(last, f)))), f


@pytest.mark.parametrize("precision", ["fp64", "fast"])
def test_semi_implicit_equilibrium_is_dt_insensitive(cuda, precision):
    """test_semi_implicit.py:74-104 (reference measured 1.6e-5)."""
    from my_swampe_gb300 import run_model_scan_final

    def terminal(dt):
        steps = int(round(3.0 * 86400.0 / dt))
        last = run_model_scan_final(**WASP43B, dt=dt, tmax=2 + steps, semi_implicit=True, precision=precision)
        return _np(last["last_state"].Phi_curr).astype(np.float64)

    ref, coarse = terminal(240.0), terminal(1200.0)
    rel = float(np.sqrt(np.mean((coarse - ref) ** 2))) / float(np.std(ref))
    assert np.isfinite(rel) and rel < 1e-3


def test_semi_implicit_fast_precision_is_close(cuda):
    """FP32 state (SIMT Legendre kernel) against the FP64 oracle over 60 steps.
    Relative L2 bounds: eta, Phi 1e-5 (observed 6e-7, 4e-7); delta 1e-4
    (observed 2.5e-5: the semi-implicit delta is a small difference of the
    n(n+1) dt Phi terms, so the FP32 error of the Phi transform dominates it)."""
    from my_swampe_gb300 import run_model_scan_final

    kw = dict(SYNTH, dt=600.0, tmax=62, semi_implicit=True)
    g = run_model_scan_final(**kw, precision="fast")["last_state"]
    r = o.run_model_scan_final(**kw)["last_state"]
    for f, tol in (("eta", 1e-5), ("delta", 1e-4), ("Phi", 1e-5)):
        got = _np(getattr(g, f + "_curr")).astype(np.float64)
        want = np.asarray(r[f + "_curr"])
        rel = np.linalg.norm(got - want) / np.linalg.norm(want)
        assert rel < tol, (f, rel)


def test_semi_implicit_ensemble_of_alphas(cuda):
    """Per-member si_alpha in one launch equals the direct calls."""
    from my_swampe_gb300 import run_model_scan_final

    kw = dict(SYNTH, dt=600.0, tmax=8, semi_implicit=True)
    alphas = [0.5, 0.6, 0.8]
    ens = _np(run_model_scan_final(**kw, si_alpha=alphas)["last_state"].Phi_curr)
    for i, al in enumerate(alphas):
        direct = _np(run_model_scan_final(**kw, si_alpha=al)["last_state"].Phi_curr)
        np.testing.assert_allclose(ens[i], direct, rtol=0, atol=1e-10)


def test_adjoint_rejects_raw_filter(cuda):
    """The C ABI refuses the adjoint of the RAW filter (its derivatives are
    tangent runs, and reverse-mode initial-field gradients are refused in
    Python)."""
    import torch
    from my_swampe_gb300.engine import Engine, RunFlagsC

    eng = Engine([(42, 2)], "fp64")
    lam, lamy, grad = eng.new_adjoint_buffers()
    gd = eng.groups[0]
    slots = [torch.empty((3,) + tuple(gd["fourier"].shape), dtype=eng.cdtype, device=eng.device)]
    with pytest.raises(RuntimeError, match="classic"):
        eng.adjoint_window(RunFlagsC(raw_filter=True), [gd["fourier"]], slots, lam, lamy, grad, t0=2, nsteps=2)


def test_raw_filter_fast_precision_is_close(cuda):
    """FP32 state with the RAW filter against the FP64 oracle over 60 steps.
    The step runs in the projection form (the filter mixes the initial
    condition's coefficients back into the curr carry, so the incremental form's
    premise fails), whose FP32 error scales with the fields: bounds eta, Phi
    1e-4, delta 1e-3 relative L2 (observed at dt = 240 s: 1.7e-5, 2.1e-5,
    2.2e-4)."""
    from my_swampe_gb300 import run_model_scan_final

    kw = dict(SYNTH, dt=240.0, tmax=62, raw_filter=True, williams_alpha=0.53)
    g = run_model_scan_final(**kw, precision="fast")["last_state"]
    r = o.run_model_scan_final(**kw)["last_state"]
    for f, tol in (("eta", 1e-4), ("delta", 1e-3), ("Phi", 1e-4)):
        got = _np(getattr(g, f + "_curr")).astype(np.float64)
        want = np.asarray(r[f + "_curr"])
        rel = np.linalg.norm(got - want) / np.linalg.norm(want)
        assert rel < tol, (f, rel)
