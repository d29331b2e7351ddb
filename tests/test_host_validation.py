"""Host-side behaviour that needs no GPU: argument validation at entry (the
reference's unit_tests/test_invalid_input.py cases), the loud failure of the
product path without CUDA, continuation helpers and the per-member parameter
rules.  All checks run before any device work."""
import numpy as np
import pytest
import torch

from my_swampe_gb300 import continuation
from my_swampe_gb300.model import run_model_scan, run_model_scan_final

BASE = dict(M=42, dt=600.0, Phibar=3.0e5, omega=3.2e-5, a=8.2e7)
J, I = 64, 128


def test_tmax_too_small():
    with pytest.raises(ValueError, match="tmax"):
        run_model_scan(**BASE, tmax=1)


@pytest.mark.parametrize("dt", [0.0, -30.0])
def test_dt_non_positive(dt):
    kw = dict(BASE, dt=dt)
    with pytest.raises(ValueError, match="dt"):
        run_model_scan(**kw, tmax=4)


def test_starttime_after_tmax():
    with pytest.raises(ValueError, match="starttime"):
        run_model_scan(**BASE, tmax=4, starttime=10)


def test_unsupported_test_selector():
    with pytest.raises(NotImplementedError, match="test=99"):
        run_model_scan(**BASE, tmax=4, test=99)


@pytest.mark.parametrize("M", [21, 85, 0])
def test_unsupported_M(M):
    kw = dict(BASE, M=M)
    with pytest.raises(ValueError, match="M"):
        run_model_scan(**kw, tmax=4)


def test_partial_initial_conditions():
    with pytest.raises(ValueError, match="eta0_init.*delta0_init.*Phi0_init"):
        run_model_scan(**BASE, tmax=4, eta0_init=np.zeros((J, I)))


def test_partial_velocity_initial_conditions():
    z = np.zeros((J, I))
    with pytest.raises(ValueError, match="U0_init.*V0_init"):
        run_model_scan(**BASE, tmax=4, eta0_init=z, delta0_init=z, Phi0_init=z, U0_init=z)


def test_wrong_shape_initial_condition():
    z = np.zeros((J, I))
    with pytest.raises(ValueError, match="Phi0_init"):
        run_model_scan(**BASE, tmax=4, eta0_init=z, delta0_init=z, Phi0_init=np.zeros((J + 1, I)))


def test_contflag_without_contTime():
    with pytest.raises(ValueError, match="contTime"):
        run_model_scan(**BASE, tmax=4, contflag=True)


def test_contTime_non_numeric():
    with pytest.raises(ValueError, match="numeric"):
        run_model_scan(**BASE, tmax=4, contflag=True, contTime="ten")


def test_semi_implicit_and_raw_reject_expflag():
    # test_semi_implicit.py::test_semi_implicit_rejects_explicit_scheme,
    # test_raw_filter.py::test_raw_filter_rejects_explicit_scheme
    with pytest.raises(ValueError, match="semi_implicit"):
        run_model_scan(**BASE, tmax=4, semi_implicit=True, expflag=True)
    with pytest.raises(ValueError, match="raw_filter"):
        run_model_scan(**BASE, tmax=4, raw_filter=True, expflag=True)


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the no-GPU failure")
def test_semi_implicit_has_no_cpu_fallback():
    with pytest.raises(RuntimeError, match="CUDA"):
        run_model_scan(**BASE, tmax=4, semi_implicit=True, raw_filter=True)


def test_final_rejects_return_history():
    with pytest.raises(TypeError):
        run_model_scan_final(**BASE, tmax=4, return_history=True)


def test_member_parameter_lengths_must_agree():
    with pytest.raises(ValueError, match="same length"):
        run_model_scan(**BASE, tmax=4, taurad=[1e4, 2e4], DPhieq=[1e5, 2e5, 3e5])
    with pytest.raises(ValueError, match="scalars or 1-D"):
        run_model_scan(**BASE, tmax=4, taurad=np.ones((2, 2)))


def test_member_axis_of_fields_must_match_parameters():
    z = np.zeros((3, J, I))
    with pytest.raises(ValueError, match="member axis"):
        run_model_scan(**BASE, tmax=4, taurad=[1e4, 2e4], eta0_init=z, delta0_init=z, Phi0_init=z)


def test_valid_call_without_cuda_fails_loudly():
    """The product path has no CPU fallback."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError, match="CUDA|GPU|libswampe"):
        run_model_scan(**BASE, tmax=4)


def test_continuation_timestamps_round_trip():
    """continuation.py:67-132: timestamp = floor(dt * t / unit) and back; exact
    when dt * t is a whole number of units."""
    for units, dt, t in (("hours", 600.0, 36), ("minutes", 30.0, 14), ("seconds", 12.0, 5), ("days", 1200.0, 720),
                         ("steps", 600.0, 17)):
        ts = continuation.compute_timestamp(units, t, dt)
        assert continuation.compute_t_from_timestamp(units, float(ts), dt) == t, units
    assert continuation.compute_timestamp("hours", 12, 600.0) == "2"
    assert continuation.compute_timestamp("hours", 13, 600.0) == "2"  # floor, as the reference's int()
    with pytest.raises(ValueError, match="units"):
        continuation.compute_timestamp("fortnights", 1, 1.0)


def test_continuation_pickles_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    fields = [rng.standard_normal((J, I)) for _ in range(5)]
    spin, geo = rng.standard_normal((10, 2)), rng.standard_normal((10, 2))
    continuation.save_data(7, *fields, spin, geo, custompath=str(tmp_path))
    back = continuation.load_data(7, custompath=str(tmp_path))
    for a, b in zip(fields, back):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(continuation.read_pickle("spinup-winds", custompath=str(tmp_path)), spin)


def test_fwd_grad_argument_rules():
    """autodiff_utils.py:27-89: theta must be 1-D, empty theta gives an empty
    gradient, a non-positive chunk is refused (before any evaluation)."""
    from my_swampe_gb300.autodiff_utils import fwd_grad

    def never(theta):
        raise AssertionError("loss evaluated")

    with pytest.raises(ValueError, match="1-D"):
        fwd_grad(never, torch.zeros((2, 2)))
    assert fwd_grad(never, torch.zeros(0)).shape == (0,)
    with pytest.raises(ValueError, match="chunk"):
        fwd_grad(never, torch.zeros(3), chunk=0)


def test_fwd_grad_on_a_cpu_function():
    """The helper itself is plain forward-mode AD: check it on a closed form."""
    from my_swampe_gb300.autodiff_utils import fwd_grad

    theta = torch.tensor([0.3, -1.2, 2.0], dtype=torch.float64)
    g = fwd_grad(lambda t: (t[0] * t[1]) ** 2 + torch.sin(t[2]), theta, chunk=2)
    want = torch.tensor([2 * theta[0] * theta[1] ** 2, 2 * theta[1] * theta[0] ** 2, torch.cos(theta[2])])
    assert torch.allclose(g, want, rtol=1e-14, atol=0)


# run_model_scan_final's keywords and defaults (reference model.py:1844-1886)
_FINAL_SIGNATURE = dict(
    M=None, dt=None, tmax=None, Phibar=None, omega=None, a=None, test=None, g=9.8, forcflag=True, taurad=86400.0,
    taudrag=86400.0, DPhieq=4 * (10**6), a1=0.05, diffflag=True, modalflag=True, alpha=0.01, expflag=False,
    K6=1.24 * (10**33), K6Phi=None, contflag=False, custompath=None, contTime=None, timeunits="hours",
    starttime=None, eta0_init=None, delta0_init=None, Phi0_init=None, U0_init=None, V0_init=None,
    semi_implicit=False, si_alpha=0.5, raw_filter=False, williams_alpha=0.53, diagnostics=False,
    remat_step=False, jit_scan=True, donate_state=False,
)


def test_run_model_scan_final_keeps_the_reference_signature():
    import inspect

    from my_swampe_gb300 import run_model_scan_final

    params = inspect.signature(run_model_scan_final).parameters
    for name, default in _FINAL_SIGNATURE.items():
        assert name in params, name
        p = params[name]
        assert p.kind == inspect.Parameter.KEYWORD_ONLY, name
        if default is None and name in ("M", "dt", "tmax", "Phibar", "omega", "a"):
            assert p.default is inspect.Parameter.empty, name
        else:
            assert p.default == default, (name, p.default, default)
    assert "return_history" not in params


def test_scan_core_entry_points_exist():
    import inspect

    from my_swampe_gb300 import model

    for fn, names in ((model._init_state_from_fields, ("static", "flags", "test", "eta0", "delta0", "Phi0", "U0", "V0")),
                      (model.simulate_scan_last, ("static", "flags", "state0", "t_seq", "test", "Uic", "Vic",
                                                  "remat_step")),
                      (model.simulate_scan, ("static", "flags", "state0", "t_seq", "test", "Uic", "Vic")),
                      (model._step_once_state_only, ("state", "t", "static", "flags", "test", "Uic", "Vic"))):
        assert tuple(inspect.signature(fn).parameters)[: len(names)] == names, fn.__name__
    import dataclasses

    assert dataclasses.is_dataclass(model.Static) and model.RunFlags(alpha=0.02).alpha == 0.02
