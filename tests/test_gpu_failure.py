"""Failure detection without a GPU fault.

1. The blow-up gate (model.py:838-864, 1768-1795) per ensemble member: one
   member of four gets a wind of 20 km/s in its host-prepared initial
   condition, so its RMS wind is above blowup_rms = 8000 m/s from the first
   step.  Only that member's dead flag trips (dead_first_idx 0, every history
   row its frozen initial state); the other members' fields are bit-identical
   to a run of the clean ensemble (their diagnostics, reduced with atomics,
   equal to round-off).  Both precisions (the tensor-core Legendre kernel
   has its own gate).
2. The bounded waits of the tensor-core kernels: with the plan's poll limit
   at 0 (swp_plan_set_wait_limit) every mbarrier wait gives up at once.  The
   forward and adjoint Legendre kernels then report through the device error
   word (swp_device_status -> 1, Engine.check_device_status raises), drain
   what they issued and return; the context stays usable, and with the default
   limit restored the next run equals a clean engine's bit for bit.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

BASE = dict(M=42, dt=600.0, tmax=10, Phibar=3.0e5, omega=3.2e-5, a=8.2e7, test=None)


def _ensemble_ics(B=4, bad=None):
    from oracle import swampe_oracle as o

    geo = o.cached_geometry(42)
    J, I = geo["J"], geo["I"]
    mu = geo["mus"][:, None] * np.ones((1, I))
    rng = np.random.default_rng(21)
    eta0 = np.stack([2 * 3.2e-5 * mu] * B)
    Phi0 = np.stack([3e3 * np.cos(np.pi * mu) * (1 + 0.1 * k) + rng.standard_normal((J, I)) for k in range(B)])
    U0 = np.stack([20.0 * np.sqrt(1 - mu**2)] * B)
    if bad is not None:
        U0[bad] = 2.0e4
    z = np.zeros((B, J, I))
    return dict(eta0_init=eta0, delta0_init=z, Phi0_init=Phi0, U0_init=U0, V0_init=z)


@pytest.mark.parametrize("precision", ["fp64", "fast"])
def test_blowup_gate_freezes_only_the_blown_member(cuda, precision):
    from my_swampe_gb300 import run_model_scan

    par = dict(taurad=[36000.0, 50000.0, 70000.0, 90000.0], taudrag=[21600.0] * 4, DPhieq=[1e6, 1.2e6, 1.4e6, 1.6e6])
    clean = run_model_scan(**BASE, **par, **_ensemble_ics(), precision=precision)
    bad = run_model_scan(**BASE, **par, **_ensemble_ics(bad=2), precision=precision)
    assert clean["dead_first_idx"].tolist() == [-1, -1, -1, -1]
    assert bad["dead_first_idx"].tolist() == [-1, -1, 0, -1]
    assert bad["last_state"].dead.tolist() == [False, False, True, False]
    assert bool(bad["outs"]["dead"][2].all()) and not bool(bad["outs"]["dead"][[0, 1, 3]].any())
    keep = [0, 1, 3]
    for k in ("eta", "delta", "Phi", "U", "V"):
        assert torch.equal(bad["outs"][k][keep], clean["outs"][k][keep]), k
    # the diagnostics are sums over latitude blocks reduced with atomics, whose
    # order varies from run to run: equal to round-off
    for k in ("rms", "spin_min", "phi_min", "phi_max"):
        torch.testing.assert_close(bad["outs"][k][keep], clean["outs"][k][keep], rtol=1e-12, atol=0, msg=k)
    for name in ("eta_curr", "delta_curr", "Phi_curr", "U_curr", "V_curr", "etam_curr", "Phim_curr", "Am_curr"):
        assert torch.equal(getattr(bad["last_state"], name)[keep], getattr(clean["last_state"], name)[keep]), name
    # the dead member keeps its initial state in every history row
    ics = _ensemble_ics(bad=2)
    tol = 1e-9 if precision == "fp64" else 1e-3
    for k, f in (("eta", "eta0_init"), ("Phi", "Phi0_init"), ("U", "U0_init")):
        h = bad["outs"][k][2].double().cpu().numpy()
        for row in h:
            np.testing.assert_allclose(row, ics[f][2], rtol=0, atol=tol * max(np.max(np.abs(ics[f][2])), 1.0))
    assert float(bad["outs"]["rms"][2][0]) > 8000.0


def test_tensor_core_wait_limit_reports_and_recovers(cuda):
    from my_swampe_gb300 import _lib, workloads
    from my_swampe_gb300.engine import Engine, RunFlagsC

    def fresh():
        eng = Engine([(42, 8)], "fast")
        wl = workloads.forced_ensemble(eng, seed=3, Phibar=3.0e5, dt=600.0)
        workloads.apply_params(eng, 0, wl["params"])
        return eng, wl

    eng, wl = fresh()
    assert eng.uses_tensor_cores
    lib = _lib.load()
    flags = RunFlagsC()
    eng.init_state([wl["ics"]], flags)
    eng.forward(flags, t0=2, nsteps=1)
    s_in = [eng.groups[0]["fourier"].clone()]
    eng.forward(flags, t0=3, nsteps=1)
    s_out = [eng.groups[0]["fourier"].clone()]
    eng.check_device_status()  # clean so far

    assert lib.swp_plan_set_wait_limit(eng._plan, 0) == 0
    eng.forward(flags, t0=4, nsteps=1)          # forward tensor-core Legendre kernel gives up
    with pytest.raises(RuntimeError, match="timed out"):
        eng.check_device_status()
    eng.check_device_status()                   # the word was cleared by the read
    lam, lamy, grad = eng.new_adjoint_buffers()
    lam[0].normal_()
    eng.adjoint_step(flags, s_in, s_out, lam, lamy, grad, t=3)  # adjoint tensor-core kernel gives up
    with pytest.raises(RuntimeError, match="timed out"):
        eng.check_device_status()

    # default limit: the context is usable and the steps are exact again
    assert lib.swp_plan_set_wait_limit(eng._plan, _lib.WAIT_LIMIT_DEFAULT) == 0
    eng.init_state([wl["ics"]], flags)
    eng.forward(flags, t0=2, nsteps=3)
    eng.check_device_status()
    got = eng.output_physical(flags)[0]
    ref_eng, ref_wl = fresh()
    ref_eng.init_state([ref_wl["ics"]], flags)
    ref_eng.forward(flags, t0=2, nsteps=3)
    want = ref_eng.output_physical(flags)[0]
    assert torch.equal(got, want)


def test_differentiable_run_reports_a_timeout_at_backward(cuda):
    """A tensor-core wait that runs out inside a differentiable run (forward or
    adjoint sweep) surfaces as an error of the backward pass, which checks the
    device status before it returns gradients."""
    from my_swampe_gb300 import _lib, workloads
    from my_swampe_gb300.adjoint import integrate
    from my_swampe_gb300.engine import Engine, RunFlagsC

    eng = Engine([(42, 8)], "fast")
    wl = workloads.forced_ensemble(eng, seed=3, Phibar=3.0e5, dt=600.0)
    workloads.apply_params(eng, 0, wl["params"])
    assert eng.uses_tensor_cores
    lib = _lib.load()
    p = {k: torch.as_tensor(wl["params"][k], dtype=torch.float64, device=eng.device).expand(8).clone()
         .requires_grad_(True) for k in ("taurad", "taudrag", "DPhieq")}
    p["Phibar"] = torch.full((8,), float(wl["params"]["Phibar"]), dtype=torch.float64, device=eng.device)

    def run():
        out = integrate(eng, RunFlagsC(), t0=2, nsteps=4, params=[p], ics=[wl["ics"]], store="all")[0]
        (out[2].double() ** 2).mean().backward()

    run()  # clean
    assert lib.swp_plan_set_wait_limit(eng._plan, 0) == 0
    try:
        with pytest.raises(RuntimeError, match="timed out"):
            run()
    finally:
        assert lib.swp_plan_set_wait_limit(eng._plan, _lib.WAIT_LIMIT_DEFAULT) == 0
    eng.check_device_status()  # cleared by the failed check
    run()
