"""The benchmark workloads as GPU tests (reduced lengths where the CPU oracle
is the checker):
  steady zonal geostrophic flow, M=42, one member (test=2 regime, explicit ICs)
  M=63 ensemble of 32: gradients of mean((Phi_T - Phi_target)^2) vs central FD
  mixed truncations (M=42, 63, 106) in one launch == separate launches
"""
import math

import numpy as np
import pytest

from oracle import swampe_oracle as o

pytestmark = pytest.mark.gpu


def _steady_ics(M, a=6.37122e6, Omega=7.292e-5):
    geo = o.cached_geometry(M)
    mu = geo["mus"][:, None] * np.ones((1, geo["I"]))
    u0 = 2 * math.pi * a / (12 * 86400)
    Phi0 = -(a * Omega * u0 + u0 * u0 / 2) * mu**2
    eta0 = 2 * (u0 / a + Omega) * mu
    U0 = u0 * np.sqrt(1 - mu**2)
    z = np.zeros_like(mu)
    return dict(eta0_init=eta0, delta0_init=z, Phi0_init=Phi0, U0_init=U0, V0_init=z), dict(a=a, omega=Omega)


def test_steady_zonal_flow_and_blowup_gate(cuda):
    """Williamson test-2 balanced zonal flow (a = 6.37122e6, u0 = 2 pi a / 12 d,
    dt = 600 s, no diffusion).  The reference scheme does not hold this steady
    state: its modified-Euler coefficients (modEuler_tdiff.py:72-74) make it
    drift (2% by step 60) and blow up (RMS wind > 8000 m/s near step 140).
    Checked: the GPU history follows the oracle, and the blow-up gate
    (model.py:838-864) trips at the same step with the state frozen after it."""
    from my_swampe_gb300 import run_model_scan

    ics, p = _steady_ics(42)
    kw = dict(M=42, dt=600.0, Phibar=2.94e4, test=2, forcflag=False, diffflag=False, **p, **ics)
    g = run_model_scan(tmax=2 + 150, **kw)
    r = o.run_model_scan(tmax=2 + 150, **kw)
    dg, dr = int(g["dead_first_idx"]), r["dead_first_idx"]
    assert dr > 0 and dg == dr, (dg, dr)
    rms_g = g["outs"]["rms"].cpu().numpy()
    np.testing.assert_allclose(rms_g[:60], r["outs"]["rms"][:60], rtol=1e-8)
    Phi_g = g["outs"]["Phi"].cpu().numpy()
    Phi_r = np.asarray(r["outs"]["Phi"])
    scale = np.max(np.abs(Phi_r[:60]))
    assert np.max(np.abs(Phi_g[:60] - Phi_r[:60])) <= 1e-8 * scale
    # frozen after the gate: every later history row equals the last live state
    assert np.array_equal(Phi_g[dg], Phi_g[-1])
    assert bool(g["last_state"].dead)


def test_mixed_truncations_in_one_launch(cuda):
    """Groups at M=42, 63, 106 stepped by one engine (grouped launches) give the
    same states as three single-group engines."""
    import torch
    from my_swampe_gb300 import workloads
    from my_swampe_gb300.engine import Engine, RunFlagsC

    spec = [(42, 3, 30.0), (63, 2, 20.0), (106, 1, 12.0)]
    mixed = Engine([(M, B) for M, B, _ in spec], "fp64")
    ics = []
    for g, (M, B, dt) in enumerate(spec):
        wl = workloads.forced_ensemble(mixed, g=g, seed=100 + g, dt=dt)
        workloads.apply_params(mixed, g, wl["params"])
        ics.append(wl["ics"])
    flags = RunFlagsC()
    mixed.init_state(ics, flags)
    mixed.forward(flags, t0=2, nsteps=6)
    out_mixed = mixed.output_physical(flags)
    for g, (M, B, dt) in enumerate(spec):
        single = Engine([(M, B)], "fp64")
        wl = workloads.forced_ensemble(single, seed=100 + g, dt=dt)
        workloads.apply_params(single, 0, wl["params"])
        single.init_state([wl["ics"]], flags)
        single.forward(flags, t0=2, nsteps=6)
        out = single.output_physical(flags)[0]
        diff = (out_mixed[g] - out).abs().max().item()
        assert diff == 0.0 or diff <= 1e-12 * out.abs().max().item(), (M, diff)


def test_M63_ensemble_gradients_vs_central_fd(cuda):
    """M=63 (96 x 192), B=2 forced, 60 steps, checkpoints every 25: gradients of
    mean((Phi_T - Phi_target)^2) w.r.t. taurad, DPhieq vs central FD (h = 1e-4
    relative; FD noise at 1e-6 relative is above the 1e-5 check here)."""
    import torch
    from my_swampe_gb300 import workloads
    from my_swampe_gb300.engine import Engine, RunFlagsC
    from my_swampe_gb300.adjoint import integrate

    eng = Engine([(63, 2)], "fp64")
    wl = workloads.forced_ensemble(eng, seed=5, dt=20.0)
    workloads.apply_params(eng, 0, wl["params"])
    flags = RunFlagsC()
    nsteps = 60
    # target: perturbed taurad / DPhieq
    p = dict(wl["params"])
    p2 = dict(p, taurad=p["taurad"] * 1.1, DPhieq=p["DPhieq"] * 0.9)
    workloads.apply_params(eng, 0, p2)
    eng.init_state([wl["ics"]], flags)
    eng.forward(flags, t0=2, nsteps=nsteps)
    target = eng.output_physical(flags)[0][2].clone()
    workloads.apply_params(eng, 0, p)
    dev = eng.device
    par = {k: p[k].clone().requires_grad_(True) for k in ("taurad", "taudrag", "DPhieq")}
    par["Phibar"] = torch.full((2,), p["Phibar"], dtype=torch.float64, device=dev, requires_grad=True)
    ic = wl["ics"].clone().requires_grad_(True)
    out = integrate(eng, flags, 2, nsteps, [par], [ic], ckpt_every=25)[0]
    loss = torch.mean((out[2] - target) ** 2)
    loss.backward()

    def L(**kw):
        q = dict(p)
        q.update(kw)
        workloads.apply_params(eng, 0, q)
        eng.init_state([wl["ics"]], flags)
        eng.forward(flags, t0=2, nsteps=nsteps)
        res = eng.output_physical(flags)[0][2]
        workloads.apply_params(eng, 0, p)
        return ((res - target) ** 2).mean(dim=(1, 2))  # per member (members are independent)

    for name in ("taurad", "DPhieq"):
        h = 1e-4 * p[name]
        lp = L(**{name: p[name] + h})
        lm = L(**{name: p[name] - h})
        # d(mean over members)/d(member param) = (1/B) d(member loss)/d(param)
        fd = ((lp - lm) / (2 * h) / 2).cpu().numpy()
        ad = par[name].grad.cpu().numpy()
        np.testing.assert_allclose(ad, fd, rtol=1e-5, err_msg=name)
