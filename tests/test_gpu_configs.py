"""The benchmark workloads as GPU tests:
  steady zonal geostrophic flow, M=42, one member (test=2 regime, explicit ICs)
  forced single member, M=42, FP64, 28,800 steps (10 days at dt = 30 s): the
    oracle over a 50-step prefix at the reference's tolerances, then finite
    and ungated to the end
  forced ensemble, M=42, B=8, 1440 steps: the fast path's error against the
    FP64 path (relative L2 of Phi <= 1e-5)
  M=63 ensemble of 32, 2000 steps, checkpoints every 50: gradients of
    mean((Phi_T - Phi_target)^2) in FP64 and in the fast precision against
    central differences
  mixed truncations (M=42, 63, 106) in one launch == separate launches, and the
    64 / 32 / 8 member mixed ensemble over 1440 steps in the fast precision with
    its error per group against FP64
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


def _forced_single_ics(seed=2024):
    """Config 2's initial state: rest (eta = 2 Omega mu, delta = U = V = 0) with
    Phi = seeded Gaussian noise of amplitude 1e-3 Phibar on the spectral
    coefficients with n <= 10."""
    geo = o.cached_geometry(42)
    J, I = geo["J"], geo["I"]
    mu = geo["mus"][:, None] * np.ones((1, I))
    rng = np.random.default_rng(seed)
    c = np.zeros((43, 43), complex)
    for m in range(11):
        for n in range(m, 11):
            c[m, n] = 1e-3 * 4.0e6 * (rng.standard_normal() + (1j * rng.standard_normal() if m > 0 else 0.0))
    Phi0 = np.real(o.invrs_fft(o.NUMPY, o.invrs_leg(o.NUMPY, c, I, 42, geo["Pmn"]), I))
    z = np.zeros((J, I))
    return dict(eta0_init=2 * 3.2e-5 * mu, delta0_init=z, Phi0_init=Phi0, U0_init=z, V0_init=z)


def test_forced_single_member_ten_days(cuda):
    """B=1, FP64, forced synchronously rotating regime (a = 8.2e7, Omega =
    3.2e-5, Phibar = DPhieq = 4e6, taurad = taudrag = 1 day, dt = 30 s), 28,800
    steps.  The first 50 steps against the oracle at the reference's
    tolerances (same quadrature; Phi reaches 4.5e4 here, so FP64 round-off of
    1e-12 relative is already 4.5e-8 absolute: after 100 steps it was 6.4e-8);
    the whole run finite, never gated, with Phi within the forcing's range."""
    import torch
    from conftest import ATOL, exact_quadrature
    from my_swampe_gb300 import run_model_scan, run_model_scan_final

    kw = dict(M=42, dt=30.0, Phibar=4.0e6, omega=3.2e-5, a=8.2e7, test=None, taurad=86400.0, taudrag=86400.0,
              DPhieq=4.0e6, **_forced_single_ics())
    g = run_model_scan(tmax=2 + 50, **kw)
    with exact_quadrature():
        r = o.run_model_scan(tmax=2 + 50, record=("Phi",), **kw)
    assert int(g["dead_first_idx"]) == -1 and r["dead_first_idx"] == -1
    for f in ("eta", "delta", "Phi", "U", "V"):
        np.testing.assert_allclose(getattr(g["last_state"], f + "_curr").cpu().numpy(),
                                   np.asarray(r["last_state"][f + "_curr"]), rtol=0, atol=ATOL[f], err_msg=f)
    np.testing.assert_allclose(g["outs"]["Phi"].cpu().numpy(), np.asarray(r["outs"]["Phi"]), rtol=0, atol=ATOL["Phi"])
    full = run_model_scan(tmax=2 + 28800, return_history=False, diagnostics=True, **kw)
    last = full["last_state"]
    assert not bool(last.dead)
    for f in ("eta_curr", "delta_curr", "Phi_curr", "U_curr", "V_curr"):
        assert bool(torch.isfinite(getattr(last, f)).all()), f
    # Phi + Phibar relaxes towards Phieq in [Phibar, Phibar + DPhieq]
    phi = last.Phi_curr
    assert float(phi.min()) > -4.0e6 and float(phi.max()) < 2 * 4.0e6
    fin = run_model_scan_final(tmax=2 + 28800, **kw)["last_state"]
    assert torch.equal(fin.Phi_curr, last.Phi_curr)


def test_fast_path_error_after_1440_steps(cuda):
    """Forced ensemble (B=8, the benchmark's regime and parameter sampling),
    1440 steps: the fast path (FP32 state, tensor-core Legendre kernels)
    against the FP64 path.  Relative L2 bounds: Phi 1e-5 (the split-precision
    path's accuracy target), eta 1e-5, delta 5e-5 (the smallest field); the same for the
    Robert-Asselin filtered (prev) fields."""
    import torch
    from my_swampe_gb300 import workloads
    from my_swampe_gb300.engine import Engine, RunFlagsC

    outs = {}
    for prec in ("fp64", "fast"):
        eng = Engine([(42, 8)], prec)
        if prec == "fast":
            assert eng.uses_tensor_cores
        wl = workloads.forced_ensemble(eng, seed=1234)
        workloads.apply_params(eng, 0, wl["params"])
        flags = RunFlagsC()
        eng.init_state([wl["ics"]], flags)
        eng.forward(flags, t0=2, nsteps=1440)
        eng.check_device_status()
        outs[prec] = eng.output_physical(flags)[0].double()
    for k, name, tol in ((0, "eta", 1e-5), (1, "delta", 5e-5), (2, "Phi", 1e-5), (5, "eta_prev", 1e-5),
                         (6, "delta_prev", 5e-5), (7, "Phi_prev", 1e-5)):
        ref = outs["fp64"][k]
        rel = float(torch.linalg.vector_norm(outs["fast"][k] - ref) / torch.linalg.vector_norm(ref))
        assert rel <= tol, (name, rel)


def _m63_losses(eng, wl, p, target, nsteps):
    from my_swampe_gb300 import workloads
    from my_swampe_gb300.engine import RunFlagsC

    flags = RunFlagsC()
    workloads.apply_params(eng, 0, p)
    eng.init_state([wl["ics"].to(eng.rdtype)], flags)
    eng.forward(flags, t0=2, nsteps=nsteps)
    res = eng.output_physical(flags)[0][2].double()
    return ((res - target) ** 2).mean(dim=(1, 2))  # per member (members are independent)


@pytest.mark.parametrize("precision", ["fp64", "fast"])
def test_M63_ensemble_of_32_gradients_2000_steps(cuda, precision):
    """M=63 (96 x 192), B=32 forced, dt = 20 s, 2000 steps, checkpoints every
    50: gradients of mean((Phi_T - Phi_target)^2) (target: a run at taurad x1.1,
    DPhieq x0.9) in taurad, taudrag, DPhieq, Phibar against central differences
    of the FP64 forward (h = 1e-6 relative) on members 0, 7, 19, 31.

    A central difference over 2000 steps carries the round-off of the two runs
    divided by 2h; it is measured as the change of the difference between
    steps h and 2h (the truncation error is ~h^2, far below it), and allowed
    twice.  FP64 adjoint: |ad - fd| <= 1e-5 |fd| + 2 noise.  Fast precision
    (FP32 state, tensor-core 3xTF32 Legendre kernels, its own adjoint): 1e-3
    relative L2 over the members, and per member 5e-2 |fd| + 2 noise: the
    smallest member gradient (taudrag of member 0, 2.7e-4 against 11.7 for
    member 31) is a cancellation of much larger terms, which the FP32 rounding
    leaves within 4%."""
    import torch
    from my_swampe_gb300 import workloads
    from my_swampe_gb300.adjoint import integrate
    from my_swampe_gb300.engine import Engine, RunFlagsC

    B, nsteps = 32, 2000
    e64 = Engine([(63, B)], "fp64")
    wl = workloads.forced_ensemble(e64, seed=63, dt=20.0)
    p = dict(wl["params"])
    p["Phibar"] = torch.full((B,), float(p["Phibar"]), dtype=torch.float64, device=e64.device)
    p_tgt = dict(p, taurad=p["taurad"] * 1.1, DPhieq=p["DPhieq"] * 0.9)
    target = None
    flags = RunFlagsC()
    workloads.apply_params(e64, 0, p_tgt)
    e64.init_state([wl["ics"]], flags)
    e64.forward(flags, t0=2, nsteps=nsteps)
    target = e64.output_physical(flags)[0][2].clone()
    eng = e64 if precision == "fp64" else Engine([(63, B)], "fast")
    workloads.apply_params(eng, 0, p)
    par = {k: p[k].clone().requires_grad_(True) for k in ("taurad", "taudrag", "DPhieq", "Phibar")}
    ic = wl["ics"].to(eng.rdtype).clone().requires_grad_(True)
    out = integrate(eng, flags, 2, nsteps, [par], [ic], ckpt_every=50, store="checkpoint")[0]
    loss = torch.mean((out[2].double() - target) ** 2)
    loss.backward()
    members = [0, 7, 19, 31]
    tol = 1e-5 if precision == "fp64" else 5e-2

    def fd_at(name, h):
        lp = _m63_losses(e64, wl, dict(p, **{name: p[name] + h}), target, nsteps)
        lm = _m63_losses(e64, wl, dict(p, **{name: p[name] - h}), target, nsteps)
        return ((lp - lm) / (2 * h) / B).cpu().numpy()

    for name in ("taurad", "taudrag", "DPhieq", "Phibar"):
        h = 1e-6 * p[name].abs()
        fd = fd_at(name, h)[members]
        noise = np.abs(fd - fd_at(name, 2 * h)[members])
        ad = par[name].grad.cpu().numpy()[members]
        err = np.abs(ad - fd)
        assert np.all(err <= tol * np.abs(fd) + 2 * noise), (precision, name, ad, fd, noise)
        if precision == "fast":
            assert np.linalg.norm(ad - fd) <= 1e-3 * np.linalg.norm(fd), (name, ad, fd)
    assert np.isfinite(ic.grad.cpu().numpy()).all()


def test_mixed_truncations_1440_steps_fast_vs_fp64(cuda):
    """64 members at M=42 (dt 30 s), 32 at M=63 (dt 20 s) and 8 at M=106
    (dt 12 s), forced, parameters sampled per member, in one plan (tensor-core
    Legendre kernels for every group): the fast path against the
    FP64 path, relative L2 per group after 1440 steps (bounds: Phi, eta 1e-5;
    delta 5e-5).

    At M=106 the reference's own FP64 algorithm is unstable in this regime: its
    damaged basis (the scaling-table underflow it reproduces) makes the
    forward-inverse Legendre round trip amplify modes m = 80..89 (eigenvalue
    1.33 at m = 83, test_oracle_golden.py), so the FP64 run overflows after
    ~150 steps.  The fast path's incremental steps transform only the
    increment, so they neither amplify those modes nor re-project them as the
    reference does: the group is compared after 50 steps, where the FP64 run is
    still clean (observed Phi 5.4e-6, eta 2.6e-7, delta 4.4e-4: delta carries
    the most content at those modes; bound 1e-3), and must stay finite to 1440."""
    import torch
    from my_swampe_gb300 import workloads
    from my_swampe_gb300.engine import Engine, RunFlagsC

    spec = [(42, 64, 30.0), (63, 32, 20.0), (106, 8, 12.0)]
    outs = {}
    for prec in ("fp64", "fast"):
        eng = Engine([(M, B) for M, B, _ in spec], prec)
        if prec == "fast":
            assert eng.tensor_core_groups == [0, 1, 2]
        ics = []
        for g, (M, B, dt) in enumerate(spec):
            wl = workloads.forced_ensemble(eng, g=g, seed=500 + 1000 * g, dt=dt)
            workloads.apply_params(eng, g, wl["params"])
            ics.append(wl["ics"])
        flags = RunFlagsC()
        eng.init_state(ics, flags)
        eng.forward(flags, t0=2, nsteps=50)
        early = [o_.double() for o_ in eng.output_physical(flags)]
        eng.forward(flags, t0=52, nsteps=1390)
        eng.check_device_status()
        outs[prec] = (early, [o_.double() for o_ in eng.output_physical(flags)])
    for g, (M, B, _) in enumerate(spec):
        at = 0 if M == 106 else 1
        bounds = ((0, "eta", 1e-5), (1, "delta", 1e-3 if M == 106 else 5e-5), (2, "Phi", 1e-5))
        for k, name, tol in bounds:
            ref = outs["fp64"][at][g][k]
            rel = float(torch.linalg.vector_norm(outs["fast"][at][g][k] - ref) / torch.linalg.vector_norm(ref))
            assert rel <= tol, (M, name, rel)
    assert bool(torch.isfinite(outs["fast"][1][2]).all())
