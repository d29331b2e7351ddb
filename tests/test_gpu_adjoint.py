"""Hand-written adjoint (through the C ABI) against torch autograd through the
CPU oracle and against central finite differences of the GPU forward.
Tolerances: gradient fields within 1e-8 of their max (FP64 on both sides);
parameter gradients within 1e-6 relative of central FD (h = 1e-6 relative)."""
import numpy as np
import pytest

from oracle import swampe_oracle as o

pytestmark = pytest.mark.gpu


def _case(M=42, seed=0):
    geo = o.cached_geometry(M)
    J, I = geo["J"], geo["I"]
    rng = np.random.default_rng(seed)
    mu = geo["mus"][:, None]
    omega, a, Phibar = 3.2e-5, 8.2e7, 3.0e5
    eta0 = 2 * omega * mu * np.ones((1, I))
    lam = np.linspace(-np.pi, np.pi, I, endpoint=False)[None, :]
    Phi0 = 2e3 * np.cos(lam) * np.sqrt(1 - mu**2) + 50.0 * rng.standard_normal((J, I))
    delta0 = 1e-9 * rng.standard_normal((J, I))
    U0 = 5.0 * np.sqrt(1 - mu**2) * np.ones((1, I)) + 0.1 * rng.standard_normal((J, I))
    V0 = 0.1 * rng.standard_normal((J, I))
    params = dict(dt=1200.0, a=a, omega=omega, Phibar=Phibar, taurad=36000.0, taudrag=21600.0, DPhieq=1.0e6,
                  K6=1.24e33)
    W = rng.standard_normal((5, J, I))
    return params, (eta0, delta0, Phi0, U0, V0), W


def _gpu_grads(params, ics, W, nsteps, ckpt_every, M=42, precision="fp64", store="checkpoint", scheme=0):
    import torch
    from my_swampe_gb300.engine import Engine, RunFlagsC
    from my_swampe_gb300.adjoint import integrate

    eng = Engine([(M, 1)], precision)
    eng.set_params(0, dt=params["dt"], a=params["a"], omega=params["omega"], K6=params["K6"],
                   K6Phi=params["K6"], alpha=0.01)
    dev = eng.device
    p = {k: torch.tensor([params[k]], dtype=torch.float64, device=dev, requires_grad=True)
         for k in ("taurad", "taudrag", "DPhieq", "Phibar")}
    ic = torch.tensor(np.stack(ics)[:, None], dtype=torch.float64, device=dev, requires_grad=True)
    out = integrate(eng, RunFlagsC(scheme=scheme), t0=2, nsteps=nsteps, params=[p], ics=[ic], ckpt_every=ckpt_every,
                    store=store)[0]
    Wt = torch.tensor(W[:, None], dtype=torch.float64, device=dev)
    loss = (out.double() * Wt).sum()
    loss.backward()
    return float(loss.detach()), {k: float(v.grad[0]) for k, v in p.items()}, ic.grad[:, 0].cpu().numpy()


def _oracle_grads(params, ics, W, nsteps, M=42, expflag=False, semi_implicit=False):
    import torch

    xp = o.torch_backend()
    p = {k: torch.tensor(params[k], dtype=torch.float64, requires_grad=True) for k in ("taurad", "taudrag", "DPhieq", "Phibar")}
    ic = [torch.tensor(x, dtype=torch.float64, requires_grad=True) for x in ics]
    r = o.run_model_scan_final(xp, M=M, dt=params["dt"], tmax=2 + nsteps, Phibar=p["Phibar"], omega=params["omega"],
                               a=params["a"], test=None, taurad=p["taurad"], taudrag=p["taudrag"], DPhieq=p["DPhieq"],
                               K6=params["K6"], eta0_init=ic[0], delta0_init=ic[1], Phi0_init=ic[2], U0_init=ic[3],
                               V0_init=ic[4], expflag=expflag, semi_implicit=semi_implicit)["last_state"]
    outs = [r[f + "_curr"] for f in ("eta", "delta", "Phi", "U", "V")]
    loss = sum((x * torch.tensor(W[k])).sum() for k, x in enumerate(outs))
    loss.backward()
    return float(loss.detach()), {k: float(v.grad) for k, v in p.items()}, np.stack([x.grad.numpy() for x in ic])


def test_adjoint_matches_torch_autograd_through_oracle(cuda):
    params, ics, W = _case()
    nsteps = 4
    lg, pg, icg = _gpu_grads(params, ics, W, nsteps, ckpt_every=3)
    lo, po, ico = _oracle_grads(params, ics, W, nsteps)
    assert abs(lg - lo) <= 1e-9 * abs(lo)
    for k in po:
        assert abs(pg[k] - po[k]) <= 1e-7 * max(abs(po[k]), 1e-300), (k, pg[k], po[k])
    for f in range(5):
        scale = np.max(np.abs(ico[f]))
        err = np.max(np.abs(icg[f] - ico[f]))
        assert err <= 1e-8 * scale, (f, err, scale)


@pytest.mark.parametrize("store", ["checkpoint", "all"])
def test_explicit_adjoint_matches_torch_autograd_through_oracle(cuda, store):
    """The explicit leapfrog's hand-written adjoint (transposed combination of
    explicit_tdiff.py, the Fourier prev carry, its own drag terms in the taudrag
    gradient) against torch autograd through the oracle's expflag path: the
    loss, the four parameter gradients and the initial-field gradients."""
    params, ics, W = _case(seed=5)
    params = dict(params, dt=300.0)
    nsteps = 5
    lg, pg, icg = _gpu_grads(params, ics, W, nsteps, ckpt_every=3, store=store, scheme=1)
    lo, po, ico = _oracle_grads(params, ics, W, nsteps, expflag=True)
    assert abs(lg - lo) <= 1e-9 * abs(lo)
    for k in po:
        assert abs(pg[k] - po[k]) <= 1e-7 * max(abs(po[k]), 1e-300), (k, pg[k], po[k])
    for f in range(5):
        scale = np.max(np.abs(ico[f]))
        err = np.max(np.abs(icg[f] - ico[f]))
        assert err <= 1e-8 * scale, (f, err, scale)


@pytest.mark.parametrize("store", ["checkpoint", "all"])
def test_semi_implicit_adjoint_matches_torch_autograd_through_oracle(cuda, store):
    """The semi-implicit scheme's adjoint (its transposed per-degree solve, the
    filtered mid carry and the lagged remainders) gives the initial-field
    gradients; the parameter gradients come from tangent runs.  Against torch
    autograd through the oracle's semi_implicit path, 6 steps (the first with
    the lag initialisation, the later ones with the Robert-Asselin update)."""
    params, ics, W = _case(seed=6)
    nsteps = 6
    lg, pg, icg = _gpu_grads(params, ics, W, nsteps, ckpt_every=4, store=store, scheme=2)
    lo, po, ico = _oracle_grads(params, ics, W, nsteps, semi_implicit=True)
    assert abs(lg - lo) <= 1e-9 * abs(lo)
    for k in po:
        assert abs(pg[k] - po[k]) <= 1e-7 * max(abs(po[k]), 1e-300), (k, pg[k], po[k])
    for f in range(5):
        scale = np.max(np.abs(ico[f]))
        err = np.max(np.abs(icg[f] - ico[f]))
        assert err <= 1e-8 * scale, (f, err, scale)


def test_adjoint_checkpoint_window_invariance(cuda):
    params, ics, W = _case(seed=1)
    ref = _gpu_grads(params, ics, W, 7, ckpt_every=7)
    for K in (1, 3):
        got = _gpu_grads(params, ics, W, 7, ckpt_every=K)
        for k in ref[1]:
            assert abs(got[1][k] - ref[1][k]) <= 1e-12 * abs(ref[1][k]) + 1e-300
        np.testing.assert_allclose(got[2], ref[2], rtol=0, atol=1e-12 * np.max(np.abs(ref[2])))


@pytest.mark.parametrize("scheme", [0, 1])
def test_param_gradients_match_central_fd(cuda, scheme):
    """unit_tests/test_autodiff.py:102-129 style central differences of the GPU
    forward.  With h = 1e-6 relative the difference quotient is limited by the
    forward's own round-off (~1e-10 per grid value, summed over 40k values),
    so it is checked to 5e-3; with h = 1e-4 relative (truncation error ~h^2)
    it is checked to 2e-5.  Scheme 1 is the explicit leapfrog (dt = 300 s)."""
    import torch
    from my_swampe_gb300.engine import Engine, RunFlagsC

    params, ics, W = _case(seed=2)
    if scheme == 1:
        params = dict(params, dt=300.0)
    nsteps = 6
    _, pg, _ = _gpu_grads(params, ics, W, nsteps, ckpt_every=4, scheme=scheme)
    eng = Engine([(42, 2)], "fp64")
    eng.set_params(0, dt=params["dt"], a=params["a"], omega=params["omega"], K6=params["K6"], K6Phi=params["K6"], alpha=0.01)
    Wt = torch.tensor(W, device=eng.device)
    ic = torch.tensor(np.stack(ics)[:, None], dtype=torch.float64, device=eng.device).expand(5, 2, *W.shape[1:]).contiguous()
    flags = RunFlagsC(scheme=scheme)
    for k in ("taurad", "taudrag", "DPhieq", "Phibar"):
        assert pg[k] != 0.0
        for rel_h, tol in ((1e-6, 5e-3), (1e-4, 2e-5)):
            base = {q: params[q] for q in ("taurad", "taudrag", "DPhieq", "Phibar")}
            h = rel_h * abs(params[k])
            vals = {q: torch.tensor([base[q], base[q]], dtype=torch.float64) for q in base}
            vals[k] = torch.tensor([params[k] + h, params[k] - h], dtype=torch.float64)
            eng.set_params(0, **vals)
            eng.init_state([ic], flags)
            eng.forward(flags, t0=2, nsteps=nsteps)
            out = eng.output_physical(flags)[0][:5]
            fd = float(((out[:, 0] - out[:, 1]) * Wt).sum()) / (2 * h)
            assert abs(pg[k] - fd) <= tol * abs(fd), (k, rel_h, pg[k], fd)


def test_fast_adjoint_matches_fp64_adjoint(cuda):
    """The FP32 adjoint (incremental steps after the first) against the FP64 one."""
    params, ics, W = _case(seed=4)
    l64, p64, ic64 = _gpu_grads(params, ics, W, 12, ckpt_every=5, precision="fp64")
    l32, p32, ic32 = _gpu_grads(params, ics, W, 12, ckpt_every=5, precision="fast")
    for k in p64:
        assert abs(p32[k] - p64[k]) <= 2e-4 * abs(p64[k]), (k, p32[k], p64[k])
    for f in range(5):
        scale = np.max(np.abs(ic64[f]))
        rel = np.linalg.norm(ic32[f] - ic64[f]) / max(np.linalg.norm(ic64[f]), 1e-300)
        assert rel <= 2e-4, (f, rel)


@pytest.mark.parametrize("precision", ["fp64", "fast"])
def test_stored_states_adjoint_matches_checkpointed(cuda, precision):
    """The adjoint over stored states (no recomputation) equals the checkpointed
    adjoint: same loss bit for bit, same initial-field gradients bit for bit
    (no atomics on that path), parameter gradients to the order of their FP64
    atomic reductions."""
    params, ics, W = _case(seed=4)
    loss_a, g_a, ic_a = _gpu_grads(params, ics, W, nsteps=23, ckpt_every=5, precision=precision, store="all")
    loss_c, g_c, ic_c = _gpu_grads(params, ics, W, nsteps=23, ckpt_every=5, precision=precision, store="checkpoint")
    assert loss_a == loss_c
    np.testing.assert_array_equal(ic_a, ic_c)
    for k in g_a:
        assert abs(g_a[k] - g_c[k]) <= 1e-12 * max(abs(g_c[k]), 1e-300), (k, g_a[k], g_c[k])


def test_unforced_out_of_place_steps_ignore_stale_memory(cuda):
    """Unforced (test = 2) runs: the out-of-place steps of the stored-states form
    and of the checkpointed form's window recompute write zero forcing terms
    instead of leaving a slot's previous contents (the caching allocator hands
    back dirty memory): both forms give the in-place forward and one gradient."""
    import torch
    from my_swampe_gb300 import adjoint, run_model_scan_final
    from my_swampe_gb300.engine import Engine, RunFlagsC
    from my_swampe_gb300.model import _analytic_ic

    kw = dict(M=42, dt=600.0, omega=7.2921159e-5, a=6.37122e6, test=2, forcflag=False, Phibar=3.0e3)
    ref = run_model_scan_final(**kw, tmax=8)["last_state"]
    f = _analytic_ic(42, 6.37122e6, 7.2921159e-5, 3.0e3, 2, 0.05, torch.device("cuda"))
    grads = {}
    for store in ("all", "checkpoint"):
        junk = torch.full((64 * 1024 * 1024,), 1e30, dtype=torch.float64, device="cuda")  # 512 MB of garbage
        del junk
        eng = Engine([(42, 1)], "fp64")
        eng.set_params(0, dt=600.0, a=6.37122e6, omega=7.2921159e-5, K6=1.24e33, K6Phi=1.24e33, alpha=0.01)
        ics = torch.stack(f, 0)[:, None].clone().requires_grad_(True)
        params = dict(taurad=torch.full((1,), 86400.0, dtype=torch.float64, device="cuda"),
                      taudrag=torch.full((1,), 86400.0, dtype=torch.float64, device="cuda"),
                      DPhieq=torch.zeros(1, dtype=torch.float64, device="cuda"),
                      Phibar=torch.full((1,), 3.0e3, dtype=torch.float64, device="cuda"))
        out = adjoint.integrate(eng, RunFlagsC(test=2, forcflag=False), 2, 6, [params], [ics], ckpt_every=2,
                                store=store)[0]
        for k, name in enumerate(("eta_curr", "delta_curr", "Phi_curr", "U_curr", "V_curr")):
            want = getattr(ref, name)
            err = float((out[k, 0] - want).abs().max())
            assert err <= 1e-9 * float(want.abs().max()) + 1e-300, (store, name, err)
        grads[store] = torch.autograd.grad((out ** 2).sum(), ics)[0]
    assert bool(torch.all(torch.isfinite(grads["all"])))
    torch.testing.assert_close(grads["all"], grads["checkpoint"], rtol=1e-10, atol=1e-300)
