"""The tangent-linear (forward-mode) model on the GPU, the counterpart of
jax.jvp / jax.jacfwd through run_model_scan (autodiff_utils.py:27-89 fwd_grad):
against central differences of the FP64 forward, against the hand-written
adjoint by the dot-product identity <w, J v> = <J^T w, v>, and fwd_grad
against the reverse-mode gradient."""
import pytest
import torch
import torch.autograd.forward_ad as fwAD

from my_swampe_gb300._lib import NTANGENT as NTAN

pytestmark = pytest.mark.gpu

NSTEPS = 12


def _setup(prec="fp64", B=2, test=None, seed=5):
    from my_swampe_gb300 import workloads
    from my_swampe_gb300.engine import Engine, RunFlagsC

    eng = Engine([(42, B)], prec)
    wl = workloads.forced_ensemble(eng, dt=600.0, Phibar=3.0e5, seed=seed)
    flags = RunFlagsC(test=test, diagnostics=False, t_start=2)
    g = torch.Generator(device="cpu").manual_seed(seed)
    ics = wl["ics"]
    # a smooth direction: the ICs' own structure with random member weights, plus
    # a smooth Phi pattern
    w = torch.rand((5, B, 1, 1), generator=g, dtype=torch.float64).to(eng.device) - 0.5
    dics = (ics * w).contiguous()
    dics[2] += 1e-2 * wl["ics"][2].flip(-1)
    p = wl["params"]
    dpar = torch.zeros((NTAN, B), dtype=torch.float64, device=eng.device)
    dpar[:4] = torch.stack([0.1 * p["taurad"], 0.1 * p["taudrag"], 0.1 * p["DPhieq"],
                            torch.full((B,), 0.05 * 3.0e5, dtype=torch.float64, device=eng.device)])
    dpar[:4] *= torch.rand((4, B), generator=g, dtype=torch.float64).to(eng.device) - 0.5
    return eng, flags, wl, ics, dics, dpar


# the parameters that enter only the coefficient tables: tangent row, direction
# scale, and the centred-difference step (their effect over 12 steps is small
# next to the fields, so a step too small leaves the difference to round-off:
# the error of these steps is <= 1e-6 except K6, K6Phi at <= 1e-6 .. 1e-5)
COEF_PARAMS = (("a", 4, 1e-2, 1e-4), ("dt", 5, 1e-2, 1e-4), ("K6", 6, 1e-1, 1e-2), ("K6Phi", 7, 1e-1, 1e-2),
               ("omega", 8, 1e-1, 1e-5))


def _forward(eng, flags, wl, ics, params_shift=None, h=0.0):
    from my_swampe_gb300 import workloads

    p = dict(wl["params"])
    if params_shift is not None:
        names = ("taurad", "taudrag", "DPhieq", "Phibar", "a", "dt", "K6", "K6Phi", "omega", "si_alpha", "alpha",
                 "williams_alpha")
        defaults = dict(si_alpha=0.5, alpha=0.01, williams_alpha=0.53)
        for k in range(params_shift.shape[0]):
            name = names[k]
            if name not in p:
                p[name] = defaults[name]
            p[name] = p[name] + h * params_shift[k]
    workloads.apply_params(eng, 0, p)
    eng.init_state([ics.to(eng.rdtype)], flags)
    eng.forward(flags, t0=2, nsteps=NSTEPS)
    return eng.output_physical(flags)[0][:5].double()


def _tangent(eng, flags, wl, ics, dics, dpar):
    from my_swampe_gb300 import workloads

    workloads.apply_params(eng, 0, wl["params"])
    eng.init_state([ics.to(eng.rdtype)], flags)
    tf, tr, _ = eng.new_tangent_buffers()
    eng.tangent_init(flags, [ics], [dics], tf, tr, [dpar])
    eng.tangent_forward(flags, 2, NSTEPS, tf, tr, [dpar])
    return eng.tangent_output(flags, tf, tr, [dpar])[0][:5].double()


@pytest.mark.parametrize("test", [None, 2])
def test_tangent_matches_central_differences(cuda, test):
    eng, flags, wl, ics, dics, dpar = _setup(test=test)
    tl = _tangent(eng, flags, wl, ics, dics, dpar)
    h = 1e-6
    fp = _forward(eng, flags, wl, ics + h * dics, dpar, h)
    fm = _forward(eng, flags, wl, ics - h * dics, dpar, -h)
    fd = (fp - fm) / (2 * h)
    for k, name in enumerate(("eta", "delta", "Phi", "U", "V")):
        rel = float(torch.linalg.norm(tl[k] - fd[k]) / torch.linalg.norm(fd[k]))
        assert rel < 2e-6, (name, rel)


@pytest.mark.parametrize("name,row,scale,h", COEF_PARAMS)
def test_coefficient_tangents_match_central_differences(cuda, name, row, scale, h):
    """Tangents along a, dt, K6, K6Phi, omega (they enter the step only through
    its coefficient tables) against central differences of the FP64 forward."""
    eng, flags, wl, ics, _, _ = _setup()
    p = wl["params"]
    base = float(p.get(name, p["K6"]))
    dpar = torch.zeros((NTAN, 2), dtype=torch.float64, device=eng.device)
    dpar[row] = torch.tensor([scale * base, -0.5 * scale * base], dtype=torch.float64)
    zero = torch.zeros_like(ics)
    tl = _tangent(eng, flags, wl, ics, zero, dpar)
    fd = (_forward(eng, flags, wl, ics, dpar, h) - _forward(eng, flags, wl, ics, dpar, -h)) / (2 * h)
    for k, fname in enumerate(("eta", "delta", "Phi", "U", "V")):
        nrm = float(torch.linalg.norm(fd[k]))
        rel = float(torch.linalg.norm(tl[k] - fd[k])) / max(nrm, 1e-300)
        assert rel < 1e-5, (name, fname, rel, nrm)


def test_coefficient_gradients_by_reverse_mode(cuda):
    """Reverse-mode gradients with respect to a, dt, K6, K6Phi, omega through
    integrate (one tangent run per parameter) against central differences."""
    from my_swampe_gb300 import adjoint, workloads

    eng, flags, wl, ics, _, _ = _setup()
    workloads.apply_params(eng, 0, wl["params"])
    p = wl["params"]
    wgt = torch.randn((5, 2, 64, 128), dtype=torch.float64, device=eng.device)
    vals = {k: torch.full((2,), float(p.get(k, p["K6"])), dtype=torch.float64, device=eng.device)
            for k in ("a", "dt", "K6", "K6Phi", "omega")}
    base = {k: (p[k] if torch.is_tensor(p[k]) else torch.full((2,), float(p[k]), dtype=torch.float64,
                                                               device=eng.device))
            for k in ("taurad", "taudrag", "DPhieq", "Phibar")}
    xs = {k: v.clone().requires_grad_(True) for k, v in vals.items()}
    out = adjoint.integrate(eng, flags, 2, NSTEPS, [dict(base, **xs)], [ics], store="all")[0]
    grads = torch.autograd.grad((wgt * out).sum(), [xs[k] for k in vals])
    rel_h = dict(a=1e-5, dt=1e-5, K6=1e-3, K6Phi=1e-3, omega=1e-5)
    for (k, v), gk in zip(vals.items(), grads):
        h = rel_h[k] * float(v[0])
        with torch.no_grad():
            lp = float((wgt * adjoint.integrate(eng, flags, 2, NSTEPS, [dict(base, **dict(vals, **{k: v + h}))],
                                                [ics], store="all")[0]).sum())
            lm = float((wgt * adjoint.integrate(eng, flags, 2, NSTEPS, [dict(base, **dict(vals, **{k: v - h}))],
                                                [ics], store="all")[0]).sum())
        fd = (lp - lm) / (2 * h)  # both members perturbed together: the sum of their gradients
        # the tangent model itself is pinned above; this checks the reverse-mode plumbing
        assert abs(float(gk.sum()) - fd) <= 1e-3 * abs(fd), (k, float(gk.sum()), fd)


@pytest.mark.parametrize("scheme", [0, 1, 2])
def test_tangent_adjoint_dot_product(cuda, scheme):
    """<w, J v> from the tangent model equals <J^T w, v> from the adjoint (FP64),
    for the modified-Euler, explicit and semi-implicit schemes (the last one's
    reverse-mode parameter terms are tangent runs, its initial-field terms the
    adjoint)."""
    from my_swampe_gb300 import adjoint
    from my_swampe_gb300.engine import RunFlagsC

    eng, flags, wl, ics, dics, dpar = _setup()
    flags = RunFlagsC(scheme=scheme, diagnostics=False, t_start=2)
    p = wl["params"]
    names = ("taurad", "taudrag", "DPhieq", "Phibar")
    base = {k: (p[k] if torch.is_tensor(p[k]) else torch.full((2,), float(p[k]), dtype=torch.float64,
                                                               device=eng.device)) for k in names}
    from my_swampe_gb300 import workloads

    workloads.apply_params(eng, 0, p)
    wgt = torch.randn((5, 2, 64, 128), dtype=torch.float64, device=eng.device)
    # reverse: J^T w
    xs = {k: base[k].clone().requires_grad_(True) for k in names}
    x0 = ics.clone().requires_grad_(True)
    out = adjoint.integrate(eng, flags, t0=2, nsteps=NSTEPS, params=[xs], ics=[x0], store="all")[0]
    grads = torch.autograd.grad((wgt * out).sum(), [x0] + [xs[k] for k in names])
    lhs = float((grads[0] * dics).sum()) + sum(float((grads[1 + k] * dpar[k]).sum()) for k in range(4))
    # forward: J v
    with fwAD.dual_level():
        dual_p = {k: fwAD.make_dual(base[k], dpar[i].contiguous()) for i, k in enumerate(names)}
        dual_x = fwAD.make_dual(ics, dics)
        out2 = adjoint.integrate(eng, flags, t0=2, nsteps=NSTEPS, params=[dual_p], ics=[dual_x], store="all")[0]
        jv = fwAD.unpack_dual(out2).tangent
    rhs = float((wgt * jv).sum())
    assert abs(lhs - rhs) <= 1e-10 * max(abs(lhs), abs(rhs)), (lhs, rhs)


def test_fwd_grad_matches_reverse_mode(cuda):
    """autodiff_utils.fwd_grad (forward mode, one tangent run per parameter)
    against torch.autograd.grad through the adjoint, for a shared parameter vector."""
    from my_swampe_gb300 import adjoint, workloads
    from my_swampe_gb300.autodiff_utils import fwd_grad

    eng, flags, wl, ics, _, _ = _setup()
    workloads.apply_params(eng, 0, wl["params"])
    target = _forward(eng, flags, wl, ics)[2] * 1.01
    integ = adjoint.Integration(eng, flags, 2, NSTEPS, store="all")

    def loss_fn(theta):
        params = dict(taurad=theta[0] * torch.ones(2, dtype=torch.float64, device=eng.device),
                      taudrag=theta[1] * torch.ones(2, dtype=torch.float64, device=eng.device),
                      DPhieq=theta[2] * torch.ones(2, dtype=torch.float64, device=eng.device),
                      Phibar=theta[3] * torch.ones(2, dtype=torch.float64, device=eng.device))
        out = adjoint.integrate(eng, flags, 2, NSTEPS, [params], [ics], integration=integ)[0]
        return ((out[2] - target) ** 2).mean()

    theta = torch.tensor([36000.0, 21600.0, 1.0e6, 3.0e5], dtype=torch.float64, device=eng.device)
    g_fwd = fwd_grad(loss_fn, theta)
    th = theta.clone().requires_grad_(True)
    g_rev = torch.autograd.grad(loss_fn(th), th)[0]
    rel = (g_fwd - g_rev).abs() / g_rev.abs()
    assert bool(torch.all(rel < 1e-8)), (g_fwd, g_rev)


@pytest.mark.parametrize("chunk", [None, 3])
def test_batched_fwd_grad_equals_sequential(cuda, chunk):
    """fwd_grad(batched=True): the p directions as p members of one run, each
    with its own tangent (chunk=3: two runs of 3 and 1 members), against the
    sequential form on the drop-in API."""
    from my_swampe_gb300 import run_model_scan_final, workloads
    from my_swampe_gb300.autodiff_utils import fwd_grad
    from my_swampe_gb300.engine import Engine

    eng = Engine([(42, 1)], "fp64")
    wl = workloads.forced_ensemble(eng, dt=600.0, Phibar=3.0e5, seed=7)
    ics = [wl["ics"][k, 0] for k in range(5)]  # (J, I) each
    target = 1.01 * ics[2]
    kw = dict(M=42, dt=600.0, tmax=2 + NSTEPS, omega=3.2e-5, a=8.2e7, K6=1.24e33)

    def run(th):  # th: (k, 4) rows -> (k, J, I) terminal Phi of k members
        k = th.shape[0]
        f = [x.expand(k, *x.shape) for x in ics]
        return run_model_scan_final(**kw, taurad=th[:, 0], taudrag=th[:, 1], DPhieq=th[:, 2], Phibar=th[:, 3],
                                    eta0_init=f[0], delta0_init=f[1], Phi0_init=f[2], U0_init=f[3],
                                    V0_init=f[4])["last_state"].Phi_curr

    def loss_batched(th):
        return ((run(th) - target) ** 2).mean(dim=(1, 2))

    def loss_one(th):
        return loss_batched(th[None])[0]

    theta = torch.tensor([36000.0, 21600.0, 1.0e6, 3.0e5], dtype=torch.float64, device=eng.device)
    g_seq = fwd_grad(loss_one, theta)
    g_bat = fwd_grad(loss_batched, theta, chunk=chunk, batched=True)
    rel = (g_bat - g_seq).abs() / g_seq.abs()
    assert bool(torch.all(rel < 1e-12)), (g_bat, g_seq)


def test_fast_tangent_close_to_fp64(cuda):
    """FP32 tangent model (incremental steps) against the FP64 one."""
    t64 = _tangent(*_setup("fp64"))
    eng, flags, wl, ics, dics, dpar = _setup("fast")
    t32 = _tangent(eng, flags, wl, ics, dics, dpar)
    for k, name in enumerate(("eta", "delta", "Phi")):
        rel = float(torch.linalg.norm(t32[k] - t64[k]) / torch.linalg.norm(t64[k]))
        assert rel < 1e-4, (name, rel)


def test_tangent_refuses_unsupported(cuda):
    from my_swampe_gb300.engine import RunFlagsC

    eng, flags, wl, ics, dics, dpar = _setup()
    tf, tr, _ = eng.new_tangent_buffers()
    for bad in (RunFlagsC(test=1), RunFlagsC(diagnostics=True)):
        with pytest.raises(RuntimeError):
            eng.tangent_forward(bad, 2, 2, tf, tr, [dpar])


SI_PARAMS = (("taurad", 0, 1e-1, 1e-4), ("taudrag", 1, 1e-1, 1e-4), ("DPhieq", 2, 1e-1, 1e-4),
             ("Phibar", 3, 1e-2, 1e-2), ("a", 4, 1e-2, 1e-4), ("dt", 5, 1e-2, 1e-4), ("K6", 6, 1e-1, 1e-2),
             ("K6Phi", 7, 1e-1, 1e-2), ("omega", 8, 1e-1, 1e-5), ("si_alpha", 9, 1e-1, 1e-4))


def _si_setup(precision="fp64"):
    from my_swampe_gb300.engine import RunFlagsC

    eng, _, wl, ics, dics, _ = _setup(precision)
    eng.set_params(0, si_alpha=0.6)
    wl["params"]["si_alpha"] = 0.6
    return eng, RunFlagsC(scheme=2, diagnostics=False, t_start=2), wl, ics, dics


@pytest.mark.parametrize("name,row,scale,h", SI_PARAMS)
def test_semi_implicit_parameter_tangents_match_central_differences(cuda, name, row, scale, h):
    """Tangent of the semi-implicit step (the implicit solve, its coefficients
    and the lagged remainder) along each parameter, against central differences."""
    eng, flags, wl, ics, _ = _si_setup()
    p = wl["params"]
    base = p[name] if torch.is_tensor(p.get(name)) else torch.full((2,), float(p[name]), dtype=torch.float64,
                                                                       device=eng.device)
    dpar = torch.zeros((NTAN, 2), dtype=torch.float64, device=eng.device)
    dpar[row] = scale * base * torch.tensor([1.0, -0.5], dtype=torch.float64, device=eng.device)
    tl = _tangent(eng, flags, wl, ics, torch.zeros_like(ics), dpar)
    fd = (_forward(eng, flags, wl, ics, dpar, h) - _forward(eng, flags, wl, ics, dpar, -h)) / (2 * h)
    for k, fname in enumerate(("eta", "delta", "Phi", "U", "V")):
        nrm = float(torch.linalg.norm(fd[k]))
        rel = float(torch.linalg.norm(tl[k] - fd[k])) / max(nrm, 1e-300)
        assert rel < 1e-5, (name, fname, rel, nrm)


def test_semi_implicit_initial_field_tangent(cuda):
    eng, flags, wl, ics, dics = _si_setup()
    dpar = torch.zeros((NTAN, 2), dtype=torch.float64, device=eng.device)
    tl = _tangent(eng, flags, wl, ics, dics, dpar)
    h = 1e-6
    fd = (_forward(eng, flags, wl, ics + h * dics) - _forward(eng, flags, wl, ics - h * dics)) / (2 * h)
    for k, fname in enumerate(("eta", "delta", "Phi", "U", "V")):
        rel = float(torch.linalg.norm(tl[k] - fd[k]) / torch.linalg.norm(fd[k]))
        assert rel < 2e-6, (fname, rel)


@pytest.mark.parametrize("M,scheme", [(63, 0), (106, 0), (63, 2)])
def test_tangent_other_truncations(cuda, M, scheme):
    """Tangent along an initial-field direction plus Phibar and a (one
    combined direction) at M = 63 and 106, against central differences."""
    from my_swampe_gb300 import workloads
    from my_swampe_gb300.engine import Engine, RunFlagsC

    eng = Engine([(M, 2)], "fp64")
    wl = workloads.forced_ensemble(eng, dt=300.0, Phibar=3.0e5, seed=9)
    flags = RunFlagsC(scheme=scheme, diagnostics=False, t_start=2)
    ics = wl["ics"]
    dics = (ics * 0.01).contiguous()
    dpar = torch.zeros((NTAN, 2), dtype=torch.float64, device=eng.device)
    dpar[3] = 3.0e3
    dpar[4] = 8.2e5

    def fwd(sh):
        p = dict(wl["params"])
        p["Phibar"] = p["Phibar"] + sh * dpar[3]
        p["a"] = p["a"] + sh * dpar[4]
        workloads.apply_params(eng, 0, p)
        eng.init_state([ics + sh * dics], flags)
        eng.forward(flags, t0=2, nsteps=6)
        return eng.output_physical(flags)[0][:5].double()

    workloads.apply_params(eng, 0, wl["params"])
    eng.init_state([ics], flags)
    tf, tr, _ = eng.new_tangent_buffers()
    eng.tangent_init(flags, [ics], [dics], tf, tr, [dpar])
    eng.tangent_forward(flags, 2, 6, tf, tr, [dpar])
    tl = eng.tangent_output(flags, tf, tr, [dpar])[0][:5].double()
    h = 1e-3
    fd = (fwd(h) - fwd(-h)) / (2 * h)
    for k, fname in enumerate(("eta", "delta", "Phi", "U", "V")):
        rel = float(torch.linalg.norm(tl[k] - fd[k]) / torch.linalg.norm(fd[k]))
        assert rel < 1e-5, (M, scheme, fname, rel)


@pytest.mark.parametrize("name,row,scale,h", [("taurad", 0, 1e-1, 1e-4), ("taudrag", 1, 1e-1, 1e-4),
                                              ("Phibar", 3, 1e-2, 1e-2), ("a", 4, 1e-2, 1e-4),
                                              ("dt", 5, 1e-2, 1e-4), ("K6", 6, 1e-1, 1e-2)])
def test_explicit_scheme_tangents_match_central_differences(cuda, name, row, scale, h):
    """Tangent of the explicit leapfrog (expflag) along parameters, and along
    an initial-field direction, against central differences."""
    from my_swampe_gb300.engine import RunFlagsC

    eng, _, wl, ics, dics, _ = _setup()
    flags = RunFlagsC(scheme=1, diagnostics=False, t_start=2)
    p = wl["params"]
    base = p[name] if torch.is_tensor(p.get(name)) else torch.full((2,), float(p[name]), dtype=torch.float64,
                                                                       device=eng.device)
    dpar = torch.zeros((NTAN, 2), dtype=torch.float64, device=eng.device)
    dpar[row] = scale * base * torch.tensor([1.0, -0.5], dtype=torch.float64, device=eng.device)
    tl = _tangent(eng, flags, wl, ics, 1e-3 * dics, dpar)
    fd = (_forward(eng, flags, wl, ics + h * 1e-3 * dics, dpar, h) -
          _forward(eng, flags, wl, ics - h * 1e-3 * dics, dpar, -h)) / (2 * h)
    for k, fname in enumerate(("eta", "delta", "Phi", "U", "V")):
        rel = float(torch.linalg.norm(tl[k] - fd[k]) / torch.linalg.norm(fd[k]))
        assert rel < 1e-5, (name, fname, rel)
