"""Derivatives in the filter weights: alpha (the Robert-Asselin coefficient)
and, with the Robert-Asselin-Williams filter, williams_alpha, plus every other
parameter under the RAW filter.  They are tangent-linear runs: the tangent
step filters the tangent with the primal weights, and the primal step adds the
weights' tangents times its own displacement mid - 2 curr + new (model.py:
988-1087).  The initial-condition residual, which the RAW filter keeps in the
curr level with a weight that depends on alpha and williams_alpha, carries the
weights' tangents too.

Checked against torch autograd through the CPU oracle (FP64 on both sides,
explicit initial fields that are not band-limited, so the residual terms
count), against central differences of the GPU forward, and the reference's
own RAW test (unit_tests/test_raw_filter.py:62-73)."""
import numpy as np
import pytest
import torch
import torch.autograd.forward_ad as fwAD

from oracle import swampe_oracle as o

pytestmark = pytest.mark.gpu

PARAMS = ("taurad", "taudrag", "DPhieq", "Phibar", "alpha", "williams_alpha")


def _case(seed):
    geo = o.cached_geometry(42)
    J, I = geo["J"], geo["I"]
    rng = np.random.default_rng(seed)
    mu = geo["mus"][:, None]
    lam = np.linspace(-np.pi, np.pi, I, endpoint=False)[None, :]
    eta0 = 2 * 3.2e-5 * mu * np.ones((1, I))
    Phi0 = 2e3 * np.cos(lam) * np.sqrt(1 - mu**2) + 50.0 * rng.standard_normal((J, I))
    delta0 = 1e-9 * rng.standard_normal((J, I))
    U0 = 5.0 * np.sqrt(1 - mu**2) * np.ones((1, I)) + 0.1 * rng.standard_normal((J, I))
    V0 = 0.1 * rng.standard_normal((J, I))
    params = dict(dt=1200.0, a=8.2e7, omega=3.2e-5, Phibar=3.0e5, taurad=36000.0, taudrag=21600.0, DPhieq=1.0e6,
                  K6=1.24e33, alpha=0.05, williams_alpha=0.53)
    W = rng.standard_normal((5, J, I))
    return params, (eta0, delta0, Phi0, U0, V0), W


def _gpu(params, ics, W, nsteps, scheme, raw, t0=2):
    from my_swampe_gb300.adjoint import integrate
    from my_swampe_gb300.engine import Engine, RunFlagsC

    eng = Engine([(42, 1)], "fp64")
    eng.set_params(0, dt=params["dt"], a=params["a"], omega=params["omega"], K6=params["K6"], K6Phi=params["K6"])
    dev = eng.device
    p = {k: torch.tensor([params[k]], dtype=torch.float64, device=dev, requires_grad=True) for k in PARAMS}
    ic = torch.tensor(np.stack(ics)[:, None], dtype=torch.float64, device=dev)
    out = integrate(eng, RunFlagsC(scheme=scheme, raw_filter=raw, t_start=t0), t0=t0, nsteps=nsteps, params=[p],
                    ics=[ic])[0]
    loss = (out.double() * torch.tensor(W[:, None], dtype=torch.float64, device=dev)).sum()
    loss.backward()
    return float(loss.detach()), {k: float(v.grad[0]) for k, v in p.items()}


def _oracle(params, ics, W, nsteps, semi_implicit, raw, t0=2):
    xp = o.torch_backend()
    p = {k: torch.tensor(params[k], dtype=torch.float64, requires_grad=True) for k in PARAMS}
    ic = [torch.tensor(x, dtype=torch.float64) for x in ics]
    r = o.run_model_scan_final(xp, M=42, dt=params["dt"], tmax=t0 + nsteps, starttime=t0, Phibar=p["Phibar"],
                               omega=params["omega"],
                               a=params["a"], test=None, taurad=p["taurad"], taudrag=p["taudrag"], DPhieq=p["DPhieq"],
                               K6=params["K6"], alpha=p["alpha"], eta0_init=ic[0], delta0_init=ic[1],
                               Phi0_init=ic[2], U0_init=ic[3], V0_init=ic[4], semi_implicit=semi_implicit,
                               raw_filter=raw, williams_alpha=p["williams_alpha"])["last_state"]
    outs = [r[f + "_curr"] for f in ("eta", "delta", "Phi", "U", "V")]
    loss = sum((x * torch.tensor(W[k])).sum() for k, x in enumerate(outs))
    grads = torch.autograd.grad(loss, [p[k] for k in PARAMS], allow_unused=True)
    return float(loss.detach()), {k: (0.0 if g is None else float(g)) for k, g in zip(PARAMS, grads)}


@pytest.mark.parametrize("nsteps,t0", [(3, 2), (6, 2), (3, 10)])
def test_raw_parameter_gradients_match_torch_autograd_through_oracle(cuda, nsteps, t0):
    """RAW filter, modified Euler: all six parameter gradients.  3 steps leave
    the initial-condition residual in the curr level (weight -alpha (1 - w) (wm
    - 2 wc) after the first filtered step), 6 steps let it decay; a start at
    t = 10 filters from the first step on."""
    params, ics, W = _case(seed=21)
    lg, pg = _gpu(params, ics, W, nsteps, scheme=0, raw=True, t0=t0)
    lo, po = _oracle(params, ics, W, nsteps, semi_implicit=False, raw=True, t0=t0)
    assert abs(lg - lo) <= 1e-9 * abs(lo)
    for k in PARAMS:
        assert po[k] != 0.0, k
        assert abs(pg[k] - po[k]) <= 1e-7 * abs(po[k]), (k, pg[k], po[k])


def test_semi_implicit_alpha_gradient_matches_torch_autograd_through_oracle(cuda):
    """The semi-implicit leapfrog reads the filtered level as its n-1 base, so
    alpha moves the trajectory (williams_alpha plays no part)."""
    params, ics, W = _case(seed=22)
    lg, pg = _gpu(params, ics, W, 5, scheme=2, raw=False)
    lo, po = _oracle(params, ics, W, 5, semi_implicit=True, raw=False)
    assert abs(lg - lo) <= 1e-9 * abs(lo)
    assert po["alpha"] != 0.0 and pg["williams_alpha"] == 0.0
    for k in PARAMS[:5]:
        assert abs(pg[k] - po[k]) <= 1e-7 * abs(po[k]), (k, pg[k], po[k])


def test_raw_with_semi_implicit_parameter_gradients_match_oracle(cuda):
    """The RAW filter on the semi-implicit scheme's filtered lineage (its n-1
    base): all six parameter gradients against torch autograd through the oracle."""
    params, ics, W = _case(seed=25)
    params = dict(params, dt=600.0)
    lg, pg = _gpu(params, ics, W, 5, scheme=2, raw=True)
    lo, po = _oracle(params, ics, W, 5, semi_implicit=True, raw=True)
    assert abs(lg - lo) <= 1e-9 * abs(lo)
    for k in PARAMS:
        assert po[k] != 0.0, k
        assert abs(pg[k] - po[k]) <= 1e-7 * abs(po[k]), (k, pg[k], po[k])


def test_classic_filter_alpha_does_not_move_the_curr_fields(cuda):
    """Modified Euler with the classic filter never reads the filtered level:
    the alpha and williams_alpha derivatives of the curr fields are zero."""
    params, ics, W = _case(seed=23)
    _, pg = _gpu(params, ics, W, 4, scheme=0, raw=False)
    assert pg["alpha"] == 0.0 and pg["williams_alpha"] == 0.0
    assert pg["taurad"] != 0.0


COMMON = dict(M=42, dt=240.0, tmax=40, Phibar=3.0e5, omega=3.2e-5, a=8.2e7, taurad=36000.0, taudrag=21600.0,
              DPhieq=1.0e6, test=None)


def _raw_loss(**kw):
    from my_swampe_gb300 import run_model_scan_final

    args = dict(COMMON, raw_filter=True, williams_alpha=0.53, diagnostics=False)
    args.update(kw)
    Phi = run_model_scan_final(**args)["last_state"].Phi_curr
    return torch.mean(Phi ** 2)


def test_grad_wrt_williams_alpha_is_finite(cuda):
    """unit_tests/test_raw_filter.py:62-73 on the drop-in API, with a centred
    difference of the GPU forward."""
    th = torch.tensor(0.53, dtype=torch.float64, device="cuda", requires_grad=True)
    g = float(torch.autograd.grad(_raw_loss(williams_alpha=th), th)[0])
    assert np.isfinite(g) and g != 0.0
    h = 1e-4
    with torch.no_grad():
        fd = (float(_raw_loss(williams_alpha=0.53 + h)) - float(_raw_loss(williams_alpha=0.53 - h))) / (2 * h)
    assert abs(g - fd) <= 1e-5 * abs(fd), (g, fd)


@pytest.mark.parametrize("name,value,h", [("alpha", 0.01, 1e-5), ("taurad", 36000.0, 0.36),
                                          ("DPhieq", 1.0e6, 10.0), ("Phibar", 3.0e5, 3.0)])
def test_raw_parameter_gradients_match_central_fd(cuda, name, value, h):
    """Phibar also moves the analytic initial fields: that dependence enters its
    tangent run as an initial-field tangent."""
    th = torch.tensor(value, dtype=torch.float64, device="cuda", requires_grad=True)
    g = float(torch.autograd.grad(_raw_loss(**{name: th}), th)[0])
    with torch.no_grad():
        fd = (float(_raw_loss(**{name: value + h})) - float(_raw_loss(**{name: value - h}))) / (2 * h)
    assert g != 0.0 and abs(g - fd) <= 1e-5 * abs(fd), (name, g, fd)


def test_raw_forward_mode_equals_reverse(cuda):
    with fwAD.dual_level():
        d = fwAD.make_dual(torch.tensor(0.53, dtype=torch.float64, device="cuda"),
                           torch.tensor(1.0, dtype=torch.float64, device="cuda"))
        t = float(fwAD.unpack_dual(_raw_loss(williams_alpha=d)).tangent)
    th = torch.tensor(0.53, dtype=torch.float64, device="cuda", requires_grad=True)
    g = float(torch.autograd.grad(_raw_loss(williams_alpha=th), th)[0])
    assert abs(t - g) <= 1e-12 * abs(g), (t, g)


def test_raw_initial_field_derivative_forward_mode_only(cuda):
    """Forward mode along an initial field works through the RAW filter (the
    tangent of the initial-condition residual); reverse mode has no adjoint
    there and says so at entry."""
    geo = o.cached_geometry(42)
    J, I = geo["J"], geo["I"]
    rng = np.random.default_rng(24)
    mu = torch.tensor(geo["mus"], dtype=torch.float64, device="cuda")[:, None]
    eta0 = (2 * 3.2e-5 * mu).expand(J, I).contiguous()
    Phi0 = torch.tensor(3e3 * rng.standard_normal((J, I)), dtype=torch.float64, device="cuda")
    U0 = (10.0 * torch.sqrt(1 - mu**2)).expand(J, I).contiguous()
    z = torch.zeros((J, I), dtype=torch.float64, device="cuda")
    kw = dict(tmax=6, eta0_init=eta0, delta0_init=z, U0_init=U0, V0_init=z)
    v = torch.tensor(rng.standard_normal((J, I)), dtype=torch.float64, device="cuda")
    with fwAD.dual_level():
        t = float(fwAD.unpack_dual(_raw_loss(**kw, Phi0_init=fwAD.make_dual(Phi0, v))).tangent)
    h = 1e-2
    with torch.no_grad():
        fd = (float(_raw_loss(**kw, Phi0_init=Phi0 + h * v)) - float(_raw_loss(**kw, Phi0_init=Phi0 - h * v))) / (2 * h)
    assert abs(t - fd) <= 1e-6 * abs(fd), (t, fd)
    with pytest.raises(NotImplementedError):
        _raw_loss(**kw, Phi0_init=Phi0.clone().requires_grad_(True))


def test_raw_fast_precision_gradient_matches_fp64(cuda):
    """The FP32 path (its primal Legendre step on the SIMT kernel during the
    tangent run) against the FP64 one."""
    g = []
    for precision in ("fp64", "fast"):
        th = torch.tensor(0.53, dtype=torch.float64, device="cuda", requires_grad=True)
        g.append(float(torch.autograd.grad(_raw_loss(williams_alpha=th, precision=precision), th)[0]))
    assert abs(g[1] - g[0]) <= 1e-3 * abs(g[0]), g
