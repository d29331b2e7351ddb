"""The reference's autodiff tests (unit_tests/test_autodiff.py) on the drop-in
API: torch.autograd / forward-mode AD through run_model_scan_final itself,
as jax.grad / jax.jvp go through the reference's."""
import numpy as np
import pytest
import torch
import torch.autograd.forward_ad as fwAD

pytestmark = pytest.mark.gpu

BASE = dict(M=42, dt=600.0, tmax=7, Phibar=3.0e5, omega=7.292e-5, a=6.37122e6, test=None, g=9.8, forcflag=True,
            taurad=86400.0, taudrag=86400.0, DPhieq=4.0e6, diffflag=True, modalflag=True, alpha=0.01,
            expflag=False, K6=1.24e33, diagnostics=False, jit_scan=True)


def _loss(name, theta, **extra):
    from my_swampe_gb300 import run_model_scan_final

    kw = dict(BASE, **extra)
    kw[name] = theta
    Phi = run_model_scan_final(**kw)["last_state"].Phi_curr
    return torch.mean(Phi * Phi)


@pytest.mark.parametrize("name,value", [("DPhieq", 4.0e6), ("taurad", 86400.0), ("taudrag", 86400.0),
                                        ("K6", 1.24e33), ("Phibar", 3.0e5), ("omega", 7.292e-5),
                                        ("a", 6.37122e6), ("dt", 600.0), ("alpha", 0.01)])
def test_grad_returns_finite_for_each_scalar_parameter(cuda, name, value):
    """test_autodiff.py:56-86, every parameter the reference lists.  alpha only
    filters the prev level, so the curr-field loss has a zero derivative."""
    th = torch.tensor(value, dtype=torch.float64, device="cuda", requires_grad=True)
    g = torch.autograd.grad(_loss(name, th), th)[0]
    assert g.shape == () and bool(torch.isfinite(g))
    assert (float(g) == 0.0) if name == "alpha" else (float(g) != 0.0)


@pytest.mark.parametrize("name,value,rel_h", [("K6", 1.24e33, 1e-2), ("omega", 7.292e-5, 1e-4),
                                              ("a", 6.37122e6, 1e-5), ("dt", 600.0, 1e-5)])
def test_coefficient_parameter_gradients_match_finite_differences(cuda, name, value, rel_h):
    th = torch.tensor(value, dtype=torch.float64, device="cuda", requires_grad=True)
    g_ad = float(torch.autograd.grad(_loss(name, th), th)[0])
    h = rel_h * value
    with torch.no_grad():
        g_fd = (float(_loss(name, value + h)) - float(_loss(name, value - h))) / (2 * h)
    assert abs(g_ad - g_fd) <= 1e-4 * abs(g_fd), (name, g_ad, g_fd)


def test_jvp_returns_finite_for_DPhieq(cuda):
    """test_autodiff.py:89-99"""
    with fwAD.dual_level():
        d = fwAD.make_dual(torch.tensor(4.0e6, dtype=torch.float64, device="cuda"),
                           torch.tensor(1.0, dtype=torch.float64, device="cuda"))
        out = fwAD.unpack_dual(_loss("DPhieq", d))
    assert bool(torch.isfinite(out.primal)) and bool(torch.isfinite(out.tangent))
    # forward mode equals reverse mode
    th = torch.tensor(4.0e6, dtype=torch.float64, device="cuda", requires_grad=True)
    g = torch.autograd.grad(_loss("DPhieq", th), th)[0]
    assert abs(float(out.tangent) - float(g)) <= 1e-9 * abs(float(g))


def test_grad_matches_finite_difference_for_DPhieq(cuda):
    """test_autodiff.py:102-129: centred difference with eps = 1, rel < 1e-4."""
    th = torch.tensor(4.0e6, dtype=torch.float64, device="cuda", requires_grad=True)
    g_ad = float(torch.autograd.grad(_loss("DPhieq", th), th)[0])
    with torch.no_grad():
        fp = float(_loss("DPhieq", 4.0e6 + 1.0))
        fm = float(_loss("DPhieq", 4.0e6 - 1.0))
    g_fd = (fp - fm) / 2.0
    assert g_ad != 0.0
    assert abs(g_ad - g_fd) / max(abs(g_fd), 1e-30) < 1e-4


def test_grad_wrt_initial_phi_field(cuda):
    """test_autodiff.py:132-190: gradient with respect to a (J, I) initial Phi
    (solid-body eta, zero delta and winds given explicitly)."""
    from my_swampe_gb300 import run_model_scan_final
    from oracle import swampe_oracle as o

    mus = o.cached_geometry(42)["mus"]
    eta0 = np.broadcast_to(2 * 7.292e-5 * mus[:, None], (64, 128)).copy()
    z = np.zeros((64, 128))
    phi = torch.zeros((64, 128), dtype=torch.float64, device="cuda", requires_grad=True)
    sim = run_model_scan_final(M=42, dt=1200.0, tmax=5, Phibar=3.0e5, omega=7.292e-5, a=6.37122e6, test=None,
                               eta0_init=eta0, delta0_init=z, Phi0_init=phi, U0_init=z, V0_init=z,
                               diagnostics=False)
    g = torch.autograd.grad(torch.mean(sim["last_state"].Phi_curr), phi)[0]
    assert g.shape == (64, 128)
    assert bool(torch.all(torch.isfinite(g))) and float(g.abs().max()) > 0.0


def test_history_run_gradient_equals_final_run(cuda):
    """With history and diagnostics on, the curr fields still carry the gradient,
    and the history is the plain run's."""
    from my_swampe_gb300 import run_model_scan

    th = torch.tensor(4.0e6, dtype=torch.float64, device="cuda", requires_grad=True)
    kw = dict(BASE)
    kw.pop("diagnostics")
    kw["DPhieq"] = th
    res = run_model_scan(**kw, diagnostics=True)
    Phi = res["last_state"].Phi_curr
    g1 = torch.autograd.grad(torch.mean(Phi * Phi), th)[0]
    th2 = torch.tensor(4.0e6, dtype=torch.float64, device="cuda", requires_grad=True)
    g2 = torch.autograd.grad(_loss("DPhieq", th2), th2)[0]
    assert abs(float(g1) - float(g2)) <= 1e-12 * abs(float(g2))
    np.testing.assert_allclose(res["outs"]["Phi"][-1].detach().cpu().numpy(), Phi.detach().cpu().numpy(),
                               rtol=0, atol=1e-9)


def test_phibar_gradient_includes_the_analytic_initial_condition(cuda):
    """test = 2 analytic ICs depend on Phibar: the gradient matches a centred difference."""
    from my_swampe_gb300 import run_model_scan_final

    kw = dict(M=42, dt=600.0, tmax=6, omega=7.2921159e-5, a=6.37122e6, test=2, forcflag=False)

    def loss(pb):
        Phi = run_model_scan_final(**kw, Phibar=pb)["last_state"].Phi_curr
        return torch.mean(Phi * Phi)

    th = torch.tensor(3.0e3, dtype=torch.float64, device="cuda", requires_grad=True)
    g_ad = float(torch.autograd.grad(loss(th), th)[0])
    with torch.no_grad():
        g_fd = (float(loss(3.0e3 + 0.01)) - float(loss(3.0e3 - 0.01))) / 0.02
    assert abs(g_ad - g_fd) <= 1e-6 * abs(g_fd), (g_ad, g_fd)


SYNTH = dict(M=42, Phibar=3.0e5, omega=3.2e-5, a=8.2e7, taudrag=21600.0, DPhieq=1.0e6, test=None, dt=600.0, tmax=40)


def _si_loss(**kw):
    from my_swampe_gb300 import run_model_scan_final

    args = dict(SYNTH, taurad=36000.0, si_alpha=0.5)
    args.update(kw)
    Phi = run_model_scan_final(**args, semi_implicit=True, diagnostics=False)["last_state"].Phi_curr
    return torch.mean(Phi ** 2)


def test_semi_implicit_grad_wrt_taurad_finite_nonzero(cuda):
    """test_semi_implicit.py:121-132 (through tangent runs: the scheme has no adjoint),
    with a centred-difference check."""
    th = torch.tensor(36000.0, dtype=torch.float64, device="cuda", requires_grad=True)
    g = float(torch.autograd.grad(_si_loss(taurad=th), th)[0])
    assert np.isfinite(g) and g != 0.0
    with torch.no_grad():
        fd = (float(_si_loss(taurad=36000.0 * (1 + 1e-5))) - float(_si_loss(taurad=36000.0 * (1 - 1e-5)))) / (
            2 * 36000.0 * 1e-5)
    assert abs(g - fd) <= 1e-4 * abs(fd), (g, fd)


def test_semi_implicit_grad_wrt_si_alpha_finite(cuda):
    """test_semi_implicit.py:135-149, with a centred-difference check."""
    th = torch.tensor(0.5, dtype=torch.float64, device="cuda", requires_grad=True)
    g = float(torch.autograd.grad(_si_loss(si_alpha=th), th)[0])
    assert np.isfinite(g)
    with torch.no_grad():
        fd = (float(_si_loss(si_alpha=0.5 + 1e-5)) - float(_si_loss(si_alpha=0.5 - 1e-5))) / 2e-5
    assert abs(g - fd) <= 1e-4 * abs(fd), (g, fd)


def test_semi_implicit_forward_mode_equals_reverse(cuda):
    with fwAD.dual_level():
        d = fwAD.make_dual(torch.tensor(3.0e5, dtype=torch.float64, device="cuda"),
                           torch.tensor(1.0, dtype=torch.float64, device="cuda"))
        t = float(fwAD.unpack_dual(_si_loss(Phibar=d)).tangent)
    th = torch.tensor(3.0e5, dtype=torch.float64, device="cuda", requires_grad=True)
    g = float(torch.autograd.grad(_si_loss(Phibar=th), th)[0])
    assert abs(t - g) <= 1e-9 * abs(g), (t, g)


def test_semi_implicit_initial_field_gradient_matches_finite_differences(cuda):
    """The semi-implicit scheme's adjoint (initial fields; its parameter
    gradients are tangent runs): the gradient in Phi0_init along a random
    direction against a central difference, forced, 20 steps."""
    from my_swampe_gb300 import run_model_scan_final
    from oracle import swampe_oracle as o

    geo = o.cached_geometry(42)
    J, I = geo["J"], geo["I"]
    mu = torch.tensor(geo["mus"], dtype=torch.float64, device="cuda")[:, None]
    rng = np.random.default_rng(12)
    eta0 = (2 * 3.2e-5 * mu).expand(J, I).contiguous()
    Phi0 = torch.tensor(3e3 * rng.standard_normal((J, I)), dtype=torch.float64, device="cuda")
    U0 = (10.0 * torch.sqrt(1 - mu**2)).expand(J, I).contiguous()
    z = torch.zeros((J, I), dtype=torch.float64, device="cuda")
    kw = dict(SYNTH, tmax=22, semi_implicit=True, eta0_init=eta0, delta0_init=z, U0_init=U0, V0_init=z)

    def loss(p):
        Phi = run_model_scan_final(**kw, Phi0_init=p)["last_state"].Phi_curr
        return torch.mean(Phi * Phi)

    th = Phi0.clone().requires_grad_(True)
    g = torch.autograd.grad(loss(th), th)[0]
    v = torch.tensor(rng.standard_normal((J, I)), dtype=torch.float64, device="cuda")
    h = 1e-2
    with torch.no_grad():
        fd = (float(loss(Phi0 + h * v)) - float(loss(Phi0 - h * v))) / (2 * h)
    ad = float((g * v).sum())
    assert abs(ad - fd) <= 1e-6 * abs(fd), (ad, fd)


def test_semi_implicit_phibar_gradient_with_analytic_test2_initial_condition(cuda):
    """The analytic test-2 fields depend on Phibar: that dependence reaches the
    gradient through the initial fields (the semi-implicit adjoint), the
    dynamics' through a tangent run."""
    from my_swampe_gb300 import run_model_scan_final

    kw = dict(M=42, dt=600.0, tmax=6, omega=7.2921159e-5, a=6.37122e6, test=2, forcflag=False, semi_implicit=True)

    def loss(pb):
        Phi = run_model_scan_final(**kw, Phibar=pb)["last_state"].Phi_curr
        return torch.mean(Phi * Phi)

    th = torch.tensor(3.0e3, dtype=torch.float64, device="cuda", requires_grad=True)
    g_ad = float(torch.autograd.grad(loss(th), th)[0])
    with fwAD.dual_level():
        d = fwAD.make_dual(torch.tensor(3.0e3, dtype=torch.float64, device="cuda"),
                           torch.tensor(1.0, dtype=torch.float64, device="cuda"))
        g_fw = float(fwAD.unpack_dual(loss(d)).tangent)
    with torch.no_grad():
        g_fd = (float(loss(3.0e3 + 0.01)) - float(loss(3.0e3 - 0.01))) / 0.02
    assert abs(g_ad - g_fd) <= 1e-6 * abs(g_fd), (g_ad, g_fd)
    assert abs(g_fw - g_ad) <= 1e-9 * abs(g_ad), (g_fw, g_ad)


def test_explicit_scheme_grad_matches_finite_differences(cuda):
    """expflag=True: reverse mode through the explicit scheme's adjoint."""
    def loss(d):
        return _loss("DPhieq", d, expflag=True, dt=300.0)

    th = torch.tensor(4.0e6, dtype=torch.float64, device="cuda", requires_grad=True)
    g = float(torch.autograd.grad(loss(th), th)[0])
    with torch.no_grad():
        fd = (float(loss(4.0e6 + 1.0)) - float(loss(4.0e6 - 1.0))) / 2.0
    assert g != 0.0 and abs(g - fd) <= 1e-4 * abs(fd), (g, fd)


def test_explicit_scheme_initial_field_gradient_matches_finite_differences(cuda):
    """expflag=True: the gradient in Phi0_init (explicit ICs with winds) from the
    adjoint, along a random direction, against a central difference."""
    from my_swampe_gb300 import run_model_scan_final
    from oracle import swampe_oracle as o

    geo = o.cached_geometry(42)
    J, I = geo["J"], geo["I"]
    mu = torch.tensor(geo["mus"], dtype=torch.float64, device="cuda")[:, None]
    rng = np.random.default_rng(11)
    eta0 = (2 * 7.292e-5 * mu).expand(J, I).contiguous()
    Phi0 = torch.tensor(3e3 * rng.standard_normal((J, I)), dtype=torch.float64, device="cuda")
    U0 = (10.0 * torch.sqrt(1 - mu**2)).expand(J, I).contiguous()
    z = torch.zeros((J, I), dtype=torch.float64, device="cuda")
    kw = dict(BASE, expflag=True, dt=300.0, eta0_init=eta0, delta0_init=z, U0_init=U0, V0_init=z)

    def loss(p):
        Phi = run_model_scan_final(**kw, Phi0_init=p)["last_state"].Phi_curr
        return torch.mean(Phi * Phi)

    th = Phi0.clone().requires_grad_(True)
    g = torch.autograd.grad(loss(th), th)[0]
    v = torch.tensor(rng.standard_normal((J, I)), dtype=torch.float64, device="cuda")
    h = 1e-2
    with torch.no_grad():
        fd = (float(loss(Phi0 + h * v)) - float(loss(Phi0 - h * v))) / (2 * h)
    ad = float((g * v).sum())
    assert abs(ad - fd) <= 1e-6 * abs(fd), (ad, fd)
