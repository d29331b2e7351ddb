"""Large ensembles through the drop-in API run as two concurrent halves (one
plan of two groups, a stream each).  Members are independent, so the split
run gives each member the results of the one-group run: bit for bit in FP64
(the SIMT Legendre kernels' results do not depend on their member tile), and
the gradients up to the order of the atomic sums."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

B = 128


def _kw(expflag=False):
    rng = np.random.default_rng(7)
    return dict(M=42, dt=300.0 if expflag else 600.0, tmax=9, Phibar=3.0e5, omega=7.292e-5, a=6.37122e6, test=None,
                g=9.8, forcflag=True, taurad=torch.tensor(10.0 ** rng.uniform(4.5, 5.5, B), dtype=torch.float64),
                taudrag=torch.tensor(10.0 ** rng.uniform(4.5, 5.5, B), dtype=torch.float64),
                DPhieq=torch.tensor(rng.uniform(1e5, 4e6, B), dtype=torch.float64), diffflag=True, modalflag=True,
                alpha=0.01, expflag=expflag, K6=1.24e33, diagnostics=False, precision="fp64")


def _run(split, **kw):
    from my_swampe_gb300 import model, run_model_scan_final

    old = model._SPLIT_MIN_B
    model._SPLIT_MIN_B = 64 if split else 10**9
    try:
        return run_model_scan_final(**kw)
    finally:
        model._SPLIT_MIN_B = old


@pytest.mark.parametrize("expflag", [False, True])
def test_split_forward_equals_one_group(cuda, expflag):
    a = _run(True, **_kw(expflag))["last_state"]
    b = _run(False, **_kw(expflag))["last_state"]
    for name in ("eta_curr", "delta_curr", "Phi_curr", "U_curr", "V_curr", "etam_curr", "Phim_curr", "etam_prev",
                 "Am_curr", "Fm_curr", "Rum_lag"):
        assert torch.equal(getattr(a, name), getattr(b, name)), name
    assert torch.equal(a.dead, b.dead)


def test_split_gradients_equal_one_group(cuda):
    grads = []
    for split in (True, False):
        kw = _kw()
        p = {k: kw[k].clone().cuda().requires_grad_(True) for k in ("taurad", "DPhieq")}
        kw.update(p)
        Phi = _run(split, **kw)["last_state"].Phi_curr
        loss = (Phi * Phi).mean()
        grads.append([x.detach() for x in torch.autograd.grad(loss, [p["taurad"], p["DPhieq"]])])
    for ga, gb in zip(*grads):
        torch.testing.assert_close(ga, gb, rtol=1e-12, atol=0)
