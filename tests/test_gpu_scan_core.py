"""The scan core's own entry points, as the retrieval calls them
(retrieval/scripts/pipeline.py:611-688, 870-927): RunFlags, build_static,
_init_state_from_fields, dataclasses.replace(static, taurad=..., taudrag=...),
simulate_scan_last and the _step_once_state_only loop; and simulate_scan
(model.py:1237-1278).

Checked: the replayed call sequence equals run_model_scan_final bit for bit;
the retrieval's fast path (state0 built once from the base parameters, steps
with replaced taurad / taudrag) equals the FP64 oracle run the same way at the
reference's tolerances; a chained run equals a single one; derivatives in the
replaced parameters (state0 fixed) match central differences in forward and
reverse mode.
"""
import dataclasses

import numpy as np
import pytest
import torch
import torch.autograd.forward_ad as fwAD

from conftest import ATOL, exact_quadrature
from oracle import swampe_oracle as o

pytestmark = pytest.mark.gpu

CFG = dict(M=42, dt=600.0, a=8.2e7, omega=3.2e-5, g=9.8, Phibar=3.0e5, DPhieq=1.0e6, K6=1.24e33, K6Phi=None)
TAU = (36000.0, 21600.0)
FIELDS = ("eta", "delta", "Phi", "U", "V")


def _flags(**kw):
    from my_swampe_gb300.model import RunFlags

    base = dict(forcflag=True, diffflag=True, expflag=False, modalflag=True, diagnostics=False, alpha=0.01,
                blowup_rms=8000.0, semi_implicit=False, raw_filter=False, si_alpha=0.5, williams_alpha=0.53)
    base.update(kw)
    return RunFlags(**base)


def _static(taurad, taudrag, **kw):
    from my_swampe_gb300.model import build_static

    c = dict(CFG, **kw)
    return build_static(M=c["M"], dt=c["dt"], a=c["a"], omega=c["omega"], g=c["g"], Phibar=c["Phibar"],
                        taurad=taurad, taudrag=taudrag, DPhieq=c["DPhieq"], K6=c["K6"], K6Phi=c["K6Phi"], test=None)


def _rest_state(static, flags, dtype=torch.float64):
    """pipeline.py:662-688: rest state eta = 2 Omega mu, Phi = Phieq - Phibar."""
    from my_swampe_gb300.model import _init_state_from_fields

    J, I = static.J, static.I
    eta0 = (2.0 * static.omega * static.mus)[:, None] * torch.ones((J, I), dtype=torch.float64, device="cuda")
    z = torch.zeros((J, I), dtype=torch.float64, device="cuda")
    Phi0 = static.Phieq - static.Phibar
    f = [x.to(dtype) for x in (eta0, z, Phi0, z, z)]
    return _init_state_from_fields(static=static, flags=flags, test=None, eta0=f[0], delta0=f[1], Phi0=f[2],
                                   U0=f[3], V0=f[4]), f


def _final(taurad, taudrag, ics, n, precision="fp64"):
    from my_swampe_gb300 import run_model_scan_final

    c = dict(CFG)
    return run_model_scan_final(M=c["M"], dt=c["dt"], tmax=2 + n, Phibar=c["Phibar"], omega=c["omega"], a=c["a"],
                                taurad=taurad, taudrag=taudrag, DPhieq=c["DPhieq"], K6=c["K6"], eta0_init=ics[0],
                                delta0_init=ics[1], Phi0_init=ics[2], U0_init=ics[3], V0_init=ics[4],
                                precision=precision)["last_state"]


@pytest.mark.parametrize("precision", ["fp64", "fast"])
def test_retrieval_call_sequence_equals_run_model_scan_final(cuda, precision):
    from my_swampe_gb300.model import _step_once_state_only, simulate_scan_last

    flags = _flags()
    n = 12
    static_base = _static(*TAU)
    dtype = torch.float64 if precision == "fp64" else torch.float32
    state0, ics = _rest_state(static_base, flags, dtype)
    t_seq = torch.arange(2, 2 + n, dtype=torch.int32)
    # the fast path with the base parameters, and the rebuilt path with others
    static = dataclasses.replace(static_base, taurad=TAU[0], taudrag=TAU[1])
    last = simulate_scan_last(static=static, flags=flags, state0=state0, t_seq=t_seq, test=None, Uic=ics[3],
                              Vic=ics[4], remat_step=False)
    want = _final(*TAU, ics, n, precision)
    for name in want._fields:
        assert torch.equal(getattr(last, name), getattr(want, name)), name
    st2 = _static(50000.0, 30000.0)
    s0b, icb = _rest_state(st2, flags, dtype)
    last2 = simulate_scan_last(static=st2, flags=flags, state0=s0b, t_seq=t_seq, test=None, Uic=icb[3], Vic=icb[4])
    want2 = _final(50000.0, 30000.0, icb, n, precision)
    for f in FIELDS:
        assert torch.equal(getattr(last2, f + "_curr"), getattr(want2, f + "_curr")), f
    # the fori_loop fallback over _step_once_state_only
    st = state0
    for t in t_seq:
        st = _step_once_state_only(st, t, static, flags, None, ics[3], ics[4])
    # the curr fields come from the Fourier carries, which are reloaded exactly;
    # the physical prev level is reloaded through an FFT round trip (round-off)
    rel = 1e-12 if precision == "fp64" else 1e-6
    for f in FIELDS:
        assert torch.equal(getattr(st, f + "_curr"), getattr(last, f + "_curr")), f
        if f in ("eta", "delta", "Phi"):
            want_prev = getattr(last, f + "_prev")
            torch.testing.assert_close(getattr(st, f + "_prev"), want_prev, rtol=0,
                                       atol=rel * float(want_prev.abs().max()))


def test_fast_path_with_replaced_parameters_matches_oracle(cuda):
    """state0 from the base parameters (its initial forcing terms too), the
    steps with replaced taurad / taudrag: the oracle run the same way."""
    from my_swampe_gb300.model import simulate_scan_last

    flags = _flags()
    n = 10
    static_base = _static(*TAU)
    state0, ics = _rest_state(static_base, flags)
    tr, td = 50000.0, 30000.0
    last = simulate_scan_last(static=dataclasses.replace(static_base, taurad=tr, taudrag=td), flags=flags,
                              state0=state0, t_seq=np.arange(2, 2 + n), test=None, Uic=ics[3], Vic=ics[4])
    with exact_quadrature():
        kw = dict(CFG)
        sb = o.build_static(o.NUMPY, M=42, dt=kw["dt"], a=kw["a"], omega=kw["omega"], g=kw["g"], Phibar=kw["Phibar"],
                            taurad=TAU[0], taudrag=TAU[1], DPhieq=kw["DPhieq"], K6=kw["K6"], K6Phi=None, test=None)
        x = [t.cpu().numpy() for t in ics]
        st = o.init_state(o.NUMPY, sb, None, *x)
        sn = dataclasses.replace(sb, taurad=tr, taudrag=td)
        fl = o.Flags(forcflag=True, diffflag=True, expflag=False, modalflag=True, diagnostics=False, alpha=0.01)
        for t in range(2, 2 + n):
            st, _ = o.step_once(o.NUMPY, st, t, sn, fl, None, x[3], x[4])
    for f in FIELDS:
        np.testing.assert_allclose(getattr(last, f + "_curr").cpu().numpy(), st[f + "_curr"], rtol=0, atol=ATOL[f],
                                   err_msg=f)
    np.testing.assert_allclose(last.Phi_prev.cpu().numpy(), st["Phi_prev"], rtol=0, atol=ATOL["Phi"])


@pytest.mark.parametrize("precision", ["fp64", "fast"])
def test_chained_runs_equal_one_run(cuda, precision):
    from my_swampe_gb300.model import simulate_scan, simulate_scan_last

    flags = _flags()
    static = _static(*TAU)
    dtype = torch.float64 if precision == "fp64" else torch.float32
    state0, ics = _rest_state(static, flags, dtype)
    one = simulate_scan_last(static=static, flags=flags, state0=state0, t_seq=range(2, 14), test=None, Uic=ics[3],
                             Vic=ics[4])
    a = simulate_scan_last(static=static, flags=flags, state0=state0, t_seq=range(2, 7), test=None, Uic=ics[3],
                           Vic=ics[4])
    b = simulate_scan_last(static=static, flags=flags, state0=a, t_seq=range(7, 14), test=None, Uic=ics[3],
                           Vic=ics[4])
    for f in FIELDS:
        assert torch.equal(getattr(b, f + "_curr"), getattr(one, f + "_curr")), f
    rel = 1e-12 if precision == "fp64" else 1e-6
    for f in ("eta", "delta", "Phi"):
        want_prev = getattr(one, f + "_prev")
        torch.testing.assert_close(getattr(b, f + "_prev"), want_prev, rtol=0, atol=rel * float(want_prev.abs().max()))
    # simulate_scan keeps the history: its last row is the final curr field
    st, outs = simulate_scan(static=static, flags=_flags(diagnostics=True), state0=a, t_seq=range(7, 14), test=None,
                             Uic=ics[3], Vic=ics[4])
    assert outs["Phi"].shape == (7, 64, 128) and outs["rms"].shape == (7,)
    torch.testing.assert_close(outs["Phi"][-1], st.Phi_curr, rtol=1e-12 if precision == "fp64" else 1e-6, atol=0)
    assert torch.equal(st.Phi_curr, one.Phi_curr)


def test_derivatives_in_replaced_parameters(cuda):
    """d Phi_T / d taurad, taudrag with state0 fixed: forward mode (dual
    tangents on static.taurad) and reverse mode against central differences."""
    from my_swampe_gb300.model import simulate_scan_last

    flags = _flags()
    n = 10
    static_base = _static(*TAU)
    state0, ics = _rest_state(static_base, flags)

    def phi_T(tr, td):
        s = dataclasses.replace(static_base, taurad=tr, taudrag=td)
        return simulate_scan_last(static=s, flags=flags, state0=state0, t_seq=range(2, 2 + n), test=None,
                                  Uic=ics[3], Vic=ics[4]).Phi_curr

    tr0 = torch.tensor(50000.0, dtype=torch.float64, device="cuda")
    td0 = torch.tensor(30000.0, dtype=torch.float64, device="cuda")
    w = torch.randn((64, 128), dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(1))
    h = 1e-4
    fd_tr = float((w * (phi_T(tr0 * (1 + h), td0) - phi_T(tr0 * (1 - h), td0))).sum() / (2 * h * tr0))
    fd_td = float((w * (phi_T(tr0, td0 * (1 + h)) - phi_T(tr0, td0 * (1 - h)))).sum() / (2 * h * td0))
    with fwAD.dual_level():
        d = fwAD.make_dual(tr0, torch.ones_like(tr0))
        jv = float((w * fwAD.unpack_dual(phi_T(d, td0)).tangent).sum())
    assert abs(jv - fd_tr) <= 1e-5 * abs(fd_tr), (jv, fd_tr)
    tr = tr0.clone().requires_grad_(True)
    td = td0.clone().requires_grad_(True)
    g_tr, g_td = torch.autograd.grad((w * phi_T(tr, td)).sum(), [tr, td])
    assert abs(float(g_tr) - fd_tr) <= 1e-5 * abs(fd_tr), (float(g_tr), fd_tr)
    assert abs(float(g_td) - fd_td) <= 1e-5 * abs(fd_td), (float(g_td), fd_td)


def test_refuses_states_it_cannot_represent(cuda):
    from my_swampe_gb300.model import simulate_scan_last

    flags = _flags()
    static = _static(*TAU)
    state0, ics = _rest_state(static, flags)
    rng = torch.Generator("cuda").manual_seed(0)
    bump = torch.randn(state0.Phi_curr.shape, dtype=torch.float64, device="cuda", generator=rng)
    odd = state0._replace(Phi_prev=state0.Phi_prev + bump, Phi_curr=state0.Phi_curr + 2 * bump)
    with pytest.raises(NotImplementedError, match="beyond the truncation"):
        simulate_scan_last(static=static, flags=flags, state0=odd, t_seq=range(2, 4), test=None, Uic=ics[3],
                           Vic=ics[4])
    with pytest.raises(ValueError, match="consecutive"):
        simulate_scan_last(static=static, flags=flags, state0=state0, t_seq=[2, 4], test=None, Uic=ics[3],
                           Vic=ics[4])
