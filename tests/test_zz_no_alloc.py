"""swp_adjoint_step_noalloc: the adjoint step for callers that cannot call
cudaMalloc where they run it (inside another framework's custom call or
callback that owns the allocator, hard-latency loops, embedded users of the
C ABI).  Its scratch lives in a fixed device array inside the library.

Checked through the C ABI against swp_adjoint_step (caller-provided scratch)
on two calls in a row with different adjoint inputs:
  - an FP64 plan of one group (SIMT kernels);
  - a fast plan at M = 42 (FP32 state, tensor-core Legendre adjoint), whose
    scratch holds 8-byte complex values;
  - an FP64 plan of two groups (M = 42 and 63), whose scratch is carved at two
    offsets of the array.
Both entry points run the same kernels, so the adjoint state agrees to 1e-12
of its maximum (FP64) or 1e-6 (FP32), and the gradients to the same relative
bound (only the order of the atomic gradient reductions may differ).
The refusals that swp_adjoint_step makes before launching anything hold for
this entry too.  This file is collected last so that a run stopping at the
first failure has run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PLANS = {
    "fp64_one_group": ("fp64", [(42, 3)]),
    "fast_tensor_cores": ("fast", [(42, 3)]),
    "fp64_two_groups": ("fp64", [(42, 2), (63, 1)]),
}


def _engine_after_steps(precision, groups):
    from my_swampe_gb300 import workloads
    from my_swampe_gb300.engine import Engine, RunFlagsC

    eng = Engine(groups, precision)
    ics = []
    for g in range(len(groups)):
        wl = workloads.forced_ensemble(eng, g=g, seed=11 + g, Phibar=3.0e5)
        workloads.apply_params(eng, g, wl["params"])
        ics.append(wl["ics"])
    flags = RunFlagsC()
    eng.init_state(ics, flags)
    eng.forward(flags, t0=2, nsteps=2)
    s_in = [gd["fourier"].clone() for gd in eng.groups]
    eng.forward(flags, t0=4, nsteps=1)
    s_out = [gd["fourier"].clone() for gd in eng.groups]
    return eng, flags, s_in, s_out


@pytest.mark.parametrize("plan", list(PLANS))
def test_noalloc_adjoint_step_matches_caller_scratch(cuda, plan):
    import torch
    from my_swampe_gb300 import _lib

    precision, groups = PLANS[plan]
    eng, flags, s_in, s_out = _engine_after_steps(precision, groups)
    if plan == "fast_tensor_cores":
        assert eng.uses_tensor_cores
    tol = 1e-12 if precision == "fp64" else 1e-6
    ng = len(groups)
    lib = _lib.load()
    st_in = eng._states(fourier=s_in)
    st_out = eng._states(fourier=s_out)
    fl = flags.c()
    gen = torch.Generator(device=eng.device).manual_seed(5)
    for call in range(2):
        lam_a, lam_b, grad_a, grad_b, lamy = [], [], [], [], []
        for g, gd in enumerate(eng.groups):
            lam0 = torch.randn(s_in[g].shape, dtype=eng.cdtype, device=eng.device, generator=gen)
            lam_a.append(lam0.clone())
            lam_b.append(lam0.clone())
            grad_a.append(torch.zeros((_lib.NGRAD, gd["B"]), dtype=torch.float64, device=eng.device))
            grad_b.append(torch.zeros_like(grad_a[-1]))
            lamy.append(torch.zeros((5,) + tuple(s_in[g].shape[1:]), dtype=eng.cdtype, device=eng.device))
        adj_a = (_lib.GroupAdjoint * ng)()
        adj_b = (_lib.GroupAdjoint * ng)()
        for g in range(ng):
            adj_a[g].lam, adj_a[g].lam_y, adj_a[g].grad = lam_a[g].data_ptr(), lamy[g].data_ptr(), grad_a[g].data_ptr()
            adj_b[g].lam, adj_b[g].lam_y, adj_b[g].grad = lam_b[g].data_ptr(), None, grad_b[g].data_ptr()
        rc = lib.swp_adjoint_step(eng._plan, st_in, st_out, adj_a, ctypes.byref(fl), 4, eng.stream)
        assert rc == 0, lib.swp_last_error(eng._plan)
        rc = lib.swp_adjoint_step_noalloc(eng._plan, st_in, st_out, adj_b, ctypes.byref(fl), 4, eng.stream)
        assert rc == 0, lib.swp_last_error(eng._plan)
        eng.check_device_status()
        for g in range(ng):
            a, b = lam_a[g].cpu().numpy(), lam_b[g].cpu().numpy()
            assert np.isfinite(b).all()
            np.testing.assert_allclose(b, a, rtol=0, atol=tol * np.max(np.abs(a)), err_msg=f"{plan} group {g}")
            ga, gb = grad_a[g].cpu().numpy(), grad_b[g].cpu().numpy()
            np.testing.assert_allclose(gb, ga, rtol=tol, atol=1e-300, err_msg=f"{plan} group {g} gradients")
            assert np.max(np.abs(ga)) > 0


def test_noalloc_refuses_what_the_adjoint_step_refuses(cuda):
    """Refused on the host before any launch: RAW-filtered flags
    (SWP_ERR_UNSUPPORTED: the adjoint kernels do not implement the filter), an
    out-of-range test value and a missing adjoint buffer (SWP_ERR_ARG)."""
    from my_swampe_gb300 import _lib
    from my_swampe_gb300.engine import Engine, RunFlagsC

    eng = Engine([(42, 2)], "fp64")
    lib = _lib.load()
    st = eng._states()
    lam = eng.new_adjoint_buffers()[0][0]
    adj = (_lib.GroupAdjoint * 1)()
    adj[0].lam = lam.data_ptr()
    rc = lib.swp_adjoint_step_noalloc(eng._plan, st, st, adj, ctypes.byref(RunFlagsC(raw_filter=True).c()), 3,
                                      eng.stream)
    assert rc == 5, lib.swp_last_error(eng._plan)
    bad_test = RunFlagsC().c()
    bad_test.test = 7
    assert lib.swp_adjoint_step_noalloc(eng._plan, st, st, adj, ctypes.byref(bad_test), 3, eng.stream) == 1
    adj[0].lam = None
    rc = lib.swp_adjoint_step_noalloc(eng._plan, st, st, adj, ctypes.byref(RunFlagsC().c()), 3, eng.stream)
    assert rc == 1 and b"missing adjoint buffer" in lib.swp_last_error(eng._plan)


def test_noalloc_rejects_plans_beyond_the_scratch_size(cuda):
    from my_swampe_gb300 import _lib
    from my_swampe_gb300.engine import Engine, RunFlagsC

    # 5 * 107 * 160 * 16 bytes per member at M=106 in FP64: 64 members need ~88 MB > 16 MiB
    eng = Engine([(106, 64)], "fp64")
    lib = _lib.load()
    st = eng._states()
    adj = (_lib.GroupAdjoint * 1)()
    lam = eng.new_adjoint_buffers()[0][0]
    adj[0].lam = lam.data_ptr()
    rc = lib.swp_adjoint_step_noalloc(eng._plan, st, st, adj, ctypes.byref(RunFlagsC().c()), 3, eng.stream)
    assert rc == _lib.SWP_OK + 1
    assert b"SWP_NOALLOC_SCRATCH_BYTES" in lib.swp_last_error(eng._plan)
