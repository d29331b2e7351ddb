"""swp_adjoint_step_noalloc: the adjoint step for callers that cannot call
cudaMalloc where they run it (inside another framework's custom call or
callback that owns the allocator, hard-latency loops, embedded users of the
C ABI).  Its scratch lives in a fixed device array inside the library.

Checked through the C ABI against swp_adjoint_step (caller-provided scratch)
on two calls in a row with different adjoint inputs, at the tolerance of the
other adjoint tests (1e-12 relative: both run the same kernels; only the
order of the atomic gradient reductions may differ).  This file is collected
last so that a run stopping at the first failure has run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_adjoint_step_matches_caller_scratch(cuda):
    import torch
    from my_swampe_gb300 import _lib, workloads
    from my_swampe_gb300.engine import Engine, RunFlagsC

    eng = Engine([(42, 3)], "fp64")
    wl = workloads.forced_ensemble(eng, seed=11, Phibar=3.0e5)
    workloads.apply_params(eng, 0, wl["params"])
    flags = RunFlagsC()
    eng.init_state([wl["ics"]], flags)
    eng.forward(flags, t0=2, nsteps=2)
    s_in = eng.groups[0]["fourier"].clone()
    eng.forward(flags, t0=4, nsteps=1)
    s_out = eng.groups[0]["fourier"].clone()
    lib = _lib.load()
    st_in = eng._states(fourier=[s_in])
    st_out = eng._states(fourier=[s_out])
    fl = flags.c()
    gen = torch.Generator(device=eng.device).manual_seed(5)
    for call in range(2):
        lam0 = torch.randn(s_in.shape, dtype=torch.complex128, device=eng.device, generator=gen)
        lam_a, lam_b = lam0.clone(), lam0.clone()
        grad_a = torch.zeros((_lib.NGRAD, 3), dtype=torch.float64, device=eng.device)
        grad_b = torch.zeros_like(grad_a)
        lamy = torch.zeros((5,) + tuple(s_in.shape[1:]), dtype=torch.complex128, device=eng.device)
        adj_a = (_lib.GroupAdjoint * 1)()
        adj_a[0].lam, adj_a[0].lam_y, adj_a[0].grad = lam_a.data_ptr(), lamy.data_ptr(), grad_a.data_ptr()
        adj_b = (_lib.GroupAdjoint * 1)()
        adj_b[0].lam, adj_b[0].lam_y, adj_b[0].grad = lam_b.data_ptr(), None, grad_b.data_ptr()
        rc = lib.swp_adjoint_step(eng._plan, st_in, st_out, adj_a, ctypes.byref(fl), 4, eng.stream)
        assert rc == 0, lib.swp_last_error(eng._plan)
        rc = lib.swp_adjoint_step_noalloc(eng._plan, st_in, st_out, adj_b, ctypes.byref(fl), 4, eng.stream)
        assert rc == 0, lib.swp_last_error(eng._plan)
        torch.cuda.synchronize()
        a, b = lam_a.cpu().numpy(), lam_b.cpu().numpy()
        assert np.isfinite(b).all()
        np.testing.assert_allclose(b, a, rtol=0, atol=1e-12 * np.max(np.abs(a)))
        ga, gb = grad_a.cpu().numpy(), grad_b.cpu().numpy()
        np.testing.assert_allclose(gb, ga, rtol=1e-12, atol=1e-300)
        assert np.max(np.abs(ga)) > 0


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
