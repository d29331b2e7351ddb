"""Argument checks of the C ABI that need a plan, and so a GPU.  The kernels
move Fourier rows with 16-byte accesses, so a complex buffer that is not
16-byte aligned is refused with SWP_ERR_ARG before any kernel runs.  The
plan stays usable afterwards."""
import ctypes

import pytest
import torch

pytestmark = pytest.mark.gpu

SWP_ERR_ARG = 1  # include/swampe_gb300.h


@pytest.mark.parametrize("prec", ["fast", "fp64"])
def test_misaligned_fourier_buffers_are_refused(cuda, prec):
    from my_swampe_gb300 import workloads
    from my_swampe_gb300.engine import Engine, RunFlagsC

    eng = Engine([(42, 2)], prec)
    wl = workloads.forced_ensemble(eng, g=0, seed=3)
    workloads.apply_params(eng, 0, wl["params"])
    eng.init_state([wl["ics"].to(eng.rdtype)], RunFlagsC())
    gd = eng.groups[0]
    nbytes = gd["fourier"].numel() * gd["fourier"].element_size()
    raw = torch.zeros(nbytes + 16, dtype=torch.uint8, device=eng.device)
    flags = RunFlagsC()
    st = eng._states()
    st[0].fourier = raw.data_ptr() + 8  # 8-byte aligned only
    rc = eng.lib.swp_forward(eng._plan, st, ctypes.byref(flags.c()), 2, 1, 0, 0, eng.stream)
    assert rc == SWP_ERR_ARG
    lam, lamy, grad = eng.new_adjoint_buffers()
    adj = eng._adjs(lam, lamy, grad)
    adj[0].lam = raw.data_ptr() + 8
    good = eng._states()
    rc = eng.lib.swp_adjoint_step(eng._plan, good, good, adj, ctypes.byref(flags.c()), 3, eng.stream)
    assert rc == SWP_ERR_ARG
    # nothing was launched: the device is clean and the plan still steps
    torch.cuda.synchronize()
    eng.check_device_status()
    eng.forward(flags, 2, 1)
    torch.cuda.synchronize()
