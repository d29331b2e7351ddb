"""Concurrent group schedule (swp_plan_set_concurrency): each group's step chain
on its own stream gives bit-identical results to the joint launches, for the
forward, the stored-states and checkpointed adjoints and the tangent model."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def _engine(concurrent, precision="fast"):
    from my_swampe_gb300 import workloads
    from my_swampe_gb300.engine import Engine

    eng = Engine([(42, 4), (42, 4)], precision, concurrent=concurrent)
    wls = [workloads.forced_ensemble(eng, g=g, seed=100 + 10 * g) for g in range(2)]
    for g in range(2):
        workloads.apply_params(eng, g, wls[g]["params"])
    return eng, wls


@pytest.mark.parametrize("precision", ["fast", "fp64"])
@pytest.mark.parametrize("store", ["all", "checkpoint"])
def test_concurrent_groups_identical(cuda, precision, store):
    from my_swampe_gb300 import adjoint
    from my_swampe_gb300.engine import RunFlagsC

    res = []
    for conc in (False, True):
        eng, wls = _engine(conc, precision)
        ics = [wl["ics"].to(eng.rdtype).clone().requires_grad_(True) for wl in wls]
        params = [{k: wl["params"][k] for k in ("taurad", "taudrag", "DPhieq")} for wl in wls]
        for p in params:
            p["Phibar"] = torch.full((4,), 4.0e6, dtype=torch.float64, device="cuda")
        outs = adjoint.integrate(eng, RunFlagsC(), 2, 12, params, ics, ckpt_every=5, store=store)
        loss = sum((o[2].double() ** 2).mean() for o in outs)
        grads = torch.autograd.grad(loss, ics)
        res.append(([o.detach() for o in outs], [g.detach() for g in grads]))
    for a, b in zip(res[0][0] + res[0][1], res[1][0] + res[1][1]):
        assert torch.equal(a, b)


def test_concurrent_forward_and_tangent_identical(cuda):
    from my_swampe_gb300.engine import RunFlagsC

    fl = RunFlagsC()
    res = []
    for conc in (False, True):
        eng, wls = _engine(conc, "fp64")
        ics = [wl["ics"] for wl in wls]
        eng.init_state(ics, fl)
        eng.forward(fl, t0=2, nsteps=10)
        phys = [o.clone() for o in eng.output_physical(fl)]
        eng.init_state(ics, fl)
        tf, tr, dp = eng.new_tangent_buffers()
        for d in dp:
            d[3] = 100.0
        eng.tangent_init(fl, ics, [0.01 * x for x in ics], tf, tr, dp)
        eng.tangent_forward(fl, 2, 10, tf, tr, dp)
        tan = [o.clone() for o in eng.tangent_output(fl, tf, tr, dp)]
        res.append(phys + tan)
    for a, b in zip(*res):
        assert torch.equal(a, b)
