"""Differentiable integration: a ``torch.autograd.Function`` over a whole run.

Forward: two-level initial state from physical fields, ``nsteps`` modified-
Euler steps in the CUDA kernels, full Fourier state checkpointed every
``ckpt_every`` steps, physical (eta, delta, Phi, U, V) of the final state
returned.  Backward: for each checkpoint window, last first, the window is
recomputed from its checkpoint (states kept per step) and the hand-written
adjoint step kernels run backwards through it; the adjoint of the initial-
state construction then gives gradients of the initial physical fields.
Gradients with respect to taurad, taudrag, DPhieq and Phibar are reduced per
member in FP64 on the device.

This replaces reverse-mode ``jax.grad`` through ``run_model_scan_final``
(reference ``unit_tests/test_autodiff.py:49-129``; ``model.py:1330-1334``
per-step remat) with O(nsteps / ckpt_every) stored states.

Forward mode (``torch.autograd.forward_ad`` dual tensors through
:func:`integrate`, or :func:`my_swampe_gb300.autodiff_utils.fwd_grad`) runs
the hand-written tangent-linear model alongside a primal re-run: what
``jax.jvp`` / ``jax.jacfwd`` give the reference.
"""
from __future__ import annotations

from typing import List, Sequence

import torch

from . import _lib
from .engine import Engine, RunFlagsC

GRAD_PARAMS = ("taurad", "taudrag", "DPhieq", "Phibar")
PARAM_ROW = {"taurad": _lib.P_TAURAD, "taudrag": _lib.P_TAUDRAG, "DPhieq": _lib.P_DPHIEQ, "Phibar": _lib.P_PHIBAR,
             "a": _lib.P_A, "dt": _lib.P_DT, "K6": _lib.P_K6, "K6Phi": _lib.P_K6PHI, "omega": _lib.P_OMEGA,
             "si_alpha": _lib.P_SIALPHA, "alpha": _lib.P_ALPHA, "williams_alpha": _lib.P_WALPHA}


class Integration:
    """Forward + adjoint of a whole run for an :class:`Engine` (all groups).

    Two ways to give the adjoint the primal states it needs:

    * ``store="all"``: the forward sweep keeps every state (nsteps + 1 Fourier
      states per group) and the adjoint runs straight over them: no
      recomputation.  At B=256, M=42, FP32, 1440 steps that is 154 GB, which
      GB300's HBM holds.
    * ``store="checkpoint"``: the state every ``ckpt_every`` steps is kept; each
      window is recomputed from its checkpoint before its adjoint steps (one
      extra forward sweep, memory O(nsteps / ckpt_every + ckpt_every)).

    ``store="auto"`` (default) keeps everything when it fits in
    ``mem_fraction`` of the free device memory, else checkpoints.
    """

    def __init__(self, engine: Engine, flags: RunFlagsC, t0: int, nsteps: int, ckpt_every: int = 50,
                 store: str = "auto", mem_fraction: float = 0.8):
        # the semi-implicit scheme's adjoint propagates the state (initial-field
        # gradients); its parameter gradients are per-parameter tangent runs.  The
        # RAW filter has no adjoint: its parameter gradients are tangent runs too,
        # and it has no reverse-mode initial-field gradients
        self.param_tangents = flags.scheme == 2 or bool(flags.raw_filter)
        self.raw_filter = bool(flags.raw_filter)
        if flags.test == 1:
            raise NotImplementedError("the adjoint of test=1 (fixed winds) is not implemented")
        if nsteps < 1:
            raise ValueError("nsteps must be >= 1 for a differentiable run")
        self.eng = engine
        self.flags = RunFlagsC(scheme=flags.scheme, forcflag=flags.forcflag, diffflag=flags.diffflag,
                               modalflag=flags.modalflag, test=flags.test, diagnostics=False, t_start=int(t0),
                               raw_filter=bool(flags.raw_filter))
        self.t0 = int(t0)
        self.nsteps = int(nsteps)
        self.K = max(1, min(int(ckpt_every), self.nsteps))
        self.nwin = (self.nsteps + self.K - 1) // self.K
        self.ckpt: List[torch.Tensor] = []
        self.ics: List[torch.Tensor] = []
        self._slots = None
        self._states = None
        self.ic_derivs = [{} for _ in engine.groups]
        if store not in ("auto", "all", "checkpoint"):
            raise ValueError(f"store must be 'auto', 'all' or 'checkpoint', got {store!r}")
        if store == "auto":
            need = (self.nsteps + 1) * engine.state_bytes()
            free, _ = torch.cuda.mem_get_info(engine.device)
            # memory torch's caching allocator holds but no tensor uses (e.g. the
            # stored states of a previous run) is available too
            free += torch.cuda.memory_reserved(engine.device) - torch.cuda.memory_allocated(engine.device)
            store = "all" if need <= mem_fraction * free else "checkpoint"
        self.store = store

    def release(self) -> None:
        """Drop the stored states, checkpoints and window slots."""
        self._states = None
        self._slots = None
        self.ckpt = []

    # ------------------------------------------------------------- forward
    def run_forward(self, ics: Sequence[torch.Tensor]) -> List[torch.Tensor]:
        eng = self.eng
        self.ics = [x.to(device=eng.device, dtype=eng.rdtype).contiguous() for x in ics]
        eng.init_state(self.ics, self.flags)
        if self.raw_filter:  # no adjoint sweep follows: nothing to keep
            eng.forward(self.flags, t0=self.t0, nsteps=self.nsteps)
            return [o[:5] for o in eng.output_physical(self.flags)]
        if self.store == "all":
            if self._states is None:
                self._states = [torch.empty((self.nsteps + 1,) + tuple(gd["fourier"].shape), dtype=eng.cdtype,
                                            device=eng.device) for gd in eng.groups]
            eng.forward_stored(self.flags, self.t0, self.nsteps, self._states)
            out = eng.output_physical(self.flags)
            return [o[:5] for o in out]
        if not self.ckpt:
            self.ckpt = [torch.empty((self.nwin,) + tuple(gd["fourier"].shape), dtype=eng.cdtype, device=eng.device)
                         for gd in eng.groups]
        eng.forward_checkpointed(self.flags, self.t0, self.nsteps, self.K, self.ckpt)
        out = eng.output_physical(self.flags)
        return [o[:5] for o in out]

    # ------------------------------------------------------- forward mode
    def run_tangent(self, ics: Sequence[torch.Tensor], dics: Sequence[torch.Tensor],
                    dpar: Sequence[torch.Tensor]) -> List[torch.Tensor]:
        """Primal run from ``ics`` with its tangent-linear model along ``dics``
        (5, B, J, I) and ``dpar`` (NTANGENT, B), rows in ``_lib.TANGENT_PARAMS``.
        Returns per group the tangent of the final physical curr fields."""
        eng = self.eng
        xs = [x.to(device=eng.device, dtype=eng.rdtype).contiguous() for x in ics]
        eng.init_state(xs, self.flags)
        tfour, tresid, _ = eng.new_tangent_buffers()
        dp = [d.to(device=eng.device, dtype=torch.float64).contiguous() for d in dpar]
        eng.tangent_init(self.flags, xs, dics, tfour, tresid, dp)
        eng.tangent_forward(self.flags, self.t0, self.nsteps, tfour, tresid, dp)
        out = eng.tangent_output(self.flags, tfour, tresid, dp)
        return [o[:5] for o in out]

    # ------------------------------------------------------------ backward
    def run_backward(self, dphys: Sequence[torch.Tensor]):
        """The adjoint sweep: initial-field gradients and (modified Euler,
        explicit) the gradients in taurad, taudrag, DPhieq, Phibar."""
        eng = self.eng
        lam, lamy, grad = eng.adjoint_buffers()
        eng.adjoint_seed(dphys, lam)
        if self.store == "all":
            eng.adjoint_stored(self.flags, self._states, lam, lamy, grad, t0=self.t0, nsteps=self.nsteps)
            dic = eng.adjoint_init(self.flags, self.ics, lam, grad)
            return dic, grad
        if self._slots is None:
            self._slots = [torch.empty((self.K + 1,) + tuple(gd["fourier"].shape), dtype=eng.cdtype, device=eng.device)
                           for gd in eng.groups]
        for w in reversed(range(self.nwin)):
            n = min(self.K, self.nsteps - w * self.K)
            eng.adjoint_window(self.flags, [c[w] for c in self.ckpt], self._slots, lam, lamy, grad,
                               t0=self.t0 + w * self.K, nsteps=n)
        dic = eng.adjoint_init(self.flags, self.ics, lam, grad)
        return dic, grad


NP = _lib.NTANGENT        # differentiable per-member parameters (_lib.TANGENT_PARAMS)
NF = NP + 1               # flat inputs per group: the parameters, then the initial fields


class _IntegrateFn(torch.autograd.Function):
    """flat = per group: the NP parameters of ``_lib.TANGENT_PARAMS`` as (B,)
    tensors, then the initial fields (5, B, J, I).  Reverse mode: the adjoint
    sweep gives the initial-field and taurad / taudrag / DPhieq / Phibar
    gradients; a parameter that enters only the coefficient tables or the
    filter weights (a, dt, K6, K6Phi, omega, si_alpha, alpha, williams_alpha)
    gets its per-member gradient from one tangent-linear run along it (members
    are independent, so one run serves all of them).  With the semi-implicit
    scheme or the RAW filter every parameter gradient is such a run."""

    @staticmethod
    def _set_params(eng, flat):
        for g in range(len(eng.groups)):
            vals = flat[NF * g: NF * g + NP]
            eng.set_params(g, **{k: v.detach() for k, v in zip(_lib.TANGENT_PARAMS, vals)})

    @staticmethod
    def forward(ctx, integ: Integration, *flat):
        eng = integ.eng
        _IntegrateFn._set_params(eng, flat)
        ics = [flat[NF * g + NP].detach() for g in range(len(eng.groups))]
        outs = integ.run_forward(ics)
        ctx.integ = integ
        ctx.in_dtypes = [x.dtype for x in flat]
        ctx.save_for_forward(*flat)
        ctx.save_for_backward(*flat)
        return tuple(o.to(flat[NP].dtype) for o in outs)

    @staticmethod
    def jvp(ctx, _integ_t, *flat_t):
        """Forward mode: the tangent-linear model along the input tangents."""
        integ = ctx.integ
        eng = integ.eng
        flat = ctx.saved_tensors
        _IntegrateFn._set_params(eng, flat)
        ics, dics, dpar = [], [], []
        for g, gd in enumerate(eng.groups):
            ic = flat[NF * g + NP]
            ics.append(ic.detach())
            t = flat_t[NF * g: NF * g + NF]
            rows = [(x if x is not None else torch.zeros(gd["B"], device=eng.device)).to(eng.device, torch.float64)
                    for x in t[:NP]]
            rows = [r.expand(gd["B"]) for r in rows]
            dic = t[NP] if t[NP] is not None else torch.zeros_like(ic)
            for k, name in enumerate(_lib.TANGENT_PARAMS):
                if name in integ.ic_derivs[g]:
                    dic = dic + rows[k][None, :, None, None].to(dic.dtype) * integ.ic_derivs[g][name].to(dic.dtype)
            dics.append(dic)
            dpar.append(torch.stack(rows))
        outs = integ.run_tangent(ics, dics, dpar)
        eng.check_device_status()
        return tuple(o.to(flat[NP].dtype) for o in outs)

    @staticmethod
    def backward(ctx, *gouts):
        integ = ctx.integ
        eng = integ.eng
        flat = ctx.saved_tensors
        dphys = [(g if g is not None else torch.zeros((5, gd["B"], gd["J"], gd["I"]), device=eng.device))
                 for g, gd in zip(gouts, eng.groups)]
        res = [None] * (1 + NF * len(eng.groups))
        first_extra = _lib.NGRAD
        if integ.param_tangents:
            # semi-implicit: the adjoint for the initial fields (when asked for),
            # tangent runs for every parameter
            first_extra = 0
            if any(ctx.needs_input_grad[1 + NF * g + NP] for g in range(len(eng.groups))):
                if integ.raw_filter:
                    raise NotImplementedError("reverse-mode initial-field gradients through the RAW filter are not "
                                              "implemented (forward mode and parameter gradients are)")
                dic, _ = integ.run_backward(dphys)
                for g in range(len(eng.groups)):
                    res[1 + NF * g + NP] = dic[g].to(ctx.in_dtypes[NF * g + NP])
        else:
            dic, grad = integ.run_backward(dphys)
            for g in range(len(eng.groups)):
                o = 1 + NF * g
                gr = grad[g]  # the engine's buffer: copied out
                for k, row in enumerate((_lib.G_TAURAD, _lib.G_TAUDRAG, _lib.G_DPHIEQ, _lib.G_PHIBAR)):
                    res[o + k] = gr[row].to(ctx.in_dtypes[NF * g + k], copy=True)
                res[o + NP] = dic[g].to(ctx.in_dtypes[NF * g + NP])
        # parameters without an adjoint term: one tangent run per parameter that needs a gradient
        extra = [k for k in range(first_extra, NP)
                 if any(ctx.needs_input_grad[1 + NF * g + k] for g in range(len(eng.groups)))]
        if extra:
            _IntegrateFn._set_params(eng, flat)
            ics = [flat[NF * g + NP].detach() for g in range(len(eng.groups))]
            for k in extra:
                dpar = []
                for gd in eng.groups:
                    d = torch.zeros((NP, gd["B"]), dtype=torch.float64, device=eng.device)
                    d[k] = 1.0
                    dpar.append(d)
                name = _lib.TANGENT_PARAMS[k]
                dics = [integ.ic_derivs[g][name].to(x.dtype) if name in integ.ic_derivs[g] else torch.zeros_like(x)
                        for g, x in enumerate(ics)]
                jk = integ.run_tangent(ics, dics, dpar)
                for g in range(len(eng.groups)):
                    w = dphys[g].to(torch.float64)
                    res[1 + NF * g + k] = (w * jk[g].to(torch.float64)).sum(dim=(0, 2, 3)).to(ctx.in_dtypes[NF * g + k])
        # a bounded wait of a tensor-core kernel (recomputed forward, adjoint,
        # tangent runs) that ran out makes these gradients invalid: raise
        eng.check_device_status()
        return tuple(res)


def integrate(engine: Engine, flags: RunFlagsC, t0: int, nsteps: int, params: Sequence[dict], ics: Sequence[torch.Tensor],
              ckpt_every: int = 50, integration: Integration = None, store: str = "auto", ic_derivs=None):
    """Differentiable run of every group of ``engine``.

    params[g]: dict with (B,) tensors (or scalars) 'taurad', 'taudrag', 'DPhieq',
    'Phibar', and optionally 'a', 'dt', 'K6', 'K6Phi', 'omega', 'si_alpha',
    'alpha', 'williams_alpha' (absent ones keep the values set with
    engine.set_params and get no gradient);
    ics[g]: (5, B, J, I) physical eta, delta, Phi, U, V.  Returns per group a
    (5, B, J, I) tensor of the final physical curr fields.  Passing the same
    ``integration`` object across calls reuses its checkpoint buffers and the
    library's captured CUDA graphs.  ``store`` selects how the adjoint gets
    its primal states (see :class:`Integration`).  ``ic_derivs[g]`` optionally
    maps a parameter name to d(ics[g]) / d(parameter) (5, B, J, I): initial
    fields that depend on a parameter outside the autograd graph (the
    semi-implicit scheme's tangent runs take them as initial-field tangents).
    """
    integ = integration if integration is not None else Integration(engine, flags, t0, nsteps, ckpt_every, store)
    integ.ic_derivs = ic_derivs if ic_derivs is not None else [{} for _ in engine.groups]
    flat = []
    for g, gd in enumerate(engine.groups):
        for row, k in enumerate(_lib.TANGENT_PARAMS):
            if k in params[g]:
                v = torch.as_tensor(params[g][k], device=engine.device, dtype=torch.float64)
            elif k in GRAD_PARAMS:
                raise KeyError(f"params[{g}] needs {k!r}")
            else:
                v = gd["params"][PARAM_ROW[k]].clone()
            flat.append(v.expand(gd["B"]) if v.dim() == 0 else v)
        flat.append(ics[g])
    return list(_IntegrateFn.apply(integ, *flat))
