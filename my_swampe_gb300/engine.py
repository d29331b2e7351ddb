"""Device-state owner for one or more truncation groups.

An :class:`Engine` holds a ``libswampe_gb300`` plan (static geometry built on
the GPU in FP64) and the torch tensors that carry the model state of every
group in the layout the kernels use:

* ``fourier[g]`` : complex ``(NFOURIER, M+1, B, J)`` -- Fourier-space carries
  (prev/curr of eta, delta, Phi; U, V; A..E, PhiF, F, G; RA-filtered prev)
* ``resid[g]``   : real ``(5, B, J, I)`` -- initial condition minus its
  band-limited part (so physical outputs are exact even for non-band-limited ICs)
* ``params[g]``  : float64 ``(NPAR, B)`` -- per-member scalars
* ``member[g]``  : float64 ``(4, B)``    -- per-member residual weights and flags

PyTorch is used only for device memory and streams; every arithmetic step of
the model runs in the library's CUDA kernels.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence, Tuple

import torch

from . import _lib

PRECISIONS = {"fp64": _lib.SWP_FP64, "fast": _lib.SWP_FAST}

PARAM_NAMES = ("dt", "a", "omega", "Phibar", "taurad", "taudrag", "DPhieq", "K6", "K6Phi", "alpha",
               "si_alpha", "williams_alpha")

# member tiles chosen by Engine.autotune, per (precision, ((M, B), ...))
_TUNED: Dict[Tuple, List[int]] = {}


@dataclass
class RunFlagsC:
    """Scheme switches passed to the kernels (model.py RunFlags, :156-226)."""

    scheme: int = 0          # 0 modified Euler, 1 explicit, 2 semi-implicit
    forcflag: bool = True
    diffflag: bool = True
    modalflag: bool = True
    test: Optional[int] = None
    diagnostics: bool = False
    blowup_rms: float = 8000.0
    t_start: int = 2
    raw_filter: bool = False

    def c(self) -> _lib.Flags:
        return _lib.Flags(
            int(self.scheme), int(bool(self.forcflag)), int(bool(self.diffflag)), int(bool(self.modalflag)),
            0 if self.test is None else int(self.test), int(bool(self.diagnostics)), float(self.blowup_rms),
            int(self.t_start), int(bool(self.raw_filter)),
        )


def _require_cuda(device) -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("my_swampe_gb300 needs a CUDA GPU: there is no CPU fallback")
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    if dev.type != "cuda":
        raise RuntimeError(f"device must be a CUDA device, got {dev}")
    return dev


class Engine:
    """One plan + device state for a list of ``(M, B)`` groups."""

    def __init__(self, groups: Sequence[Tuple[int, int]], precision: str = "fp64", device=None,
                 autotune: bool = False, concurrent: bool = False):
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(PRECISIONS)}, got {precision!r}")
        for M, _ in groups:
            if int(M) not in (42, 63, 106):
                raise ValueError(f"Unsupported value of M={M}. Only 42, 63, and 106 are supported.")
        if not 1 <= len(groups) <= 4:
            raise ValueError("between 1 and 4 truncation groups per engine")
        self.device = _require_cuda(device)
        self.lib = _lib.load()
        self.precision = precision
        self.rdtype = torch.float64 if precision == "fp64" else torch.float32
        self.cdtype = torch.complex128 if precision == "fp64" else torch.complex64
        ng = len(groups)
        Ms = (ctypes.c_int * ng)(*[int(m) for m, _ in groups])
        Bs = (ctypes.c_int * ng)(*[int(b) for _, b in groups])
        self._plan = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            rc = self.lib.swp_plan_create(ng, Ms, Bs, PRECISIONS[precision], ctypes.byref(self._plan))
        if rc != _lib.SWP_OK:
            msg = self.lib.swp_last_error(self._plan).decode() if self._plan.value else ""
            if self._plan.value:
                self.lib.swp_plan_destroy(self._plan)
            self._plan = ctypes.c_void_p()
            if rc == 1 and "Unsupported" in msg:
                raise ValueError(msg)
            raise RuntimeError(f"swp_plan_create failed ({_lib.ERRORS.get(rc, rc)}): {msg}")
        self.groups: List[Dict] = []
        for g in range(ng):
            M, J, I, B = (ctypes.c_int() for _ in range(4))
            _lib.check(self.lib.swp_plan_dims(self._plan, g, ctypes.byref(M), ctypes.byref(J), ctypes.byref(I), ctypes.byref(B)), self._plan, "dims")
            gd = dict(M=M.value, N=M.value, J=J.value, I=I.value, B=B.value)
            dev = self.device
            gd["fourier"] = torch.zeros((_lib.NFOURIER, gd["M"] + 1, gd["B"], gd["J"]), dtype=self.cdtype, device=dev)
            gd["resid"] = torch.zeros((_lib.NRESID, gd["B"], gd["J"], gd["I"]), dtype=self.rdtype, device=dev)
            gd["params"] = torch.zeros((_lib.NPAR, gd["B"]), dtype=torch.float64, device=dev)
            gd["params"][_lib.P_SIALPHA] = 0.5   # RunFlags defaults (model.py:186-187)
            gd["params"][_lib.P_WALPHA] = 0.53
            gd["member"] = torch.zeros((_lib.NMEMBER, gd["B"]), dtype=torch.float64, device=dev)
            # tangents of the residual weights (member rows w_curr, w_mid) of a tangent run
            gd["dweights"] = torch.zeros((2, gd["B"]), dtype=torch.float64, device=dev)
            self.groups.append(gd)
        self._geo_cache: Dict[int, Dict[str, torch.Tensor]] = {}
        if autotune:
            self.autotune()
        if concurrent:
            self.set_concurrency(True)

    def set_concurrency(self, on: bool) -> None:
        """Run each group's step chain on its own stream (see swp_plan_set_concurrency)."""
        self._check(self.lib.swp_plan_set_concurrency(self._plan, int(bool(on))), "set_concurrency")

    # ------------------------------------------------------------------ utils
    def __del__(self):
        try:
            if getattr(self, "_plan", None) is not None and self._plan.value:
                self.lib.swp_plan_destroy(self._plan)
                self._plan = ctypes.c_void_p()
        except Exception:  # pragma: no cover
            pass

    @property
    def stream(self) -> int:
        return torch.cuda.current_stream(self.device).cuda_stream

    def _states(self, fourier=None, hist=None, diag=None) -> ctypes.Array:
        arr = (_lib.GroupState * len(self.groups))()
        for g, gd in enumerate(self.groups):
            f = gd["fourier"] if fourier is None else fourier[g]
            arr[g].fourier = f.data_ptr()
            arr[g].resid = gd["resid"].data_ptr()
            arr[g].params = gd["params"].data_ptr()
            arr[g].member = gd["member"].data_ptr()
            arr[g].diag = diag[g].data_ptr() if diag is not None and diag[g] is not None else None
            arr[g].hist = hist[g].data_ptr() if hist is not None and hist[g] is not None else None
        return arr

    def _check(self, rc, what):
        _lib.check(rc, self._plan, what)

    def tiles(self) -> List[Tuple[int, int]]:
        """(member tile of the SIMT Legendre kernels, latitude rows per grid CTA) per group
        (groups on the tensor-core kernels keep a SIMT tile for the steps without a
        tensor-core form)."""
        out = []
        for g in range(len(self.groups)):
            mt, jb = ctypes.c_int(), ctypes.c_int()
            self._check(self.lib.swp_plan_tiles(self._plan, g, ctypes.byref(mt), ctypes.byref(jb)), "tiles")
            out.append((mt.value, jb.value))
        return out

    def autotune(self, nrep: int = 5, use_cache: bool = True) -> List[int]:
        """Pick the Legendre kernel of every group -- the tensor-core kernels (0)
        or a SIMT member tile (1, 2, 4, 8) -- by timing (swp_plan_autotune) on
        scratch copies of this engine's buffers.  Results are cached per
        (precision, groups) for the process."""
        key = (self.precision, tuple((gd["M"], gd["B"]) for gd in self.groups))
        if use_cache and key in _TUNED:
            for g, mt in enumerate(_TUNED[key]):
                self._check(self.lib.swp_plan_set_tile(self._plan, g, int(mt)), "set_tile")
            return list(_TUNED[key])
        scratch = [gd["fourier"].clone() for gd in self.groups]
        lam, lamy, grad = self.new_adjoint_buffers()
        chosen = (ctypes.c_int * len(self.groups))()
        self._check(self.lib.swp_plan_autotune(self._plan, self._states(fourier=scratch), self._adjs(lam, lamy, grad),
                                               ctypes.byref(RunFlagsC().c()), int(nrep), chosen, self.stream),
                    "autotune")
        _TUNED[key] = [int(x) for x in chosen]
        return list(_TUNED[key])

    @property
    def uses_tensor_cores(self) -> bool:
        """True when the modified-Euler steps of some group run the tcgen05 Legendre kernels."""
        return bool(self.lib.swp_plan_uses_tensor_cores(self._plan))

    @property
    def tensor_core_groups(self) -> List[int]:
        """The groups whose modified-Euler steps run the tcgen05 Legendre kernels."""
        mask = int(self.lib.swp_plan_uses_tensor_cores(self._plan))
        return [g for g in range(len(self.groups)) if (mask >> g) & 1]

    def check_device_status(self) -> None:
        """Synchronise and raise if a bounded device wait ran out since the last check."""
        st = ctypes.c_int(0)
        self._check(self.lib.swp_device_status(self._plan, ctypes.byref(st), self.stream), "device status")
        if st.value:
            raise RuntimeError("libswampe_gb300: a tensor-core kernel timed out waiting on the GPU; "
                               "the step results since the last check are invalid")

    # ------------------------------------------------------------- geometry
    def geometry(self, g: int = 0) -> Dict[str, torch.Tensor]:
        """FP64 mus, w and dense Pmn, Hmn (J, M+1, N+1) built on the GPU."""
        if g in self._geo_cache:
            return self._geo_cache[g]
        gd = self.groups[g]
        J, M = gd["J"], gd["M"]
        mus = torch.empty(J, dtype=torch.float64, device=self.device)
        w = torch.empty(J, dtype=torch.float64, device=self.device)
        P = torch.empty((J, M + 1, M + 1), dtype=torch.float64, device=self.device)
        H = torch.empty_like(P)
        self._check(self.lib.swp_geometry(self._plan, g, mus.data_ptr(), w.data_ptr(), P.data_ptr(), H.data_ptr(), self.stream), "geometry")
        out = dict(mus=mus, w=w, Pmn=P, Hmn=H)
        self._geo_cache[g] = out
        return out

    # ------------------------------------------------------------ parameters
    def set_params(self, g: int, **kw) -> None:
        """Set per-member scalars (float or length-B tensor) of group g."""
        gd = self.groups[g]
        for name, v in kw.items():
            row = PARAM_NAMES.index(name)
            # values only: a parameter's gradient or tangent flows through adjoint.integrate
            t = torch.as_tensor(v, dtype=torch.float64, device=self.device).detach()
            gd["params"][row].copy_(t.expand(gd["B"]) if t.dim() == 0 else t.reshape(gd["B"]))

    # ------------------------------------------------------------------ state
    def new_diag(self, nsteps: int) -> List[torch.Tensor]:
        """Per-step diagnostic rows (nsteps+1, 5, B) initialised for min/max/sum."""
        out = []
        for gd in self.groups:
            d = torch.zeros((nsteps + 1, _lib.NDIAG, gd["B"]), dtype=torch.float64, device=self.device)
            d[:, _lib.D_SPIN] = 1e300
            d[:, _lib.D_PHIMIN] = 1e300
            d[:, _lib.D_PHIMAX] = -1e300
            out.append(d)
        return out

    def init_state(self, ics: Sequence[torch.Tensor], flags: RunFlagsC, diag=None) -> None:
        """ics[g]: physical (5, B, J, I) eta, delta, Phi, U, V in the compute dtype."""
        ptrs = []
        keep = []
        for g, gd in enumerate(self.groups):
            x = ics[g].to(device=self.device, dtype=self.rdtype).contiguous()
            if tuple(x.shape) != (5, gd["B"], gd["J"], gd["I"]):
                raise ValueError(f"initial fields of group {g} must have shape {(5, gd['B'], gd['J'], gd['I'])}")
            keep.append(x)
            ptrs.append(x.data_ptr())
            gd["fourier"].zero_()
            gd["member"].zero_()
            gd["member"][_lib.MS_WCURR] = 1.0
            gd["member"][_lib.MS_WMID] = 1.0
        self._check(self.lib.swp_init_state(self._plan, self._states(diag=diag), _lib.ptr_array(ptrs), ctypes.byref(flags.c()), self.stream), "init_state")
        self._ic_keep = keep

    def diagnose_winds(self, eta_delta: Sequence[torch.Tensor]) -> List[torch.Tensor]:
        """U, V from physical eta, delta (model.py:644-666).  Clobbers the Fourier state."""
        ins, outs = [], []
        for g, gd in enumerate(self.groups):
            x = eta_delta[g].to(device=self.device, dtype=self.rdtype).contiguous()
            ins.append(x)
            outs.append(torch.empty((2, gd["B"], gd["J"], gd["I"]), dtype=self.rdtype, device=self.device))
        self._check(self.lib.swp_diagnose_winds(self._plan, self._states(), _lib.ptr_array([x.data_ptr() for x in ins]),
                                                _lib.ptr_array([o.data_ptr() for o in outs]), self.stream), "diagnose_winds")
        return outs

    def forward(self, flags: RunFlagsC, t0: int, nsteps: int, row0: int = 0, diag=None, hist=None,
                write_prev_last: bool = True, fourier=None) -> None:
        self._check(self.lib.swp_forward(self._plan, self._states(fourier=fourier, hist=hist, diag=diag), ctypes.byref(flags.c()),
                                         int(t0), int(nsteps), int(row0), int(bool(write_prev_last)), self.stream), "forward")

    def output_physical(self, flags: RunFlagsC, fourier=None) -> List[torch.Tensor]:
        outs = [torch.empty((8, gd["B"], gd["J"], gd["I"]), dtype=self.rdtype, device=self.device) for gd in self.groups]
        self._check(self.lib.swp_output_physical(self._plan, self._states(fourier=fourier), _lib.ptr_array([o.data_ptr() for o in outs]),
                                                 ctypes.byref(flags.c()), self.stream), "output_physical")
        return outs

    def state_copy(self, ckpt: Sequence[torch.Tensor], to_ckpt: bool) -> None:
        self._check(self.lib.swp_state_copy(self._plan, self._states(), _lib.ptr_array([c.data_ptr() for c in ckpt]),
                                            0 if to_ckpt else 1, self.stream), "state_copy")

    # ---------------------------------------------------------------- adjoint
    def _adjs(self, lam, lamy, grad) -> ctypes.Array:
        arr = (_lib.GroupAdjoint * len(self.groups))()
        for g in range(len(self.groups)):
            arr[g].lam = lam[g].data_ptr()
            arr[g].lam_y = lamy[g].data_ptr() if lamy is not None else None
            arr[g].grad = grad[g].data_ptr() if grad is not None else None
        return arr

    def new_adjoint_buffers(self):
        lam = [torch.zeros_like(gd["fourier"]) for gd in self.groups]
        lamy = [torch.zeros((5,) + tuple(gd["fourier"].shape[1:]), dtype=self.cdtype, device=self.device) for gd in self.groups]
        grad = [torch.zeros((_lib.NGRAD, gd["B"]), dtype=torch.float64, device=self.device) for gd in self.groups]
        return lam, lamy, grad

    def adjoint_buffers(self):
        """This engine's own adjoint buffers (lam, lam_y, grad), kept across calls
        so that the captured adjoint graphs, which hold their addresses, are
        replayed rather than captured again; grad is zeroed.  Whatever is handed
        to a caller from them must be copied first."""
        if getattr(self, "_adj_bufs", None) is None:
            self._adj_bufs = self.new_adjoint_buffers()
        for gr in self._adj_bufs[2]:
            gr.zero_()
        return self._adj_bufs

    def adjoint_seed(self, dphys: Sequence[torch.Tensor], lam) -> None:
        """lam <- adjoint of the Fourier state from gradients of the physical curr fields (5, B, J, I)."""
        xs = [d.to(device=self.device, dtype=self.rdtype).contiguous() for d in dphys]
        self._check(self.lib.swp_adjoint_seed(self._plan, self._states(), self._adjs(lam, None, None),
                                              _lib.ptr_array([x.data_ptr() for x in xs]), self.stream), "adjoint_seed")

    def adjoint_step(self, flags: RunFlagsC, four_in, four_out, lam, lamy, grad, t: int = 3) -> None:
        self._check(self.lib.swp_adjoint_step(self._plan, self._states(fourier=four_in), self._states(fourier=four_out),
                                              self._adjs(lam, lamy, grad), ctypes.byref(flags.c()), int(t), self.stream),
                    "adjoint_step")

    def adjoint_init(self, flags: RunFlagsC, ics: Sequence[torch.Tensor], lam, grad) -> List[torch.Tensor]:
        xs = [x.to(device=self.device, dtype=self.rdtype).contiguous() for x in ics]
        outs = [torch.empty_like(x) for x in xs]
        self._check(self.lib.swp_adjoint_init(self._plan, self._states(), self._adjs(lam, None, grad),
                                              _lib.ptr_array([x.data_ptr() for x in xs]),
                                              _lib.ptr_array([o.data_ptr() for o in outs]), ctypes.byref(flags.c()),
                                              self.stream), "adjoint_init")
        return outs

    def forward_checkpointed(self, flags: RunFlagsC, t0: int, nsteps: int, ckpt_every: int, ckpt) -> None:
        """ckpt[g]: (nwin, NFOURIER, M+1, B, J) buffer receiving the window-start states."""
        self._check(self.lib.swp_forward_checkpointed(self._plan, self._states(), ctypes.byref(flags.c()), int(t0),
                                                      int(nsteps), int(ckpt_every),
                                                      _lib.ptr_array([c.data_ptr() for c in ckpt]), self.stream),
                    "forward_checkpointed")

    def forward_stored(self, flags: RunFlagsC, t0: int, nsteps: int, states) -> None:
        """states[g]: (nsteps+1, NFOURIER, M+1, B, J) buffer receiving every state of the run."""
        self._check(self.lib.swp_forward_stored(self._plan, self._states(), ctypes.byref(flags.c()), int(t0), int(nsteps),
                                                _lib.ptr_array([x.data_ptr() for x in states]), self.stream),
                    "forward_stored")

    def adjoint_stored(self, flags: RunFlagsC, states, lam, lamy, grad, t0: int, nsteps: int) -> None:
        """Adjoint sweep over the states kept by forward_stored (no recomputation)."""
        self._check(self.lib.swp_adjoint_stored(self._plan, self._states(), _lib.ptr_array([x.data_ptr() for x in states]),
                                                self._adjs(lam, lamy, grad), ctypes.byref(flags.c()), int(t0),
                                                int(nsteps), self.stream), "adjoint_stored")

    def state_bytes(self) -> int:
        """Bytes of one Fourier state of every group."""
        return sum(gd["fourier"].numel() * gd["fourier"].element_size() for gd in self.groups)

    def adjoint_window(self, flags: RunFlagsC, ckpt_state, slots, lam, lamy, grad, t0: int, nsteps: int) -> None:
        """ckpt_state[g]: Fourier state at t0; slots[g]: (nsteps+1, NFOURIER, M+1, B, J) scratch."""
        self._check(self.lib.swp_adjoint_window(self._plan, self._states(fourier=ckpt_state),
                                                _lib.ptr_array([x.data_ptr() for x in slots]),
                                                self._adjs(lam, lamy, grad), ctypes.byref(flags.c()), int(t0),
                                                int(nsteps), self.stream), "adjoint_window")

    # ----------------------------------------------------------- tangent-linear
    def new_tangent_buffers(self):
        """Per group: tangent Fourier state, tangent IC residual, (NTANGENT, B) parameter
        tangents in the order of ``_lib.TANGENT_PARAMS``."""
        four = [torch.zeros_like(gd["fourier"]) for gd in self.groups]
        resid = [torch.zeros_like(gd["resid"]) for gd in self.groups]
        for gd in self.groups:  # a fresh tangent: the residual weights' tangents start at zero
            gd["dweights"].zero_()
        dpar = [torch.zeros((_lib.NTANGENT, gd["B"]), dtype=torch.float64, device=self.device) for gd in self.groups]
        return four, resid, dpar

    def _tans(self, tfour, tresid, dpar) -> ctypes.Array:
        arr = (_lib.GroupTangent * len(self.groups))()
        for g in range(len(self.groups)):
            if tuple(dpar[g].shape) != (_lib.NTANGENT, self.groups[g]["B"]) or dpar[g].dtype != torch.float64:
                raise ValueError(f"parameter tangents must be float64 ({_lib.NTANGENT}, B)")
            arr[g].fourier = tfour[g].data_ptr()
            arr[g].resid = tresid[g].data_ptr()
            arr[g].dparams = dpar[g].data_ptr()
            # rows a..williams_alpha enter only the coefficient tables and the filter
            # weights: their pass runs when one is set
            arr[g].coef_tangents = int(bool(torch.any(dpar[g][_lib.NGRAD:] != 0)))
            arr[g].dweights = self.groups[g]["dweights"].data_ptr()
        return arr

    def tangent_init(self, flags: RunFlagsC, ics, dics, tfour, tresid, dpar) -> None:
        """Tangent state from tangents dics[g] (5, B, J, I) of the physical ICs ics[g]
        (after init_state on the same ICs)."""
        xs = [x.to(device=self.device, dtype=self.rdtype).contiguous() for x in ics]
        ds = [x.to(device=self.device, dtype=self.rdtype).contiguous() for x in dics]
        self._check(self.lib.swp_tangent_init(self._plan, self._states(), self._tans(tfour, tresid, dpar),
                                              _lib.ptr_array([x.data_ptr() for x in xs]),
                                              _lib.ptr_array([x.data_ptr() for x in ds]), ctypes.byref(flags.c()),
                                              self.stream), "tangent_init")

    def tangent_forward(self, flags: RunFlagsC, t0: int, nsteps: int, tfour, tresid, dpar) -> None:
        """Advance the primal state and its tangent together by nsteps steps."""
        self._check(self.lib.swp_tangent_forward(self._plan, self._states(), self._tans(tfour, tresid, dpar),
                                                 ctypes.byref(flags.c()), int(t0), int(nsteps), self.stream),
                    "tangent_forward")

    def tangent_output(self, flags: RunFlagsC, tfour, tresid, dpar) -> List[torch.Tensor]:
        """Tangents of the physical fields of output_physical: (8, B, J, I) per group."""
        outs = [torch.empty((8, gd["B"], gd["J"], gd["I"]), dtype=self.rdtype, device=self.device) for gd in self.groups]
        self._check(self.lib.swp_tangent_output(self._plan, self._states(), self._tans(tfour, tresid, dpar),
                                                _lib.ptr_array([o.data_ptr() for o in outs]), ctypes.byref(flags.c()),
                                                self.stream), "tangent_output")
        return outs

    def time_kernels(self, flags: RunFlagsC, nrep: int = 20, adjoint: bool = True, fourier=None):
        """Average ms per launch (CUDA events, library stream) of the spectral, grid,
        grid-adjoint and spectral-adjoint kernels on a scratch copy of the state."""
        scratch = [gd["fourier"].clone() for gd in self.groups] if fourier is None else fourier
        lam, lamy, grad = self.new_adjoint_buffers() if adjoint else (None, None, None)
        ms = (ctypes.c_float * 4)()
        adjs = self._adjs(lam, lamy, grad) if adjoint else None
        self._check(self.lib.swp_time_kernels(self._plan, self._states(fourier=scratch), adjs,
                                              ctypes.byref(flags.c()), int(nrep), ms, self.stream), "time_kernels")
        return dict(spectral=ms[0], grid=ms[1], grid_adj=ms[2], spectral_adj=ms[3])
