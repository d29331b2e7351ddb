"""ctypes binding of libswampe_gb300.so (see include/swampe_gb300.h).

The library is built in-tree by ``my_swampe_gb300/build.py``.  There is no
fallback: if the shared object is missing or a CUDA device is absent, the
first call raises.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libswampe_gb300.so"

SWP_OK = 0
SWP_FP64 = 0
SWP_FAST = 1
NFOURIER = 19
NPAR = 12
NMEMBER = 4
NDIAG = 5
NGRAD = 4
NRESID = 5

# Fourier field indices (swp_common.cuh FourierField)
F_ETA_PREV, F_ETA, F_DELTA_PREV, F_DELTA, F_PHI_PREV, F_PHI, F_U, F_V = range(8)
F_A, F_B, F_C, F_D, F_E, F_PHIF, F_F, F_G, F_ETA_MID, F_DELTA_MID, F_PHI_MID = range(8, 19)
# parameter rows
P_DT, P_A, P_OMEGA, P_PHIBAR, P_TAURAD, P_TAUDRAG, P_DPHIEQ, P_K6, P_K6PHI, P_ALPHA, P_SIALPHA, P_WALPHA = range(12)
# the semi-implicit scheme keeps its lagged remainders Rum_lag, Rvm_lag in the unfiltered prev slots
F_RU_LAG, F_RV_LAG = F_ETA_PREV, F_DELTA_PREV
MS_WCURR, MS_WMID, MS_DEAD, MS_UPDATED = range(4)
D_RMS2, D_SPIN, D_PHIMIN, D_PHIMAX, D_DEAD = range(5)
G_TAURAD, G_TAUDRAG, G_DPHIEQ, G_PHIBAR = range(4)
# parameter tangents of the tangent-linear model (swampe_gb300.h SWP_NTANGENT)
TANGENT_PARAMS = ("taurad", "taudrag", "DPhieq", "Phibar", "a", "dt", "K6", "K6Phi", "omega", "si_alpha", "alpha",
                  "williams_alpha")
NTANGENT = len(TANGENT_PARAMS)

WAIT_LIMIT_DEFAULT = 1 << 22  # swampe_gb300.h SWP_WAIT_LIMIT_DEFAULT

ERRORS = {1: "bad argument", 2: "CUDA error", 3: "numerical failure", 4: "bad state", 5: "unsupported"}


class GroupState(ctypes.Structure):
    _fields_ = [
        ("fourier", ctypes.c_void_p),
        ("resid", ctypes.c_void_p),
        ("params", ctypes.c_void_p),
        ("member", ctypes.c_void_p),
        ("diag", ctypes.c_void_p),
        ("hist", ctypes.c_void_p),
    ]


class GroupAdjoint(ctypes.Structure):
    _fields_ = [
        ("lam", ctypes.c_void_p),
        ("lam_y", ctypes.c_void_p),
        ("grad", ctypes.c_void_p),
    ]


class GroupTangent(ctypes.Structure):
    _fields_ = [
        ("fourier", ctypes.c_void_p),
        ("resid", ctypes.c_void_p),
        ("dparams", ctypes.c_void_p),
        ("coef_tangents", ctypes.c_int),
        ("dweights", ctypes.c_void_p),
    ]


class Flags(ctypes.Structure):
    _fields_ = [
        ("scheme", ctypes.c_int),
        ("forcflag", ctypes.c_int),
        ("diffflag", ctypes.c_int),
        ("modalflag", ctypes.c_int),
        ("test", ctypes.c_int),
        ("diagnostics", ctypes.c_int),
        ("blowup", ctypes.c_double),
        ("t_start", ctypes.c_int),
        ("raw_filter", ctypes.c_int),
    ]


EMISSION_MAX_BANDS = 8  # swampe_gb300.h SWP_EMISSION_MAX_BANDS


class EmissionCfg(ctypes.Structure):
    _fields_ = [
        ("temp_mode", ctypes.c_int),
        ("R_d", ctypes.c_double),
        ("T_ref", ctypes.c_double),
        ("phi_to_T_scale", ctypes.c_double),
        ("Tmin", ctypes.c_double),
        ("model", ctypes.c_int),
        ("nbands", ctypes.c_int),
        ("wavelengths", ctypes.c_double * EMISSION_MAX_BANDS),
        ("band_weights", ctypes.c_double * EMISSION_MAX_BANDS),
        ("x_clip", ctypes.c_double),
    ]


EXPORTS = (
    "swp_plan_create", "swp_plan_destroy", "swp_plan_dims", "swp_last_error", "swp_geometry",
    "swp_init_state", "swp_diagnose_winds", "swp_forward", "swp_output_physical",
    "swp_state_copy", "swp_adjoint_step", "swp_adjoint_seed", "swp_adjoint_init",
    "swp_adjoint_window", "swp_time_kernels", "swp_forward_checkpointed", "swp_adjoint_step_noalloc",
    "swp_tc_selftest", "swp_device_status", "swp_plan_uses_tensor_cores", "swp_forward_stored",
    "swp_adjoint_stored", "swp_plan_autotune", "swp_plan_tiles", "swp_plan_set_tile",
    "swp_tangent_init", "swp_tangent_forward", "swp_tangent_output", "swp_plan_set_concurrency",
    "swp_plan_set_wait_limit", "swp_emission_map", "swp_emission_project", "swp_phase_curve_linear",
    "swp_phase_curve_simple",
)

_lib = None


def load(path: os.PathLike | str | None = None) -> ctypes.CDLL:
    """Load (once) and type the shared library.  Raises if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path is not None else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(there is no CPU fallback for the GB300 kernels)"
        )
    lib = ctypes.CDLL(str(p))
    vp, ip, i = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int
    gsp = ctypes.POINTER(GroupState)
    gap = ctypes.POINTER(GroupAdjoint)
    fp = ctypes.POINTER(Flags)
    gtp = ctypes.POINTER(GroupTangent)
    vpp = ctypes.POINTER(ctypes.c_void_p)
    sig = {
        "swp_plan_create": (i, [i, ip, ip, i, ctypes.POINTER(vp)]),
        "swp_plan_destroy": (i, [vp]),
        "swp_plan_dims": (i, [vp, i, ip, ip, ip, ip]),
        "swp_last_error": (ctypes.c_char_p, [vp]),
        "swp_geometry": (i, [vp, i, vp, vp, vp, vp, vp]),
        "swp_init_state": (i, [vp, gsp, vpp, fp, vp]),
        "swp_diagnose_winds": (i, [vp, gsp, vpp, vpp, vp]),
        "swp_forward": (i, [vp, gsp, fp, i, i, i, i, vp]),
        "swp_output_physical": (i, [vp, gsp, vpp, fp, vp]),
        "swp_state_copy": (i, [vp, gsp, vpp, i, vp]),
        "swp_adjoint_step": (i, [vp, gsp, gsp, gap, fp, i, vp]),
        "swp_adjoint_seed": (i, [vp, gsp, gap, vpp, vp]),
        "swp_adjoint_init": (i, [vp, gsp, gap, vpp, vpp, fp, vp]),
        "swp_adjoint_window": (i, [vp, gsp, vpp, gap, fp, i, i, vp]),
        "swp_time_kernels": (i, [vp, gsp, gap, fp, i, ctypes.POINTER(ctypes.c_float), vp]),
        "swp_forward_checkpointed": (i, [vp, gsp, fp, i, i, i, vpp, vp]),
        "swp_adjoint_step_noalloc": (i, [vp, gsp, gsp, gap, fp, i, vp]),
        "swp_tc_selftest": (i, [vp, vp, vp, i, i, i, vp]),
        "swp_device_status": (i, [vp, ip, vp]),
        "swp_plan_uses_tensor_cores": (i, [vp]),
        "swp_forward_stored": (i, [vp, gsp, fp, i, i, vpp, vp]),
        "swp_adjoint_stored": (i, [vp, gsp, vpp, gap, fp, i, i, vp]),
        "swp_plan_autotune": (i, [vp, gsp, gap, fp, i, ip, vp]),
        "swp_plan_tiles": (i, [vp, i, ip, ip]),
        "swp_plan_set_tile": (i, [vp, i, i]),
        "swp_tangent_init": (i, [vp, gsp, gtp, vpp, vpp, fp, vp]),
        "swp_tangent_forward": (i, [vp, gsp, gtp, fp, i, i, vp]),
        "swp_tangent_output": (i, [vp, gsp, gtp, vpp, fp, vp]),
        "swp_plan_set_concurrency": (i, [vp, i]),
        "swp_plan_set_wait_limit": (i, [vp, ctypes.c_uint]),
        "swp_emission_map": (i, [vp, vp, i, i, i, vp, ctypes.POINTER(EmissionCfg), i, i, vp, vp, vp]),
        "swp_emission_project": (i, [vp, vp, i, i, vp, i, vp, vp]),
        "swp_phase_curve_linear": (i, [vp, vp, vp, i, i, i, vp, vp]),
        "swp_phase_curve_simple": (i, [vp, i, i, i, vp, vp, i, vp, vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(rc: int, plan=None, what: str = "") -> None:
    if rc != SWP_OK:
        msg = ""
        if plan is not None:
            try:
                msg = load().swp_last_error(plan).decode()
            except Exception:  # pragma: no cover
                msg = ""
        raise RuntimeError(f"libswampe_gb300 {what} failed ({ERRORS.get(rc, rc)}): {msg}")


def ptr_array(ptrs):
    arr = (ctypes.c_void_p * len(ptrs))()
    for k, p in enumerate(ptrs):
        arr[k] = p
    return arr
