"""GB300-native time-stepping core for SWAMPE-JAX (imalsky/MY_SWAMPE).

The public entry points keep the reference signatures:
``run_model_scan``, ``run_model_scan_final``, ``run_model``, ``run_model_gpu``, and
the scan core the retrieval calls directly (``build_static``,
``model._init_state_from_fields``, ``simulate_scan``, ``simulate_scan_last``,
``model._step_once_state_only``).
The retrieval's emission stage (temperature, intensity, Ylm projection,
phase curves) is in ``my_swampe_gb300.emission``.
All numerical work runs in the hand-written sm_103a kernels of
``libswampe_gb300.so`` (built in-tree by ``my_swampe_gb300/build.py``).
"""
from .model import (  # noqa: F401
    RunFlags,
    State,
    Static,
    assert_finite_state,
    build_static,
    run_model,
    run_model_gpu,
    run_model_scan,
    run_model_scan_final,
    simulate_scan,
    simulate_scan_last,
    spectral_params,
)
from .engine import Engine, RunFlagsC  # noqa: F401
from . import emission  # noqa: F401

__version__ = "0.1.0"
