"""Pickle save/load and timestamp arithmetic around ``run_model``.

Host-side I/O with the same file naming and units as the reference
(``src/my_swampe/continuation.py:12-211``): fields are stored as
``<field>-<timestamp>`` pickles of single-level physical arrays under
``custompath`` (default ``data/``).
"""
from __future__ import annotations

import pickle
from pathlib import Path
from typing import Any, Optional

import numpy as np

_FACT = {"hours": 3600.0, "minutes": 60.0, "seconds": 1.0, "days": 3600.0 * 24.0}


def _base(custompath: Optional[str]) -> Path:
    return Path("data") if custompath is None else Path(custompath)


def write_pickle(filename: str, data: Any, custompath: Optional[str] = None) -> None:
    """``continuation.py:30-51``."""
    base = _base(custompath)
    base.mkdir(parents=True, exist_ok=True)
    with (base / filename).open("wb") as f:
        pickle.dump(data, f, protocol=pickle.HIGHEST_PROTOCOL)


def read_pickle(filename: str, custompath: Optional[str] = None) -> Any:
    """``continuation.py:46-64``."""
    with (_base(custompath) / filename).open("rb") as f:
        return pickle.load(f)


def compute_timestamp(units: str, t: int, dt: float) -> str:
    """``continuation.py:67-98``."""
    if units == "steps":
        return str(int(t))
    if units not in _FACT:
        raise ValueError("Cannot parse units. Acceptable units are: hours, minutes, seconds, steps, days.")
    return str(int(dt * t / _FACT[units]))


def compute_t_from_timestamp(units: str, timestamp: float, dt: float) -> int:
    """``continuation.py:101-132``."""
    if units == "steps":
        return int(timestamp)
    if units not in _FACT:
        raise ValueError("Cannot parse units. Acceptable units are: hours, minutes, seconds, steps, days.")
    return int(timestamp * _FACT[units] / dt)


def save_data(timestamp, etadata, deltadata, Phidata, U, V, spinupdata, geopotdata, custompath=None) -> None:
    """``continuation.py:135-179``."""
    ts = str(timestamp)
    for name, arr in (("eta", etadata), ("delta", deltadata), ("Phi", Phidata), ("U", U), ("V", V)):
        write_pickle(f"{name}-{ts}", np.asarray(arr), custompath=custompath)
    write_pickle("spinup-winds", np.asarray(spinupdata), custompath=custompath)
    write_pickle("spinup-geopot", np.asarray(geopotdata), custompath=custompath)


def load_data(timestamp, custompath: Optional[str] = None):
    """``continuation.py:182-211``: (eta, delta, Phi, U, V) numpy arrays."""
    ts = str(timestamp)
    return tuple(np.asarray(read_pickle(f"{n}-{ts}", custompath=custompath)) for n in ("eta", "delta", "Phi", "U", "V"))
