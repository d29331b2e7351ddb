import contextlib
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libswampe_gb300.so")
    config.addinivalue_line("markers", "slow: long-running test")


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from my_swampe_gb300 import build

    build.build()
    return torch.device("cuda", 0)


# Parameters of the reference's golden runs (unit_tests/test_parity_reference_regression.py:13-56)
FIXTURE_CASES = {
    "reference_case_unforced_test1": dict(
        M=42, dt=30.0, tmax=8, Phibar=3.0e3, omega=7.2921159e-5, a=6.37122e6, test=1, g=9.8,
        forcflag=False, taurad=86400.0, taudrag=86400.0, DPhieq=4.0e6, diffflag=False, modalflag=True,
        alpha=0.01, expflag=False, K6=1.24e33,
    ),
    "reference_case_forced_default": dict(
        M=42, dt=1200.0, tmax=6, Phibar=3.0e5, omega=3.2e-5, a=8.2e7, test=None, g=9.8, forcflag=True,
        taurad=10.0 * 3600.0, taudrag=6.0 * 3600.0, DPhieq=1.0e6, diffflag=True, modalflag=True,
        alpha=0.01, expflag=False, K6=1.24e33,
    ),
}
# reference tolerances (test_parity_reference_regression.py:58-64)
ATOL = {"eta": 1.0e-10, "delta": 1.0e-10, "Phi": 5.0e-8, "U": 1.0e-9, "V": 1.0e-9}
# Tolerances of the GPU FP64 path against the oracle on identical inputs
# (same Gauss-Legendre quadrature): the reference's own for the physical fields
# and their Fourier coefficients (a Fourier coefficient fft(x / I)[m] is bounded
# by max |x|); products and forcing terms, for which the reference states none,
# get 1e-11 of their maximum.
STATE_ATOL = {"etam_curr": ATOL["eta"], "etam_prev": ATOL["eta"], "deltam_curr": ATOL["delta"],
              "deltam_prev": ATOL["delta"], "Phim_curr": ATOL["Phi"], "Phim_prev": ATOL["Phi"],
              "Um_curr": ATOL["U"], "Vm_curr": ATOL["V"]}
PRODUCT_REL = 1e-11


@contextlib.contextmanager
def exact_quadrature():
    """Run the oracle on the exact (mpmath) Gauss-Legendre nodes and weights that
    the GPU path builds, instead of SciPy's roots_legendre."""
    from oracle import swampe_oracle as o

    exact = np.load(GOLDEN / "gauss_legendre.npz")
    o.set_quadrature({J: (exact[f"mu{J}"], exact[f"w{J}"]) for J in (64, 96, 160)})
    try:
        yield
    finally:
        o.set_quadrature(None)
