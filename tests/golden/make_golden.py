"""Regenerate the golden fixtures in this folder from the reference project.

The reference repository ships two FP64 fixtures produced by the upstream
NumPy SWAMPE (``unit_tests/fixtures/reference_case_{unforced_test1,forced_default}.npz``)
together with the run parameters in ``unit_tests/test_parity_reference_regression.py:13-56``.
This script copies the arrays that the parity tests assert on (terminal and
snapshot fields, snapshot steps, phase-curve projection) into compressed
``.npz`` files here, because the reference tree is not available where the
GPU tests run.

Usage:  python tests/golden/make_golden.py /path/to/reference
"""
import sys
from pathlib import Path

import numpy as np

KEEP = (
    "snapshot_steps", "final_eta", "final_delta", "final_Phi", "final_U", "final_V",
    "snapshot_eta", "snapshot_delta", "snapshot_Phi", "snapshot_U", "snapshot_V",
    "phase_angles", "phase_curve", "spinup", "geopot",
)


def main(ref_root: str) -> None:
    src = Path(ref_root) / "unit_tests" / "fixtures"
    dst = Path(__file__).resolve().parent
    for name in ("reference_case_unforced_test1", "reference_case_forced_default"):
        z = np.load(src / f"{name}.npz")
        out = {k: np.asarray(z[k]) for k in KEEP}
        for k in z.files:
            if k.startswith("param_"):
                out[k] = np.asarray(z[k])
        np.savez_compressed(dst / f"{name}.npz", **out)
        print("wrote", dst / f"{name}.npz")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/reference")
    main(sys.argv[1])
