"""bench.py's output contract, on the CPU.

- The reference arm (`--impl reference`: the oracle's FP64 step and its
  autograd adjoint on the host cores) prints one JSON line with the keys the
  bench line carries, its own value as `cpu_baseline` and `e2e`, and no host <->
  device bytes.
- The roofline's per-launch DRAM traffic comes from the committed ncu
  summaries: every kernel the roofline names has one, with its
  `traffic_bytes_per_launch` line, and the algorithmic bytes per launch follow
  the column counts of the kernels (J x (M+1) complex values per member and
  column).
"""
import json
import subprocess
import sys

import pytest

from conftest import ROOT

KEYS = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
        "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e")


def test_reference_arm_prints_one_contract_line():
    cmd = [sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "1",
           "--ref-nsteps", "2"]
    out = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, check=True).stdout
    lines = [ln for ln in out.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1, out
    d = json.loads(lines[0])
    for k in KEYS:
        assert k in d, k
    assert d["impl"] == "reference" and d["higher_is_better"] is True and d["steps"] == 1
    assert d["value"] > 0 and d["unit"] == "member-steps/s"
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["kind"] in ("port", "reference")
    assert d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


@pytest.mark.parametrize("kernel", ["spectral", "grid", "grid_adj", "spectral_adj"])
def test_roofline_traffic_and_algorithmic_bytes(kernel):
    sys.path.insert(0, str(ROOT))
    import bench

    traffic = bench._ncu_traffic(kernel)
    assert traffic is not None and traffic > 0, kernel
    alg = bench._algorithmic_bytes(kernel, 256)
    cols = {"spectral": 22, "grid": 12, "grid_adj": 18, "spectral_adj": 23}[kernel]
    assert alg == cols * 64 * 43 * 8 * 256
    # the capture moved no more than the columns the kernel must touch, plus a
    # small slack for the basis and coefficient tables: no wasted re-reads
    assert traffic <= 1.05 * alg, (kernel, traffic, alg)
