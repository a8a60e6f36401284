"""bench.py's own arm on a short run: the JSON line carries every key of the
measurement contract with consistent values (whole-job rate, roofline of the
dominant kernel, end-to-end through the C ABI with host buffers, launches)."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.gpu
def test_bench_line_contract():
    cmd = [sys.executable, "bench.py", "--steps", "3", "--warmup", "3", "--no-l1", "--no-cpu", "--no-clocks", "--no-tune",
           "--extra-workloads", "none", "--workload", "gas_water"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([x for x in r.stdout.splitlines() if x.startswith("{")][-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling", "vs_baseline",
              "dtype", "data", "config", "roofline", "e2e", "gpu_launches"):
        assert k in line, k
    assert line["n_gpus"] == 1 and line["steps"] == 3 and line["warmup"] == 3
    assert line["unit"] == "cell-updates/s" and line["higher_is_better"] is True and line["scaling"] == "weak"
    cells = line["config"]["cells"]
    assert cells == 16384 and line["config"]["workload"].startswith("gas_water")
    # the rate is the cells of one step over the step time
    assert line["value"] == pytest.approx(cells / (line["ms_per_step"] * 1e-3), rel=1e-6)
    rf = line["roofline"]
    assert rf["bound"] == "hbm" and rf["unit"] == "GB/s" and rf["peak"] > 0
    assert rf["frac"] == pytest.approx(rf["achieved"] / rf["peak"], rel=1e-9)
    assert rf["achieved"] == pytest.approx(rf["algorithmic_bytes_per_launch"] / (rf["kernel_ms"] * 1e-3) / 1e9, rel=1e-6)
    e2e = line["e2e"]
    blk = 8 * 256 * 8
    assert e2e["unit"] == "cell-updates/s" and e2e["value"] > 0
    assert e2e["d2h_bytes_per_step"] == 64 * blk and e2e["h2d_bytes_per_step"] >= 64 * blk
    # dt update + step per timed step, at least
    assert line["gpu_launches"] >= 2 * line["steps"]
