"""The reference arm of bench.py on the CPU: one JSON line with the contract's
keys, timed on the oracle (the CPU restatement of the reference method), and
no library of the GPU product mapped into the process."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_RUNNER = r"""
import json, sys
sys.argv = ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "1", "--workload", "gas_water"]
import bench
rc = bench.main()
maps = open("/proc/self/maps").read()
print(json.dumps({"rc": rc or 0, "product_loaded": "libg5gpu" in maps, "oracle_loaded": "libg5oracle" in maps}))
"""


def test_reference_arm_line_and_libraries():
    r = subprocess.run([sys.executable, "-c", _RUNNER], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    line, probe = lines[0], lines[-1]
    assert probe == {"rc": 0, "product_loaded": False, "oracle_loaded": True}
    assert line["impl"] == "reference"
    assert line["unit"] == "cell-updates/s" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["steps"] == 1 and line["warmup"] == 1 and line["n_gpus"] == 1
    assert line["config"]["workload"].startswith("gas_water") and line["config"]["cells"] == 16384
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
