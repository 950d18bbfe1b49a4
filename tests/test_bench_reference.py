"""The reference arm of bench.py (the reference's serial solver, restated in
the oracle, timed on the host cores) prints one complete JSON line; CPU only,
on small samples."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_complete_line():
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3",
                          "--sample-scale", "7"], cwd=ROOT, capture_output=True, text=True, check=True,
                         timeout=600).stdout
    d = json.loads(out.strip().splitlines()[-1])
    assert d["impl"] == "reference" and d["unit"] == "MTEPS" and d["value"] > 0
    for k in ("metric", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling", "dtype",
              "data", "config"):
        assert k in d, k
    assert d["steps"] == 1 and d["warmup"] == 3 and d["higher_is_better"] is True
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and "scale-7" in cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "MTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
