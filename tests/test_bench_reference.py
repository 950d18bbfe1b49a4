"""The reference arm of bench.py (the reference's serial solver -- its own
binary built from its sources when available, else the oracle's restatement
-- timed on the host cores) prints one complete JSON line, and its samples
come from the numpy restatement of the generator, so the process loads none
of the project's compiled code.  CPU only, on small samples."""
import json
import os
import subprocess
import sys

import numpy as np

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
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert "scale-7" in cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "MTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_sample_loads_no_project_code():
    code = ("import sys, bench\n"
            "m, dt, v, kind = bench._serial_sample(5, 8)\n"
            "maps = open('/proc/self/maps').read()\n"
            "print(m, v, kind, 'wbpr_gb300' in sys.modules, 'libwbpr' in maps)\n")
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, check=True,
                         timeout=300).stdout.split()
    assert out[-2:] == ["False", "False"], out
    assert int(out[0]) > 0 and out[2] in ("port", "reference")


def test_numpy_rmat_matches_the_library_generator():
    import wbpr_gb300 as W
    from oracle import rmat

    for scale, seed in ((6, 1), (9, 4), (11, 1001)):
        n, off, dst, cap, s, t = rmat.gen_rmat(scale, 16, 0.57, 0.19, 0.19, 1, 100, seed)
        g = W.gen_rmat(scale, 16, 0.57, 0.19, 0.19, 1, 100, seed)
        assert n == g.n and (s, t) == (g.s, g.t)
        assert np.array_equal(off, g.off) and np.array_equal(dst, g.dst) and np.array_equal(cap, g.cap)
