"""bench.py's output contract on the CPU: the reference arm's JSON line (the oracle timed on the host
cores, no host-device bytes) and the per-substep algorithmic byte count behind the roofline."""
import json
import os
import subprocess
import sys
from types import SimpleNamespace

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "3",
                        "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "substeps/s" and d["higher_is_better"] is True
    assert d["steps"] == 3 and d["warmup"] == 3 and d["n_gpus"] == 1 and d["value"] > 0
    assert d["config"]["workload"] == "cloth40_full" and d["config"]["iterations"] == 40
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]


def test_algorithmic_bytes_per_substep():
    """B = K·(B_ps + B_solve + B_res) + 96n + 72n with 24-byte positions and 8-byte factor values in
    FP64, 12 and 4 in the MIXED mode (a 4-vertex scene with 5 edges, 2 bend stencils, F = 3, K = 2)."""
    sys.path.insert(0, ROOT)
    import bench

    scene = SimpleNamespace(n=4, edges=np.zeros((5, 2), np.int32), bends=np.zeros((2, 3), np.int32))
    n, E, S, F, K = 4, 5, 2, 3, 2

    def want(xb, vb):
        ps = xb * n + 48 * n + 24 * n + 32 * E + 4 * (n + 1) + n
        solve = 2 * F * (vb + 4) + vb * n + 8 * (n + 1) + 48 * n + 8 * n
        res = 120 * n + 8 * n + 32 * E + 4 * (n + 1) + 60 * S
        return K * (ps + solve + res) + 168 * n

    assert bench.algorithmic_bytes(scene, F, K, "fp64") == want(24, 8)
    assert bench.algorithmic_bytes(scene, F, K, "mixed") == want(12, 4)
    assert bench.algorithmic_bytes(scene, F, K, "fp32-projection") == want(12, 8)
    assert bench.algorithmic_bytes(scene, F, K, "fp32-solve") == want(24, 4)
