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
    assert d["precision"] == "fp64" and d["dtype"] == "f64"
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]


def test_reference_arm_never_loads_the_product():
    """The reference arm builds its cloths with the oracle alone: after a run, neither the product
    package nor its library is in the process."""
    code = ("import sys, bench; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '1']; "
            "bench.main(); maps = open('/proc/self/maps').read(); "
            "print('PRODUCT', any(m.startswith('pd_gb300') for m in sys.modules), 'libpd_gb300' in maps, "
            "'libpd_oracle' in maps)")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    last = [ln for ln in r.stdout.splitlines() if ln.startswith("PRODUCT")][-1]
    assert last == "PRODUCT False False True"


def test_both_arms_describe_the_workload_identically(pdg):
    """`config` is built from the cloths and knobs alone, so the GPU arm (product scenes) and the CPU
    arms (oracle meshes) print the same dictionary for every workload."""
    sys.path.insert(0, ROOT)
    import bench
    from oracle import workloads as OW
    for name in ("cloth40_plain", "cloth40_full", "cloth256", "batch"):
        scenes, cfgs, sub = bench.workload(name, 24)
        meshes, ocfgs, osub = OW.build(name, 24)
        assert bench.describe_workload(name, scenes, cfgs, sub) == bench.describe_workload(name, meshes, ocfgs, osub)


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
