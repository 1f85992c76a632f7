"""Benchmark of the GB300 Projective Dynamics substep: PD substeps/s.

A step is one PD substep (predict, K iterations, velocity update) of the workload's cloth(s).
Default workload: the 40×40 cloth with distance, shear and bend constraints, 40 iterations and
a 1e-3·|g| residual gate (``pd_gb300.workloads.cloth40_full``), in the MIXED precision mode.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--precision MODE]
                  [--impl ours|reference]

Prints one JSON line. ``value`` times the substep kernel with its data resident in HBM (CUDA
events on the simulator's stream, L2 flushed between timed steps); ``e2e`` times the same
substeps through the C ABI with the state copied from pinned host memory and read back every
step. Beside them: ``pos_err`` (the mode's position error against the FP64 CPU oracle after the
workload's full substep count), ``fp64_gpu`` (the plain one-cloth-per-launch FP64 GPU path on the
same workload) and ``cpu_baseline``. ``--impl reference`` times the CPU oracle (the reference
algorithm restated) on all host cores instead. Under torchrun each rank steps its own cloth(s)
(replicas; no collective on the data path) and rank 0 reports the aggregate. The default run
(N = 1) also carries the metric's other parts, ``batch512`` (``--workload batch``), ``cloth256``
(the single large cloth) and ``gradients`` (``--workload differentiable``), measured by this script
as child processes. ``precision_variants`` times the other precision modes on the same workload,
each with its position error against the oracle.
"""
from __future__ import annotations

import argparse
import copy
import json
import os
import statistics
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "PD substeps/s (1 cloth & 512-batch) vs plain FP64 GPU at 1e-5 pos err; grads/s"
# precision modes of the GPU substep: name -> (PD_PRECISION_* value, arithmetic label)
PRECISIONS = {"fp64-exact": (0, "f64"), "fp64": (1, "f64"), "fp32-projection": (2, "f64 (f32 projection)"),
              "fp32-solve": (3, "f64 (f32 solve + f64 refinement)"),
              "mixed": (4, "f32 (positions as f32 hi/lo pairs)")}
POS_ERR_BOUND = 1e-5
# σ of the finite-difference directions in scaled units (relative κ, m/s, vertex weights)
FD_SCALE = 100.0


def kernel_name(info):
    """The substep kernel a simulator launches, from its solve kind and CTAs per cloth."""
    kind, ctas = info["solve_kind"], info["cluster_ctas"]
    if kind == 0:
        return "substepExactKernel"
    if kind == 1:
        return "substepGridKernel" if ctas > 16 else "substepClusterKernel" if ctas > 1 else "substepFastKernel"
    if kind == 2:
        return "substepMixedGridKernel" if ctas > 16 else "substepMixedClusterKernel" if ctas > 1 else "substepMixedKernel"
    if kind == 3:
        return "substepDenseClusterKernel"
    if kind == 4:
        return "substepDeltaKernel"
    if kind == 6:
        return "substepDelta64Kernel"
    return "substepCorrGridKernel" if ctas > 16 else "substepCorrClusterKernel" if ctas > 1 else "substepCorrKernel"


UNIT = "substeps/s"
L2_FLUSH_BYTES = 256 << 20


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=None)  # default: 600 substeps, 30 batch substeps, 3 gradient batches
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--workload", default="cloth40_full")
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--precision", default="mixed", choices=list(PRECISIONS))
    p.add_argument("--batch-count", type=int, default=512)
    # CTAs per cloth for the timed handle (pd_scene_config.cluster_ctas; 0 = the planner's): e.g. 16
    # keeps the FP64 supernodal cluster kernel on a small cloth instead of the FP64 team kernel
    p.add_argument("--cluster-ctas", type=int, default=0)
    p.add_argument("--cpu-sample-seconds", type=float, default=10.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-pos-err", action="store_true")
    p.add_argument("--no-fp64-gpu", action="store_true")
    p.add_argument("--no-cheb", action="store_true")
    p.add_argument("--no-autotune", action="store_true")
    p.add_argument("--no-refactor", action="store_true")
    p.add_argument("--no-headline-parts", action="store_true")  # skip the batch / gradient children
    # other precision modes on the same workload, each timed and checked against the oracle
    p.add_argument("--variants", default=None, help="comma-separated modes; default per workload, 'none' to skip")
    p.add_argument("--grad-batch", type=int, default=64)       # differentiable workload: problems per launch
    p.add_argument("--fd-directions", type=int, default=64)
    p.add_argument("--grad-side", type=int, default=64)         # smaller only for profiling captures
    p.add_argument("--grad-substeps", type=int, default=120)
    a = p.parse_args()
    if a.steps is None:
        a.steps = {"differentiable": 3, "batch": 30}.get(a.workload, 600)
    if a.variants is None:
        a.variants = {"cloth40_full": "fp64,fp32-projection,fp32-solve", "cloth40_plain": "fp64,fp32-projection",
                      "cloth256": "fp64,fp32-projection,fp32-solve"}.get(a.workload, "none")
    a.variants = [] if a.variants == "none" else [m for m in a.variants.split(",") if m and m != a.precision]
    return a


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def replica_rate(units_per_rank, seconds, world, device=None):
    """Whole-job rate of `world` replicas that each processed `units_per_rank` units in `seconds`
    (this rank's time): the slowest rank sets it (MAX over ranks; the replicas exchange nothing
    else). Returns (rate, max seconds)."""
    import torch
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    t_max = float(t.item())
    return world * units_per_rank / t_max, t_max


def workload(name, batch_count, precision="mixed", cluster_ctas=0):
    import copy
    from pd_gb300 import workloads as W
    if name == "batch":
        scenes, cfgs, sub = W.batch(count=batch_count)
    else:
        scenes, cfg, sub = W.WORKLOADS[name]()
        cfgs = [cfg] * len(scenes)
    cfgs = [copy.copy(c) for c in cfgs]
    for c in cfgs:
        c.precision = PRECISIONS[precision][0]
        c.cluster_ctas = cluster_ctas
    return scenes, cfgs, sub


L2_NOTE = ("GPU arm: a 256 MB device write between timed substeps, outside the timed events; "
           "CPU arms: caches not flushed")


def describe_workload(name, scenes, cfgs, substeps):
    """The workload's description, the same for every arm: built from the cloths' array sizes and
    the configuration knobs, which the product's scenes and the oracle's meshes both carry."""
    c = cfgs[0]
    n = sum(s.n for s in scenes)
    e = sum(int(s.edges.shape[0]) for s in scenes)
    b = sum(int(np.asarray(s.bends).reshape(-1, 3).shape[0]) for s in scenes)
    return {"workload": name, "instances": len(scenes), "vertices": n, "constraints": e, "bend_stencils": b,
            "iterations": c.max_iterations, "residual_tolerance": c.residual_tolerance, "dt": c.dt,
            "substeps_per_run": substeps, "l2": L2_NOTE}


# --------------------------------------------------------------------------------- roofline
def algorithmic_bytes(scene, factor_nnz, iterations, precision="fp64"):
    """Bytes one substep must move: projection and
    scatter, the two triangular solves over the factor's F entries, the residual, prediction and
    velocity update. FP32 projection reads 12-byte positions; an FP32 solve reads 4-byte values."""
    n = scene.n
    E = int(scene.edges.shape[0])
    S = int(np.asarray(scene.bends).reshape(-1, 3).shape[0])
    F = factor_nnz
    xb = 12 if precision in ("fp32-projection", "mixed") else 24
    vb = 4 if precision in ("fp32-solve", "mixed") else 8
    b_ps = xb * n + 24 * n * 2 + (24 * n if S else 0) + 24 * E + 8 * E + 4 * (n + 1) + n
    b_solve = 2 * F * (vb + 4) + vb * n + 8 * (n + 1) + 2 * 24 * n + 8 * n
    b_res = 24 * n * 5 + 8 * n + 32 * E + 4 * (n + 1) + ((3 * S * 12 + 24 * S) if S else 0)
    return iterations * (b_ps + b_solve + b_res) + 96 * n + 72 * n


def fp64_ops(scene, factor_nnz, iterations):
    """FP64 operations one substep issues (sqrt and divide counted as one each)."""
    n = scene.n
    E = int(scene.edges.shape[0])
    S = int(np.asarray(scene.bends).reshape(-1, 3).shape[0])
    F = factor_nnz
    edge = E * (3 + 5 + 1 + 1 + 3 + 3 + 6)        # rel, dot, sqrt, div, d, κd, residual term
    gather = 2 * E * 3 + n * 3                     # scatter sums
    solve = 3 * (2 * F * 2 + n)                     # mul + sub per factor entry, both sweeps
    res = 2 * E * 3 + 3 * S * 9 + n * 16           # residual sums, bend force, inertia + norm
    return iterations * (edge + gather + solve + res) + edge + n * 12


def profiled_traffic(kernel, workload_name, precision):
    """DRAM bytes per substep of `kernel` on this workload from a committed ncu summary: a line
    'bench-traffic <kernel> <workload> <precision>: <bytes>' in profiles/*.md, else None."""
    key = f"bench-traffic {kernel} {workload_name} {precision}:"
    d = os.path.join(ROOT, "profiles")
    try:
        names = sorted(os.listdir(d))
    except OSError:
        return None
    for nm in names:
        if not nm.endswith(".md"):
            continue
        with open(os.path.join(d, nm)) as f:
            for line in f:
                if line.strip().startswith(key):
                    try:
                        return float(line.split(":", 1)[1].split()[0])
                    except (ValueError, IndexError):
                        return None
    return None


def read_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# --------------------------------------------------------------------------------- clocks
# clocks-event reason bits of NVML (nvml.h: nvmlClocksEventReason*), the ones a run is judged by
_NVML_REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
                 0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}


class _Nvml:
    """Read-only NVML queries through ctypes (the driver's libnvidia-ml): SM clock, its maximum and
    the active clocks-event reasons of one GPU. Never changes a setting."""

    def __init__(self, cuda_index):
        import ctypes as C
        self.C = C
        self.lib = C.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.dev = C.c_void_p()
        bus = None
        try:
            import torch
            p = torch.cuda.get_device_properties(cuda_index)
            bus = f"{p.pci_domain_id:08x}:{p.pci_bus_id:02x}:{p.pci_device_id:02x}.0".encode()
        except Exception:  # noqa: BLE001 — older torch: fall back to the index
            bus = None
        ok = bus is not None and self.lib.nvmlDeviceGetHandleByPciBusId_v2(bus, C.byref(self.dev)) == 0
        if not ok and self.lib.nvmlDeviceGetHandleByIndex_v2(int(cuda_index), C.byref(self.dev)) != 0:
            raise OSError("no NVML handle for the device")
        reasons = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None)
        self.reasons_fn = reasons or self.lib.nvmlDeviceGetCurrentClocksThrottleReasons

    def sample(self):
        C = self.C
        sm, smax, r = C.c_uint(), C.c_uint(), C.c_ulonglong()
        self.lib.nvmlDeviceGetClockInfo(self.dev, 1, C.byref(sm))        # NVML_CLOCK_SM
        self.lib.nvmlDeviceGetMaxClockInfo(self.dev, 1, C.byref(smax))
        self.reasons_fn(self.dev, C.byref(r))
        return float(sm.value), float(smax.value), int(r.value)

    def close(self):
        self.lib.nvmlShutdown()


class ClockSampler:
    """SM clocks and throttle reasons during a timed region: NVML polled every millisecond from a
    thread (the timed regions of short runs last a few milliseconds), else nvidia-smi every 100 ms.
    stop() returns {sm_mhz (median), sm_max_mhz, reasons, samples, source}."""

    def __init__(self, index, period_s=0.001):
        import threading
        self.samples = []
        self.proc = None
        self.nvml = None
        try:
            self.nvml = _Nvml(index)
        except Exception:  # noqa: BLE001 — NVML missing: nvidia-smi below
            self.nvml = None
        if self.nvml is not None:
            self.stop_flag = threading.Event()

            def run():
                while not self.stop_flag.is_set():
                    try:
                        self.samples.append(self.nvml.sample())
                    except Exception:  # noqa: BLE001
                        break
                    self.stop_flag.wait(period_s)

            self.samples.append(self.nvml.sample())
            self.thread = threading.Thread(target=run, daemon=True)
            self.thread.start()
            return
        out = os.environ.get("PD_BENCH_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(out, f"clocks_bench_{os.getpid()}.csv")
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.nvml is not None:
            self.stop_flag.set()
            self.thread.join(timeout=5)
            try:
                self.samples.append(self.nvml.sample())
            except Exception:  # noqa: BLE001
                pass
            self.nvml.close()
            sm = [s[0] for s in self.samples]
            reasons = sorted({nm for _, _, r in self.samples for bit, nm in _NVML_REASONS.items() if r & bit})
            return {"sm_mhz": statistics.median(sm) if sm else None,
                    "sm_max_mhz": max(s[1] for s in self.samples) if sm else None,
                    "reasons": reasons, "samples": len(sm), "source": "NVML, 1 ms"}
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "source": "nvidia-smi, 100 ms"}


# ----------------------------------------------------------------------------- CPU baseline
def time_oracle(name, batch_count, warmup, steps, max_seconds=None, threads=0):
    """The reference algorithm (the oracle's restatement) on the host cores, on the workload built
    by the oracle alone (``oracle/workloads.py``; the product library is never loaded): `warmup`
    untimed substeps (at least one: the first substep factorizes), then up to `steps` timed
    substeps of every cloth, stopping early once `max_seconds` of timed work have run. The same
    substeps as the GPU arm times: the ones after the warm-up, from the workload's initial state.
    Returns (meshes, configs, workload substeps, substeps timed, seconds, threads)."""
    from oracle import oracle as O, workloads as OW  # checker / CPU baseline only
    ncores = threads or os.cpu_count() or 1
    meshes, ocfgs, sub = OW.build(name, batch_count, threads=ncores)
    sims = [O.OracleSim(m, c) for m, c in zip(meshes, ocfgs)]
    for _ in range(max(1, warmup)):
        for s in sims:
            s.step(1)
    done, t_total = 0, 0.0
    for _ in range(steps):
        t0 = time.perf_counter()
        for s in sims:
            s.step(1)
        t_total += time.perf_counter() - t0
        done += 1
        if max_seconds is not None and t_total > max_seconds:
            break
    return meshes, ocfgs, sub, done, t_total, ncores


def cpu_baseline(name, batch_count, warmup, steps, max_seconds):
    """The oracle on the host cores: substeps/s over a bounded sample of the same workload — the
    substeps the GPU arm times, cut short after `max_seconds`."""
    meshes, _, _, done, t, ncores = time_oracle(name, batch_count, warmup, steps, max_seconds)
    return {"value": len(meshes) * done / t, "unit": UNIT, "cores": ncores, "kind": "port",
            "sample": f"substeps {max(1, warmup) + 1}..{max(1, warmup) + done} of the workload "
                      f"({len(meshes)} cloth(s)) on the CPU oracle, {t:.1f} s, OpenMP {ncores} threads"}


def run_reference(args):
    """The reference arm: the reference algorithm (oracle restatement; the reference itself needs
    Eigen, which is not installed) on all host cores, timed over exactly `steps` substeps after
    `warmup`, on the workload built by the oracle alone. Imports nothing of the product."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    meshes, ocfgs, sub, done, dt, ncores = time_oracle(args.workload, args.batch_count, args.warmup, args.steps)
    value = len(meshes) * done / dt  # aggregate (cloth-)substeps/s
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt / done * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": describe_workload(args.workload, meshes, ocfgs, sub), "impl": "reference",
            "precision": "fp64", "parallelism": f"{ncores} host threads (OpenMP)",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": ncores, "kind": "port",
                             "sample": f"substeps {max(1, args.warmup) + 1}..{max(1, args.warmup) + done} of the "
                                       f"workload, CPU oracle (reference algorithm restated), OpenMP {ncores} threads"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------------------------ ours
def time_fp64_gpu(P, args, stream, flush, max_steps=10):
    """Substeps/s of the plain FP64 GPU path (supernodal solve, one cloth per launch) on the
    workload, timed like `value`: one launch per substep, L2 flushed between substeps."""
    import torch
    scenes, cfgs, _ = workload(args.workload, args.batch_count, "fp64")
    sim = P.Simulator(scenes, cfgs)
    sim.set_stream(stream.cuda_stream)
    if not args.no_autotune:  # the baseline gets the same autotuner
        sim.autotune(5)
    k = min(args.steps, max_steps)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(k)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(k)]
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            sim.step(1, sync=False)
            flush.fill_(1.0)
        for j in range(k):
            flush.fill_(float(j))
            starts[j].record(stream)
            sim.step(1, sync=False)
            ends[j].record(stream)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in zip(starts, ends)) / k
    return {"value": len(scenes) * 1e3 / ms, "unit": UNIT, "steps": k, "kernel": kernel_name(sim.info(0)),
            "ctas_per_cloth": sim.info(0)["cluster_ctas"], "plan": sim.plan()}


def chebyshev_line(P, args, stream, flush, max_steps=100):
    """The reference's Chebyshev mode (PD_CHEB=1: ρ 0.98 after 10 plain iterations) on the same
    single-cloth workload and precision: substeps/s timed like `value`, and the last residual after
    the workload's substeps with and without it (equal iteration budget)."""
    import torch
    scenes, cfgs, sub = workload(args.workload, args.batch_count, args.precision)
    res = {}
    for mode in (0, 1):
        cs = [copy.copy(c) for c in cfgs]
        for c in cs:
            c.cheb_mode = mode
        sim = P.Simulator(scenes, cs)
        sim.set_stream(stream.cuda_stream)
        if mode == 1:
            k = min(args.steps, max_steps)
            starts = [torch.cuda.Event(enable_timing=True) for _ in range(k)]
            ends = [torch.cuda.Event(enable_timing=True) for _ in range(k)]
            with torch.cuda.stream(stream):
                for _ in range(args.warmup):
                    sim.step(1, sync=False)
                    flush.fill_(1.0)
                for j in range(k):
                    flush.fill_(float(j))
                    starts[j].record(stream)
                    sim.step(1, sync=False)
                    ends[j].record(stream)
            torch.cuda.synchronize()
            ms = sum(a.elapsed_time(b) for a, b in zip(starts, ends)) / k
            sim = P.Simulator(scenes, cs)
        sim.step(sub)
        res[mode] = sim.stats(0)["last_residual"]
    return {"value": len(scenes) * 1e3 / ms, "unit": UNIT, "steps": k, "rho": 0.98, "plain_iterations": 10,
            "last_residual": res[1], "last_residual_plain": res[0], "substeps": sub}


def time_fp64_one_at_a_time(P, args, budget_s=120.0):
    """Aggregate cloth-substeps/s of the batch run one cloth per launch through the plain FP64
    path: every cloth gets its own simulator, one warm-up and one timed substep (CUDA events);
    the per-cloth times are summed. Past `budget_s` of wall time the remaining cloths are
    extrapolated from the mean of those timed."""
    import torch
    scenes, cfgs, _ = workload(args.workload, args.batch_count, "fp64")
    times = []
    wall = time.perf_counter()
    for s, c in zip(scenes, cfgs):
        sim = P.Simulator([s], [c])
        sim.step(1)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        sim.step(1, sync=False)
        b.record()
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b) / 1e3)
        del sim
        if time.perf_counter() - wall > budget_s:
            break
    total = sum(times) * len(scenes) / len(times)
    return {"value": len(scenes) / total, "unit": UNIT, "cloths_timed": len(times), "cloths": len(scenes),
            "how": "one cloth per launch, plain FP64 path, per-cloth launch times summed"}


def refactor_times(P, scenes, cfgs):
    """A stiffness change of cloth 0 (every κ × 1.1, then × 1.2): milliseconds of the numeric
    refactorization on the GPU (the default outside FP64_EXACT) and through the host LDLᵀ
    (PD_GB300_HOST_REFACTOR=1), each including the re-upload and, for the team kernel, the
    explicit inverse."""
    sim = P.Simulator([scenes[0]], [cfgs[0]])
    k = np.asarray(scenes[0].edge_stiffness, np.float64)
    out = {}
    for name, scale, host in (("device_ms", 1.1, False), ("host_ms", 1.2, True)):
        if host:
            os.environ["PD_GB300_HOST_REFACTOR"] = "1"
        try:
            t0 = time.perf_counter()
            sim.set_edge_stiffness(k * scale)
            out[name] = (time.perf_counter() - t0) * 1e3
        finally:
            os.environ.pop("PD_GB300_HOST_REFACTOR", None)
    out["device_factorizations"] = sim.info(0)["device_factorize_count"]
    return out


def stage_shares(P, scenes, cfgs, plan, substeps=20):
    """Where a substep's time goes (StageTimes, core/sim/Scene.h:140-149): device stage times of
    cloth 0 over `substeps` substeps on a separate handle with the timed plan, as shares of the
    total, beside the total per substep."""
    sim = P.Simulator(scenes, cfgs)
    sim.set_plan(plan)
    sim.set_stage_timing(True)
    sim.step(substeps)
    t = sim.stage_times(0)
    total = t["total"]
    keys = ("predict", "local_step", "scatter", "solve", "unpack_scan", "velocity")
    out = {k: (t[k] / total if total > 0 else 0.0) for k in keys}
    out["ms_per_substep"] = total / substeps * 1e3
    return out


_ORACLE_FINAL = {}


def oracle_final(P, name, scenes, cfgs, substeps, picks):
    """Final positions of the FP64 CPU oracle after `substeps` substeps from the initial state, for
    the cloths `picks` (each with the elimination order the GPU handle uses); computed once per
    workload and kept, so that every precision mode is compared with the same reference run."""
    from tests.helpers import oracle_twin  # checker only
    out = {}
    for i in picks:
        key = (name, i, substeps)
        if key not in _ORACLE_FINAL:
            c = copy.copy(cfgs[i])
            c.precision = PRECISIONS["fp64"][0]
            probe = P.Simulator([scenes[i]], [c])
            perm = probe.factor(0)["perm"]
            probe.close()
            orc = oracle_twin(scenes[i], cfgs[i], perm=perm, threads=os.cpu_count())
            orc.step(substeps)
            _ORACLE_FINAL[key] = orc.state()[0]
        out[i] = _ORACLE_FINAL[key]
    return out


def position_error(P, args, scenes, cfgs, substeps, plan=None, bound=POS_ERR_BOUND):
    """max |x_gpu − x_oracle| / max |x_oracle| after `substeps` substeps from the initial state, this
    precision mode against the FP64 CPU oracle, for the run as timed: every cloth on one handle with
    the timed launch plan; checked on cloth 0 and on the largest cloth."""
    from tests.helpers import max_rel  # checker only
    sim = P.Simulator(scenes, cfgs)
    if plan is not None:
        sim.set_plan(plan)
    sim.step(substeps)
    picks = sorted({0, int(np.argmax([sc.n for sc in scenes]))})
    want = oracle_final(P, args.workload, scenes, cfgs, substeps, picks)
    errs = {str(i): max_rel(sim.state(i)[0], want[i]) for i in picks}
    err = max(errs.values())
    return {"value": err, "bound": bound, "within": bool(err <= bound), "substeps": substeps,
            "cloths": errs, "against": "FP64 CPU oracle (reference algorithm restated), cloths of the run as timed"}


def time_mode(P, args, stream, flush, precision, max_steps=50):
    """Substeps/s of one precision mode on the workload, timed like `value` (autotuned plan, one
    launch per substep, L2 flushed between substeps, CUDA events on the simulator's stream)."""
    import torch
    scenes, cfgs, _ = workload(args.workload, args.batch_count, precision)
    sim = P.Simulator(scenes, cfgs)
    sim.set_stream(stream.cuda_stream)
    if not args.no_autotune:
        sim.autotune(3)
    k = min(args.steps, max_steps)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(k)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(k)]
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            sim.step(1, sync=False)
            flush.fill_(1.0)
        for j in range(k):
            flush.fill_(float(j))
            starts[j].record(stream)
            sim.step(1, sync=False)
            ends[j].record(stream)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in zip(starts, ends)) / k
    info = sim.info(0)
    return {"value": len(scenes) * 1e3 / ms, "unit": UNIT, "ms_per_step": ms, "steps": k,
            "kernel": kernel_name(info), "ctas_per_cloth": info["cluster_ctas"], "plan": sim.plan(),
            "dtype": PRECISIONS[precision][1]}, scenes, cfgs


def precision_variants(P, args, stream, flush, modes, substeps):
    """The workload in each of `modes`: throughput timed like `value` and the position error against
    the FP64 CPU oracle after the workload's `substeps` (with the timed plan). FP64's bar is 1e-10,
    the reduced-precision modes' 1e-5."""
    out = {}
    for mode in modes:
        try:
            line, scenes, cfgs = time_mode(P, args, stream, flush, mode)
            bound = 1e-10 if PRECISIONS[mode][0] <= 1 else POS_ERR_BOUND
            line["pos_err"] = position_error(P, args, scenes, cfgs, substeps, line["plan"], bound)
        except Exception as e:  # noqa: BLE001 — reported in the line, the main result stands
            line = {"error": f"{type(e).__name__}: {e}"[:300]}
        out[mode] = line
    return out


def headline_parts(args):
    """The other two parts of the metric (the 512-cloth batch and grads/s), each measured by this
    script as a child process on the same GPU after the single-cloth line: their key numbers for
    the default run's JSON line. A part that fails is reported with its error."""
    parts = {}
    runs = {"batch512": ["--workload", "batch", "--steps", "30", "--no-cpu-baseline"],
            "cloth256": ["--workload", "cloth256", "--steps", "20", "--no-cheb", "--cpu-sample-seconds", "5"],
            "gradients": ["--workload", "differentiable", "--steps", "1", "--no-cpu-baseline"]}
    for name, extra in runs.items():
        cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--warmup", str(args.warmup)] + extra
        try:
            r = subprocess.run(cmd, capture_output=True, text=True, timeout=900, env=dict(os.environ))
            line = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
        except Exception as e:  # noqa: BLE001 — reported in the line, the main result stands
            parts[name] = {"error": f"{type(e).__name__}: {e}"[:300]}
            continue
        keep = ("value", "unit", "ms_per_step", "e2e", "roofline", "pos_err", "fp64_gpu", "fp64_gpu_batched",
                "grad_check", "fp64", "cpu_baseline", "clocks", "config", "precision", "kernel", "plan", "autotune",
                "refactor", "precision_variants")
        parts[name] = {k: line[k] for k in keep if k in line}
        parts[name]["command"] = " ".join(["python", "bench.py", "--warmup", str(args.warmup)] + extra)
    return parts


def run_ours(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    import pd_gb300 as P

    scenes, cfgs, sub = workload(args.workload, args.batch_count, args.precision, args.cluster_ctas)
    total_count = len(scenes)
    described = describe_workload(args.workload, scenes, cfgs, sub)  # the whole workload, every rank's part
    parts = None
    if args.workload == "batch" and world > 1:
        # the batch's cloths split across the ranks (longest processing time first): each rank
        # steps its part, nothing crosses ranks until the final gather
        from pd_gb300 import partition as PT
        parts = PT.partition(PT.scene_costs(scenes, cfgs), world)
        scenes = [scenes[i] for i in parts[rank]]
        cfgs = [cfgs[i] for i in parts[rank]]
    sim = P.Simulator(scenes, cfgs)
    stream = torch.cuda.Stream()
    sim.set_stream(stream.cuda_stream)
    # launch plan: the autotuner times candidates on this workload (outside every timed region)
    tune = None
    if not args.no_autotune:
        t0 = time.perf_counter()
        rep = sim.autotune(3 if len(scenes) > 1 else 20)
        tune = {"candidates": len(rep["tried"]), "chosen": rep["tried"][rep["chosen"]],
                "chosen_ms": rep["ms"][rep["chosen"]], "builtin_ms": rep["ms"][0],
                "seconds": time.perf_counter() - t0}
    plan = sim.plan()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # ---- value: device-resident state, one launch per substep, L2 flushed between steps
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            sim.step(1, sync=False)
            flush.fill_(1.0)
    barrier()
    sampler = ClockSampler(local) if rank == 0 else None
    t_wall = time.perf_counter()
    iters_used = []
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.fill_(float(k))
            starts[k].record(stream)
            sim.step(1, sync=False)
            ends[k].record(stream)
    barrier()
    t_wall = time.perf_counter() - t_wall
    clocks = sampler.stop() if sampler else None
    for i in range(sim.count):
        it, _ = sim.iteration_log(i)
        iters_used.append(int(it[0]))
    ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    kernel_ms = ms / args.steps
    count = len(scenes)
    value, t_max = replica_rate(count * args.steps, ms / 1e3, world, "cuda")  # aggregate (cloth-)substeps/s
    if parts is not None:  # a partitioned batch: every rank's cloths together, over the slowest rank's time
        value = total_count * args.steps / t_max

    # ---- e2e: through the C ABI's host-state call (pd_sim_step_host): every step copies every
    # cloth's positions and velocities in from pinned host memory, runs the substep and copies
    # them back (gather kernel → substep → scatter kernel, one CUDA graph replay), and returns
    # when the results are in host memory
    host = []
    for i in range(count):
        x0, v0 = sim.state(i)
        host.append((torch.from_numpy(x0.copy()).pin_memory(), torch.from_numpy(v0.copy()).pin_memory()))
    sim.set_stream(None)
    sim.bind_host([hx.numpy() for hx, _ in host], [hv.numpy() for _, hv in host])

    def e2e_step():
        sim.step_host(1)

    for _ in range(args.warmup):
        e2e_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    barrier()
    e2e_s = time.perf_counter() - t0
    h2d = d2h = sum(2 * 24 * sc.n for sc in scenes)
    e2e_value, e2e_max = replica_rate(count * args.steps, e2e_s, world, "cuda")
    if parts is not None:
        e2e_value = total_count * args.steps / e2e_max
    gathered = None
    if parts is not None:  # the one cross-rank data step: final states to rank 0, after all timing
        from pd_gb300 import partition as PT
        states = PT.gather_states(parts, [sim.state(i) for i in range(count)], rank, world)
        gathered = None if states is None else len(states)

    # ---- the plain one-cloth-per-launch FP64 GPU path on the same workload, and the position
    # error of this mode against the FP64 CPU oracle after the workload's full substep count
    fp64_line = pos_err = refactor = stages = None
    if rank == 0:
        if len(scenes) == 1 and not args.no_refactor:
            refactor = refactor_times(P, scenes, cfgs)
        stages = stage_shares(P, scenes, cfgs, plan) if len(scenes) == 1 else None
        if not args.no_fp64_gpu:
            fp64_line = (time_fp64_one_at_a_time(P, args) if len(scenes) > 1
                         else time_fp64_gpu(P, args, stream, flush))
        if not args.no_pos_err:
            pos_err = position_error(P, args, scenes, cfgs, sub, plan)

    if rank == 0:
        info = sim.info(0)
        kernel = kernel_name(info)
        per_launch_bytes = sum(algorithmic_bytes(s, sim.info(i)["factor_nnz"], iters_used[i], args.precision)
                               for i, s in enumerate(scenes))
        peak, peak_kind = read_peaks()
        achieved = per_launch_bytes / (kernel_ms * 1e-3) / 1e9
        traffic = profiled_traffic(kernel, args.workload, args.precision)
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": kernel_ms, "higher_is_better": True,
                "scaling": "strong" if parts is not None else "weak",
                "vs_baseline": None, "dtype": PRECISIONS[args.precision][1], "data": "synthetic",
                "config": described,
                "precision": args.precision,
                "parallelism": (f"batch split over {world} ranks, {count} of {total_count} cloths on rank 0, "
                                f"final states gathered ({gathered})" if parts is not None
                                else f"replicas x{world}" if world > 1 else "single GPU"),
                "kernel": {"name": kernel, "ctas_per_cloth": info["cluster_ctas"], "factor_nnz": info["factor_nnz"],
                           "iterations_used_last_timed_substep": iters_used[0]},
                "wall_s": t_wall,
                "gpu_launches": args.steps,
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                             "kernel": kernel, "algorithmic_bytes_per_launch": per_launch_bytes},
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                        "call": "pd_sim_step_host (gather kernel, substep, scatter kernel: one CUDA graph)"
                        if info["host_state"] == P.PD_HOST_STATE_GRAPH else "pd_sim_step_host (cudaMemcpyAsync per array)"},
                "clocks": clocks, "plan": plan, "autotune": tune, "refactor": refactor, "stages": stages}
        if PRECISIONS[args.precision][0] <= 1:
            ops = sum(fp64_ops(s, sim.info(i)["factor_nnz"], iters_used[i]) for i, s in enumerate(scenes))
            fp64_peak = 503.4  # Gop/s, measured DMUL/DADD/DFMA issue rate on this GPU
            fp64_achieved = ops / (kernel_ms * 1e-3) / 1e9
            line["fp64"] = {"achieved_gops": fp64_achieved, "peak_gops": fp64_peak,
                            "frac": fp64_achieved / fp64_peak, "ops_per_launch": ops}
        if fp64_line is not None:
            fp64_line["ratio"] = value / fp64_line["value"]
            line["fp64_gpu"] = fp64_line
            if len(scenes) > 1 and not args.no_fp64_gpu:
                batched = time_fp64_gpu(P, args, stream, flush)
                batched["ratio"] = value / batched["value"]
                line["fp64_gpu_batched"] = batched
        if pos_err is not None:
            line["pos_err"] = pos_err
        if len(scenes) == 1 and not args.no_cheb:
            line["chebyshev"] = chebyshev_line(P, args, stream, flush)
        if args.variants:
            line["precision_variants"] = precision_variants(P, args, stream, flush, args.variants, sub)
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(args.workload, args.batch_count, args.warmup, args.steps,
                                                args.cpu_sample_seconds)
        if args.workload == "cloth40_full" and world == 1 and not args.no_headline_parts:
            del sim  # free the device before the children run
            line.update(headline_parts(args))
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


# ------------------------------------------------------------------------- gradients (C5)
def grad_problems(count, side=64, substeps=120):
    """`count` differentiable problems on one side×side cloth (64×64, 120 substeps: the workload;
    smaller only for profiling captures): hidden stiffness κ* from seeds 1..count, targets = final
    positions of an FP64 run with κ*; parameters at κ = 2300, v0 = 0, f = 0."""
    import pd_gb300 as P
    from pd_gb300 import workloads as W
    scene, cfg, S, _ = W.differentiable(side=side, substeps=substeps)
    cfg = copy.copy(cfg)
    cfg.precision = PRECISIONS["fp64"][0]
    kstars = [W.differentiable(side=side, substeps=substeps, seed=s + 1)[3] for s in range(count)]
    ref = P.Simulator([scene] * count, [cfg] * count)
    for i, k in enumerate(kstars):
        ref.set_edge_stiffness(k, i)
    ref.step(S)
    targets = [ref.state(i)[0] for i in range(count)]
    return scene, cfg, S, targets


def _cpu_gradient_worker(job):
    """One spawned process: builds differentiable problem `i` with the oracle alone (targets from an
    oracle run at the hidden κ*), waits for the others, then times one serial FP64 adjoint."""
    i, barrier = job
    from oracle import oracle as O, workloads as OW  # checker / CPU baseline only
    mesh, cfg, S, _ = OW.differentiable(threads=1)
    twin = O.OracleSim(mesh, cfg)
    twin.set_edge_stiffness(OW.differentiable(seed=i + 1)[3])
    twin.step(S)
    target = twin.state()[0]
    orc = O.OracleSim(mesh, cfg)
    barrier.wait()
    t0 = time.perf_counter()
    orc.gradient(S, target, np.zeros((mesh.n, 3)))
    return time.perf_counter() - t0


def cpu_gradients(workers=None):
    """The oracle's FP64 adjoint on every host core: one problem per spawned process, all started
    together; grads/s = problems ÷ the slowest process's time."""
    import multiprocessing as mp
    workers = workers or os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        barrier = mgr.Barrier(workers)
        with ctx.Pool(workers) as pool:
            times = pool.map(_cpu_gradient_worker, [(i, barrier) for i in range(workers)])
    return {"value": workers / max(times), "unit": "grads/s", "cores": workers, "kind": "port",
            "sample": f"{workers} problems, one per process, the oracle's serial FP64 adjoint each "
                      f"(slowest {max(times):.2f} s)"}


def run_gradients(args):
    """Gradients/s of the adjoint on a batch of differentiable problems, with the checks: central
    differences of the GPU loss on 64 random directions (ε = 1e-6 and 1e-4) and the FP64 CPU
    reference gradient (oracle) on problem 0."""
    import torch
    import pd_gb300 as P
    from tests.helpers import oracle_twin  # checker only
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    count = args.grad_batch
    scene, cfg, S, targets = grad_problems(count, args.grad_side, args.grad_substeps)
    zero = np.zeros((scene.n, 3))
    sim = P.Simulator([scene] * count, [cfg] * count)
    for _ in range(args.warmup):
        sim.gradient(S, targets, [zero] * count)
    sampler = ClockSampler(local)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        grads = sim.gradient(S, targets, [zero] * count)
    dt = time.perf_counter() - t0
    clocks = sampler.stop()
    value = count * args.steps / dt
    # central differences of the loss of problem 0 along random directions, one batched launch each.
    # The FP64 loss carries ~2e-10 relative rounding noise (the forward map over 1200 solves), so a
    # difference quotient resolves 1e-6 only when the step moves the loss by ~1e-4 of itself: the
    # directions are drawn in scaled units — each κ_e relative to itself, v₀ in m/s, the force in
    # units of the vertex's weight — with σ = FD_SCALE, so that ε = 1e-6 moves every parameter by
    # ~1e-4 of its scale (well inside the range where the O(ε²) truncation term is negligible)
    rng = np.random.default_rng(1)
    k0 = np.asarray(scene.edge_stiffness, np.float64)
    weight = np.asarray(scene.masses, np.float64)[:, None] * 9.81
    g0 = grads[0]
    dirs = [(k0 * rng.normal(0.0, FD_SCALE, k0.shape), rng.normal(0.0, FD_SCALE, (scene.n, 3)),
             weight * rng.normal(0.0, FD_SCALE, (scene.n, 3))) for _ in range(args.fd_directions)]
    # directional derivatives of the adjoint, and the scale ‖g‖·‖d‖ of each (per parameter group)
    adjs = np.array([g0["dkappa"] @ dk + np.sum(g0["dv0"] * dv) + np.sum(g0["dforce"] * df) for dk, dv, df in dirs])
    scales = np.array([np.linalg.norm(g0["dkappa"]) * np.linalg.norm(dk) + np.linalg.norm(g0["dv0"]) * np.linalg.norm(dv)
                       + np.linalg.norm(g0["dforce"]) * np.linalg.norm(df) for dk, dv, df in dirs])
    # central differences D(ε) at a ladder of steps, each ladder rung one batched launch of 2 problems
    # a direction (loss only); Richardson's R(ε) = (4·D(ε/2) − D(ε))/3 cancels the O(ε²) term, so a
    # larger ε (less amplified rounding noise) keeps the truncation error small
    ladder = (1e-6, 5e-6, 1e-5, 2e-5, 5e-5, 1e-4, 2e-4)
    D = {}
    fd_sim = P.Simulator([scene] * (2 * len(dirs)), [cfg] * (2 * len(dirs)))
    for eps in ladder:
        forces = []
        for j, (dk, dv, df) in enumerate(dirs):
            for s, sign in enumerate((1.0, -1.0)):
                i = 2 * j + s
                fd_sim.set_edge_stiffness(k0 + sign * eps * dk, i)
                fd_sim.set_state(i, scene.positions, sign * eps * dv)
                forces.append(sign * eps * df)
        losses = fd_sim.gradient(S, [targets[0]] * (2 * len(dirs)), forces, grad=False)
        D[eps] = np.array([(losses[2 * j]["loss"] - losses[2 * j + 1]["loss"]) / (2 * eps) for j in range(len(dirs))])
    del fd_sim

    def fd_stats(fds):
        errs = np.abs(fds - adjs) / np.maximum(np.abs(adjs), 1e-300)
        return {"max_rel": float(errs.max()), "median_rel": float(np.median(errs)),
                "directions_within_1e-6": int(np.sum(errs <= 1e-6)),
                "normwise_rel": float(np.linalg.norm(fds - adjs) / max(np.linalg.norm(adjs), 1e-300)),
                "max_rel_to_gradient_scale": float(np.max(np.abs(fds - adjs) / np.maximum(scales, 1e-300)))}

    fd_err = {f"eps_{eps:g}": fd_stats(D[eps]) for eps in ladder}
    fd_err["richardson"] = {f"eps_{eps:g}": fd_stats((4.0 * D[eps / 2] - D[eps]) / 3.0)
                            for eps in ladder if eps / 2 in D}
    # FP64 CPU reference gradient of problem 0
    orc = oracle_twin(scene, cfg, perm=sim.factor(0)["perm"])
    tc = time.perf_counter()
    r = orc.gradient(S, targets[0], zero)
    cpu_s = time.perf_counter() - tc
    rel = {k: float(np.linalg.norm(g0[k] - r[k]) / max(np.linalg.norm(r[k]), 1e-300))
           for k in ("dkappa", "dv0", "dforce")}
    info = sim.info(0)
    n3 = 3 * scene.n
    # roofline: a gradient runs the S·K forward iterations and S·K adjoint solves, each at least as
    # much traffic as a FP64 substep's iteration (algorithmic_bytes), over the measured launch time
    F = info["factor_nnz"]
    per_launch = count * 2 * S * algorithmic_bytes(scene, F, cfg.max_iterations, "fp64")
    peak, peak_kind = read_peaks()
    achieved = per_launch / (dt / args.steps) / 1e9
    fp64_gops = count * 2 * S * fp64_ops(scene, F, cfg.max_iterations) / (dt / args.steps) / 1e9
    line = {"metric": METRIC, "value": value, "unit": "grads/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "differentiable", "problems": count, "vertices": scene.n,
                       "edges": int(scene.edges.shape[0]), "substeps": S, "iterations": cfg.max_iterations,
                       "gradient_of": "mean squared distance of free vertices to targets w.r.t. per-edge stiffness, "
                                      "initial velocities, external force",
                       "kernel": "gradientClusterKernel" if info["cluster_ctas"] > 1 else "gradientKernel",
                       "ctas_per_problem": info["cluster_ctas"],
                       "factor_nnz": info["factor_nnz"], "l2": "not flushed (each step is seconds long)"},
            "gpu_launches": args.steps,
            "e2e": {"value": value, "unit": "grads/s", "h2d_bytes_per_step": count * 2 * 8 * n3,
                    "d2h_bytes_per_step": count * (8 * (2 * n3 + scene.edges.shape[0]) + 8)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None, "peak_kind": peak_kind,
                         "kernel": "gradientClusterKernel" if info["cluster_ctas"] > 1 else "gradientKernel",
                         "algorithmic_bytes_per_launch": per_launch},
            "fp64": {"achieved_gops": fp64_gops, "peak_gops": 503.4, "frac": fp64_gops / 503.4},
            "grad_check": {"fd_directions": len(dirs), "fd_direction_sigma": FD_SCALE,
                           "fd_direction_units": "κ_e relative, v₀ m/s, force in vertex weights", **fd_err, "vs_cpu_reference_rel": rel,
                           "loss_problem0": g0["loss"], "loss_cpu_reference": r["loss"]},
            "clocks": clocks,
            "cpu_baseline": ({"value": 1.0 / cpu_s, "unit": "grads/s", "cores": 1, "kind": "port",
                              "sample": "one gradient of problem 0 by the oracle's serial FP64 adjoint"}
                             if args.no_cpu_baseline else cpu_gradients())}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.workload == "differentiable":
        if args.impl == "reference":
            return run_reference_gradients(args)
        return run_gradients(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


def run_reference_gradients(args):
    """The oracle's FP64 adjoint on every host core (one problem per process), per gradient; the
    reference has no gradient of its own."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import workloads as OW  # the reference arm loads nothing of the product
    scene, _, S, _ = OW.differentiable()
    steps = max(1, min(args.steps, 3))
    runs = [cpu_gradients() for _ in range(steps)]
    value = statistics.median(r["value"] for r in runs)
    cb = dict(runs[0], value=value)
    line = {"metric": METRIC, "value": value, "unit": "grads/s", "n_gpus": args.gpus, "steps": steps,
            "warmup": 0, "ms_per_step": 1e3 / value, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "differentiable", "problems": cb["cores"], "vertices": scene.n, "substeps": S},
            "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": value, "unit": "grads/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
