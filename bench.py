"""Benchmark: D3Q19 A-A lid-driven cavity, MLUPS on GB300.

Workload (default): the 384^3 FP32 lid-driven cavity (lid u_x = 0.05,
Re = 1000, nu = 0.0192, tau = 0.5576), initialised at rest.  One bench
"step" is one lattice time step over the whole domain (alpha on even
counters, beta on odd, as src/CController.cpp:1278-1287 alternates them);
MLUPS counts interior cells x steps (src/CController.cpp:1463-1464).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--storage f32|f64|f16s|bf16s|f16sr] [--size 384] [--variant V] [--fma]
    python bench.py --workload batch|serve|precision [--batch-storages f32,f16s,f16sr]
                    [--batch-variant V] [--batch-count 512] [--batch-steps 2000]

Prints ONE JSON line (rank 0).  Keys beyond the base contract:
  roofline      -- dominant kernel's algorithmic bytes / CUDA-event time vs
                   the measured HBM copy bandwidth (MEASURED_PEAKS.json)
  cpu_baseline  -- the CPU oracle (a port of the reference kernels, OpenMP
                   over all host cores) on a bounded slab of the same domain
  e2e           -- the same job through the C ABI with pinned host buffers:
                   upload of the full population state, K steps, download of
                   density and velocity fields, all inside the timed region
  clocks        -- SM clocks and throttle reasons sampled during timing
N > 1 (torchrun): independent replicas, one cavity per GPU ("replicas
only": the single-domain path has no exchange step), max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BYTES_PER_VALUE = {"f64": 8, "f32": 4, "f16s": 2, "bf16s": 2, "f16sr": 2}
DTYPE_NAME = {"f64": "f64", "f32": "f32", "f16s": "f16 (shifted, fp32 collide)", "bf16s": "bf16 (shifted, fp32 collide)",
              "f16sr": "f16 (shifted, scaled 2^12, stochastic rounding, fp32 collide)"}
METRIC = "MLUPS"
L2_BYTES = 129 * 1024 * 1024


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--storage", default="f32", choices=list(BYTES_PER_VALUE))
    ap.add_argument("--size", type=int, default=384)
    ap.add_argument("--variant", type=int, default=-1, help="launch variant (default: the library's for the storage)")
    ap.add_argument("--fma", action="store_true", help="f64: fuse the collision's multiply-adds (not bit-exact)")
    ap.add_argument("--lid", type=float, default=0.05)
    ap.add_argument("--nu", type=float, default=0.0192)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU time of the CPU baseline sample")
    ap.add_argument("--workload", default="cavity", choices=["cavity", "batch", "precision", "serve"],
                    help="cavity: the single-domain benchmark line; batch / precision: the extension measurements")
    ap.add_argument("--no-extensions", action="store_true", help="skip the bounded extension measurements")
    ap.add_argument("--batch-count", type=int, default=512)
    ap.add_argument("--batch-steps", type=int, default=2000)
    ap.add_argument("--batch-storages", default="f32,f16s,f16sr", help="storages of --workload batch / serve")
    ap.add_argument("--batch-variant", type=int, default=-1,
                    help="register variant of --workload batch (default: autotuned per storage)")
    ap.add_argument("--batch-single-size", type=int, default=384,
                    help="--workload batch: edge of the single-domain comparison cavity (0: none)")
    ap.add_argument("--precision-size", type=int, default=512)
    ap.add_argument("--precision-steps", type=int, default=5000)
    ap.add_argument("--serve-count", type=int, default=10000)
    ap.add_argument("--serve-step-scale", type=float, default=0.01)
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def config_dict(a, world):
    return {"workload": f"lid-driven cavity {a.size}^3 {a.storage}, Re={a.size * a.lid / a.nu:.0f}, "
                        f"u_lid={a.lid}, nu={a.nu}", "domain": [a.size] * 3, "storage": a.storage,
            "step": "one lattice time step (alpha/beta alternating), whole domain",
            "l2": f"inputs larger than L2: {19 * (a.size + 2) ** 3 * BYTES_PER_VALUE[a.storage] / 1e9:.2f} GB "
                  f"population array vs {L2_BYTES / 1e6:.0f} MB L2",
            "parallelism": f"replicas x{world}" if world > 1 else "single domain, 1 GPU",
            **({"fused_multiply_add": True} if getattr(a, "fma", False) else {})}


# ---------------------------------------------------------------------------
# CPU legs (oracle as the checker/baseline only)
# ---------------------------------------------------------------------------

def cpu_run(a, seconds_target, steps_max=None, use_reference=True, threads=None):
    """Time the reference algorithm on host cores over z-slabs of the domain.

    Uses the reference's own CPU kernels (oracle/_ref) where they were built
    for this host and load (the reference runs them on one thread), else the C
    port (oracle/liblbm_oracle.so) with OpenMP over `threads` threads (default:
    all cores).  Returns (mlups, cores, kind, sample)."""
    from oracle import oracle as orc

    dtype = np.float64 if a.storage == "f64" else np.float32
    kind = "port"
    lib = None
    if use_reference and os.path.exists(orc.REF_SO):
        try:
            lib, kind = orc.Reference(), "reference"
        except OSError:  # built for another host architecture
            lib = None
    if lib is None:
        orc.build()
        lib = orc.Oracle()
        lib.set_num_threads(threads if threads else os.cpu_count() or 1)
    cores = lib.num_threads() if kind == "port" else 1
    n = a.size
    _, itau = orc.tau_of(a.nu, dtype)
    lid = dtype(a.lid)
    dd, flags = lib.init(n, n, n, dtype)
    flags[1:-1, n, 1:-1] = orc.VELOCITY_INJECTION
    # calibrate slab thickness on one alpha/beta pair of 2 planes
    probe = (1, 1, 1), (n, n, min(2, n))
    t0 = time.perf_counter()
    lib.alpha(dd, flags, itau, lid, origin=probe[0], size=probe[1])
    lib.beta(dd, flags, itau, lid, origin=probe[0], size=probe[1])
    rate = 2 * n * n * probe[1][2] / max(time.perf_counter() - t0, 1e-6)
    steps = 10 if steps_max is None else steps_max
    planes = int(max(1, min(n, seconds_target * rate / (steps * n * n))))
    o, s = (1, 1, 1), (n, n, planes)
    t0 = time.perf_counter()
    for i in range(steps):
        if i & 1:
            lib.beta(dd, flags, itau, lid, origin=o, size=s)
        else:
            lib.alpha(dd, flags, itau, lid, origin=o, size=s)
    dt = time.perf_counter() - t0
    mlups = n * n * planes * steps / dt / 1e6
    sample = (f"{steps} steps over a {n}x{n}x{planes} interior slab of the {n}^3 domain "
              f"({n * n * planes * steps / 1e6:.1f} M lattice updates, {dt:.1f} s)")
    return mlups, cores, kind, sample


def cpu_baseline(a):
    """The reference CPU path as the reference runs it (one thread: its
    kernels are not parallelised), and the C port over every host core."""
    one, cores1, kind1, sample1 = cpu_run(a, a.cpu_seconds / 3, use_reference=True, threads=1)
    allc, cores, kind, sample = cpu_run(a, a.cpu_seconds, use_reference=False)
    return {"value": round(one, 3), "unit": "MLUPS", "cores": cores1, "kind": kind1,
            "sample": sample1 + "; 1 core used, the reference CPU kernels' own parallelism",
            "nproc": os.cpu_count(),
            "all_cores": {"value": round(allc, 3), "unit": "MLUPS", "cores": cores, "kind": kind, "sample": sample}}


def reference_arm(a):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as orc

    dtype = np.float64 if a.storage == "f64" else np.float32
    use_ref = os.path.exists(orc.REF_SO)
    lib = orc.Reference() if use_ref else None
    if lib is None:
        orc.build()
        lib = orc.Oracle()
    kind = "reference" if use_ref else "port"
    cores = 1 if use_ref else lib.num_threads()
    n = a.size
    _, itau = orc.tau_of(a.nu, dtype)
    lid = dtype(a.lid)
    dd, flags = lib.init(n, n, n, dtype)
    flags[1:-1, n, 1:-1] = orc.VELOCITY_INJECTION
    gpu_kernels = reference_gpu_kernels(dd, flags, itau, lid, n)
    # per-step sample: a z-slab sized so K+W steps take about two minutes
    probe = (1, 1, 1), (n, n, min(2, n))
    t0 = time.perf_counter()
    lib.alpha(dd, flags, itau, lid, origin=probe[0], size=probe[1])
    lib.beta(dd, flags, itau, lid, origin=probe[0], size=probe[1])
    rate = 2 * n * n * probe[1][2] / max(time.perf_counter() - t0, 1e-6)
    budget = 120.0 / max(1, a.steps + a.warmup)
    planes = int(max(1, min(n, budget * rate / (n * n))))
    o, s = (1, 1, 1), (n, n, planes)
    for i in range(a.warmup):
        (lib.beta if i & 1 else lib.alpha)(dd, flags, itau, lid, origin=o, size=s)
    t0 = time.perf_counter()
    for i in range(a.steps):
        j = a.warmup + i
        (lib.beta if j & 1 else lib.alpha)(dd, flags, itau, lid, origin=o, size=s)
    dt = time.perf_counter() - t0
    value = n * n * planes * a.steps / dt / 1e6
    sample = f"each step: one lattice update of a {n}x{n}x{planes} slab of the {n}^3 domain"
    line = {"metric": METRIC, "value": round(value, 3), "unit": "MLUPS", "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": round(dt / a.steps * 1e3, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": DTYPE_NAME[a.storage], "data": "synthetic",
            "config": config_dict(a, world), "impl": "reference",
            "cpu_baseline": {"value": round(value, 3), "unit": "MLUPS", "cores": cores, "kind": kind,
                             "sample": sample},
            "e2e": {"value": round(value, 3), "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if gpu_kernels is not None:
        line["gpu_kernels"] = gpu_kernels
    print(json.dumps(line), flush=True)


def reference_gpu_kernels(dd, flags, itau, lid, n, steps=200, warmup=4):
    """MLUPS of the reference's own CUDA alpha/beta kernels on this GPU
    (oracle/ref_gpu.py: src/gpukernels built from source for sm_103a with the
    reference's nvcc flags, its 32x8x1 blocks), CUDA events over `steps`
    steps; None where the kernels were not built or no GPU is present."""
    try:
        import torch

        from oracle import ref_gpu
        if not (torch.cuda.is_available() and ref_gpu.available()):
            return None
        torch.cuda.set_device(0)
        stream = torch.cuda.current_stream()
        with ref_gpu.RefGpuCavity(dd, flags, itau, lid) as ref:
            ref.run(warmup, stream.cuda_stream)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ref.run(steps, stream.cuda_stream)
            e1.record(stream)
            e1.synchronize()
            ms = e0.elapsed_time(e1)
        return {"value": round(float(n) ** 3 * steps / (ms / 1e3) / 1e6, 1), "unit": "MLUPS", "steps": steps,
                "what": "the reference's own CUDA alpha/beta kernels (src/gpukernels, built from source for "
                        "sm_103a with its nvcc flags), 32x8x1 blocks over the domain with its halo, on this GPU"}
    except Exception as e:  # keep the CPU line whatever happens here
        return {"error": repr(e)}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_id: str):
        self.device_id = device_id
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", self.device_id, f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for name, val in zip(names, parts[3:7]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(a, kernel):
    """dram bytes per launch from a committed ncu summary, if one matches."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    d = json.load(open(p))
    key = f"{kernel}:{a.storage}"
    if key not in d:
        return None
    e = d[key]
    # scaled from the captured case to this domain by interior cells
    return e["dram_bytes_per_launch"] * (a.size ** 3) / float(e["cells"])


def batch_measure(storage, count, steps, device=0, variant=-1, ref_fields=None):
    """Aggregate MLUPS of the seeded batch of box cavities (512 edges in
    [16,96], lid in [0.02,0.1], Re log-uniform in [10,2000], seed 0), all
    advanced together; CUDA events around `steps` steps on one stream.  With
    `ref_fields` (velocities of the same batch run in FP64 for the same 4 +
    `steps` steps, batch_fields) the relative L2 and max velocity error of this
    storage against FP64 over every domain's interior."""
    import torch

    from cavityflow_cuda_gb300 import LbmBatch
    from cavityflow_cuda_gb300.workloads import batch_workload

    cav = batch_workload(count=count, seed=0)
    stream = torch.cuda.Stream()
    with LbmBatch([c.solver_args(storage) for c in cav], storage=storage, device=device) as b:
        if variant < 0:
            tuned = b.autotune(pairs=3)
        else:
            b.set_fast_variant(variant)
            tuned = (variant, [])
        b.run(4, stream=stream)
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.run(steps, stream=stream)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        info = b.info()
        err = velocity_error(batch_fields(b), ref_fields) if ref_fields is not None else None
    lups = float(info["interior_cells"]) * steps
    out = {"storage": storage, "domains": count, "steps": steps, "interior_cells": info["interior_cells"],
           "mlups": round(lups / (ms / 1e3) / 1e6, 1), "ms": round(ms, 2), "variant": tuned[0],
           "variant_ms_per_pair": [round(v, 4) for v in tuned[1]],
           "device_gb": round(info["device_bytes"] / 1e9, 3)}
    if err is not None:
        out["l2_err_vs_f64"], out["max_abs_err_vs_f64"] = err
    return out


def batch_fields(b):
    """Velocity of every domain of a batch (float64 copies)."""
    return [b.domain(i).getVelocities().astype(np.float64) for i in range(len(b))]


def batch_reference_fields(count, steps, device=0):
    """The seeded batch run in FP64 for `steps` steps; its velocity fields."""
    from cavityflow_cuda_gb300 import LbmBatch
    from cavityflow_cuda_gb300.workloads import batch_workload

    cav = batch_workload(count=count, seed=0)
    with LbmBatch([c.solver_args("f64") for c in cav], storage="f64", device=device) as b:
        b.run(steps)
        return batch_fields(b)


def velocity_error(fields, ref):
    """Relative L2 norm of the velocity difference over all fields, and the
    largest absolute difference."""
    num = den = 0.0
    worst = 0.0
    for f, r in zip(fields, ref):
        d = f - r
        num += float((d * d).sum())
        den += float((r * r).sum())
        worst = max(worst, float(np.abs(d).max()))
    return (float(np.sqrt(num / den)) if den > 0 else 0.0), worst


def single_measure(storage, n, steps, device=0):
    """MLUPS of one n^3 cavity (the comparison point of the batch)."""
    import torch

    from cavityflow_cuda_gb300 import CLbmSolverGB300, derive_lattice

    lat = derive_lattice(velocity=(0.05, 0, 0), viscosity=0.0192, domain_size=(n, n, n), storage=storage)
    stream = torch.cuda.Stream()
    with CLbmSolverGB300((n, n, n), lat["inv_tau"], lat["velocity"][0], storage=storage, device=device) as s:
        s.run(4, stream=stream)
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s.run(steps, stream=stream)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
    return float(n) ** 3 * steps / (ms / 1e3) / 1e6


def precision_measure(n, steps, nu=0.0512, lid=0.1, device=0, fp64_fma=True):
    """L2 and max velocity error of FP32, FP16-shifted and BF16-shifted storage
    against an FP64 run of this solver (same cavity), the FP64 mass drift, and
    each storage's MLUPS (CUDA events around the run).  fp64_fma: the FP64 run
    uses the fused multiply-add kernels (1.4x faster; within 1e-15 of the
    unfused FP64 over 1000 steps, far below the errors measured here)."""
    import torch

    from cavityflow_cuda_gb300 import CLbmSolverGB300
    from cavityflow_cuda_gb300.workloads import lattice_tau

    res = {"domain": [n] * 3, "steps": steps, "lid": lid, "nu": nu, "re": round(n * lid / nu, 1)}
    fields = {}
    for storage in ("f64", "f32", "f16s", "bf16s", "f16sr"):
        _, inv_tau = lattice_tau(nu, storage)
        T = np.float64 if storage == "f64" else np.float32
        stream = torch.cuda.Stream()
        fma = fp64_fma and storage == "f64"
        with CLbmSolverGB300((n, n, n), inv_tau, float(T(lid)), storage=storage, device=device,
                             fused_multiply_add=fma) as s:
            m0 = s.reduce()[0]
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s.run(steps, stream=stream)
            e1.record(stream)
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            fields[storage] = s.getVelocities().astype(np.float64)
            m1 = s.reduce()[0]
        res[storage] = {"mlups": round(float(n) ** 3 * steps / (ms / 1e3) / 1e6, 1),
                        "mass_drift_rel": float((m1 - m0) / m0)}
    ref = fields["f64"]
    norm = np.sqrt((ref ** 2).sum())
    for storage in ("f32", "f16s", "bf16s", "f16sr"):
        d = fields[storage] - ref
        res[storage]["l2_err_vs_f64"] = float(np.sqrt((d ** 2).sum()) / norm)
        res[storage]["max_abs_err_vs_f64"] = float(np.abs(d).max())
    res["f64"]["fused_multiply_add"] = bool(fp64_fma)
    res["f16s_speedup_vs_f32"] = round(res["f16s"]["mlups"] / res["f32"]["mlups"], 3)
    res["f16sr_speedup_vs_f32"] = round(res["f16sr"]["mlups"] / res["f32"]["mlups"], 3)
    return res


def serve_measure(storage, count, step_scale, budget_gb=150.0, rate=200.0, seed=1, target_ms=50, device=0,
                  l2_sample=0, l2_max_edge=64):
    """p50/p99 latency and aggregate MLUPS of the seeded request stream (cube
    edges {32..256} weighted, steps uniform in [500, 20000] times step_scale,
    lid 0.05, Re log-uniform in [10, 5000], Poisson arrivals), replayed in
    real time against a server with a budget_gb HBM budget.  l2_sample > 0:
    the results of the first l2_sample requests with edges up to l2_max_edge
    are kept and compared with the same cavities solved alone in FP64
    (relative L2 velocity error over the sample)."""
    from cavityflow_cuda_gb300 import LbmServer
    from cavityflow_cuda_gb300.workloads import serving_workload

    reqs = serving_workload(count=count, seed=seed, rate=rate)
    steps = [max(2, int(round(r.steps * step_scale))) for r in reqs]
    sample = [i for i in range(count) if reqs[i].size[0] <= l2_max_edge][:l2_sample]
    sampled = set(sample)
    kept = {}
    lat, wait, lups = [], [], 0
    with LbmServer(budget_bytes=int(budget_gb * 1e9), storage=storage, device=device, target_round_ms=target_ms,
                   max_round_steps=512) as srv:
        t0 = time.perf_counter()
        i, hsub, ids, done, first_arrival, last_finish = 0, {}, {}, 0, None, 0.0
        while done < count:
            now = time.perf_counter() - t0
            while i < count and reqs[i].arrival <= now:
                rid = srv.submit(*reqs[i].solver_args(storage), steps[i])
                ids[rid] = i
                hsub[rid] = time.perf_counter() - t0
                i += 1
            ran = srv.round()
            for c in srv.poll():
                k = ids[c["id"]]
                # finish - arrival, free of the offset between the two clocks
                lat.append((c["finish_time"] - c["submit_time"]) + (hsub[c["id"]] - reqs[k].arrival))
                wait.append(c["admit_time"] - c["submit_time"])
                lups += c["cells"] * c["steps"]
                last_finish = max(last_finish, hsub[c["id"]] + (c["finish_time"] - c["submit_time"]))
                if k in sampled:
                    kept[k] = srv.take_result(c["id"], copy=True)[1].astype(np.float64)
                else:
                    srv.take_result(c["id"], copy=False)
                done += 1
            if not ran and i < count:
                time.sleep(max(0.0, min(0.005, reqs[i].arrival - (time.perf_counter() - t0))))
        st = srv.stats()
    span = last_finish - reqs[0].arrival
    lat = np.array(lat)
    err = None
    if kept:
        from cavityflow_cuda_gb300 import CLbmSolverGB300

        ref = []
        for k in sample:
            size, inv_tau, lid_u = reqs[k].solver_args("f64")
            with CLbmSolverGB300(size, inv_tau, lid_u, storage="f64", device=device) as s:
                s.run(steps[k])
                ref.append(s.getVelocities().astype(np.float64))
        err = velocity_error([kept[k] for k in sample], ref)
    offered = sum(reqs[k].cells * steps[k] for k in range(count)) / max(reqs[-1].arrival - reqs[0].arrival, 1e-9)
    out = {"storage": storage, "requests": count, "step_scale": step_scale, "arrival_rate": rate,
           "offered_mlups": round(offered / 1e6, 1),
            "budget_gb": budget_gb, "p50_latency_s": round(float(np.percentile(lat, 50)), 3),
            "p99_latency_s": round(float(np.percentile(lat, 99)), 3),
            "p50_queue_wait_s": round(float(np.percentile(wait, 50)), 3),
            "aggregate_mlups": round(lups / span / 1e6, 1), "busy_mlups": round(st["lattice_updates"] /
                                                                               st["busy_seconds"] / 1e6, 1),
            "makespan_s": round(span, 2), "rounds": st["rounds"], "peak_gb": round(st["peak_bytes"] / 1e9, 2)}
    if err is not None:
        out["l2_err_vs_f64"], out["max_abs_err_vs_f64"] = err
        out["l2_sample"] = f"{len(sample)} requests (edges <= {l2_max_edge}), each solved alone in FP64"
    return out


def moving_wall_measure(n=384, steps=200, device=0):
    """The mass-conserving moving-wall lid beside the reference's injection
    lid: FP32 MLUPS of each at n^3 (lid 0.05, nu 0.0192; CUDA events around
    `steps` graph-replayed steps), and the relative FP64 mass change of each
    over 1000 steps of the 64^3 cavity (lid 0.05, nu 0.032, Re 100)."""
    import torch

    from cavityflow_cuda_gb300 import CLbmSolverGB300
    from cavityflow_cuda_gb300.workloads import lattice_tau

    out = {"domain": [n] * 3, "steps": steps}
    _, itau = lattice_tau(0.0192, "f32")
    for mode in ("injection", "wall"):
        stream = torch.cuda.Stream()
        with CLbmSolverGB300((n, n, n), itau, 0.05, storage="f32", device=device, lid=mode) as s:
            s.run(8, stream=stream)
            stream.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s.run(steps, stream=stream)
            e1.record(stream)
            e1.synchronize()
            ms = e0.elapsed_time(e1)
        out[f"{mode}_f32_mlups"] = round(float(n) ** 3 * steps / (ms / 1e3) / 1e6, 1)
        _, itau64 = lattice_tau(0.032, "f64")
        with CLbmSolverGB300((64, 64, 64), itau64, 0.05, storage="f64", device=device, lid=mode) as s:
            m0 = s.reduce()[0]
            s.run(1000)
            out[f"{mode}_f64_mass_change_rel_64cubed_1000_steps"] = float((s.reduce()[0] - m0) / m0)
    return out


def extensions(a):
    """The extension measurements at their stated configurations, attached to
    the benchmark line: precision (512^3, lid 0.1, nu 0.0512, 5000 steps, every
    storage against an FP64 run), the moving-wall lid beside the injection
    lid, the 512-cavity batch in FP32/F16S/F16SR with each 16-bit result's
    error against an FP64 batch, and the 10,000-request serving stream (steps
    scaled by --serve-step-scale) in FP32 and F16SR with the error of a sample
    against FP64 solves."""
    out = {}
    try:
        out["precision"] = precision_measure(a.precision_size, a.precision_steps)
        out["precision_note"] = (f"{a.precision_size}^3, {a.precision_steps} steps, lid 0.1, nu 0.0512 (Re 1000); "
                                 "errors against the FP64 run of this solver")
    except Exception as e:  # keep the main line whatever happens here
        out["precision_error"] = repr(e)
    try:
        out["moving_wall"] = moving_wall_measure()
    except Exception as e:
        out["moving_wall_error"] = repr(e)
    single = {}
    try:
        ref = batch_reference_fields(a.batch_count, 4 + a.batch_steps)
        for st in ("f32", "f16s", "f16sr"):
            out[f"batch_{st}"] = r = batch_measure(st, a.batch_count, a.batch_steps, ref_fields=ref)
            single[st] = round(single_measure(st, 384, 400), 1)
            r["single_domain_384_mlups"] = single[st]
            r["batch_over_single"] = round(r["mlups"] / single[st], 3)
        del ref
        out["batch_note"] = (f"batched MLUPS over the seeded {a.batch_count}-cavity workload, {a.batch_steps} "
                             "steps; velocity errors against the same batch in FP64; compare with "
                             "single-domain MLUPS")
    except Exception as e:
        out["batch_error"] = repr(e)
    try:
        for st in ("f32", "f16sr"):
            out[f"serve_{st}"] = r = serve_measure(st, a.serve_count, a.serve_step_scale, l2_sample=16)
            # at a small step scale the stream does not fill the GPU: aggregate = offered load
            r["arrival_bound"] = r["aggregate_mlups"] >= 0.95 * r["offered_mlups"]
        out["serve_note"] = (f"the seeded {a.serve_count}-request stream at 200 req/s, steps U[500,20000] scaled "
                             f"by {a.serve_step_scale}, 150 GB budget; offered_mlups = the stream's lattice updates "
                             "over its arrival window (when the aggregate matches it the GPU keeps up and is idle "
                             "between arrivals); the server's capacity on the unscaled stream: "
                             "profiles/serve_full_stream_f16sr.md")
    except Exception as e:
        out["serve_error"] = repr(e)
    return out


def main():
    a = parse()
    if a.impl == "reference":
        reference_arm(a)
        return
    if a.workload == "batch":
        import torch

        torch.cuda.set_device(0)
        storages = a.batch_storages.split(",")
        res = {s: batch_measure(s, a.batch_count, a.batch_steps, variant=a.batch_variant) for s in storages}
        if a.batch_single_size > 0:
            n = a.batch_single_size
            for s in storages:
                res[s][f"single_domain_{n}_mlups"] = round(single_measure(s, n, 400), 1)
                res[s]["batch_over_single"] = round(res[s]["mlups"] / res[s][f"single_domain_{n}_mlups"], 3)
        print(json.dumps({"workload": "batch", "results": res}), flush=True)
        return
    if a.workload == "serve":
        import torch

        torch.cuda.set_device(0)
        res = {s_: serve_measure(s_, a.serve_count, a.serve_step_scale) for s_ in a.batch_storages.split(",")}
        print(json.dumps({"workload": "serve", "results": res}), flush=True)
        return
    if a.workload == "precision":
        import torch

        torch.cuda.set_device(0)
        print(json.dumps({"workload": "precision", "results": precision_measure(a.precision_size, a.precision_steps)}),
              flush=True)
        return
    run_gpu(a)


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def combine_ranks(ms: float, units_per_rank: float, world: int, device=None):
    """Whole-job throughput of independent replicas: the slowest rank's time
    (all-reduce MAX) over the units all ranks processed.  Returns
    (max_ms, units_per_second)."""
    if world > 1:
        import torch
        import torch.distributed as dist

        t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, units_per_rank * world / (ms / 1e3)


def run_gpu(a):
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from cavityflow_cuda_gb300 import CLbmSolverGB300, derive_lattice, kernel_launches

    n = a.size
    lat = derive_lattice(velocity=(a.lid, 0, 0), viscosity=a.nu, domain_size=(n, n, n), timestep=1.0,
                         storage=a.storage)
    bpv = BYTES_PER_VALUE[a.storage]
    bytes_per_lup = 2 * 19 * bpv
    stream = torch.cuda.Stream()
    props = torch.cuda.get_device_properties(local)
    dev_id = str(getattr(props, "uuid", "")) or str(local)
    if dev_id and not dev_id.startswith("GPU-") and len(dev_id) == 36:
        dev_id = "GPU-" + dev_id

    with CLbmSolverGB300((n, n, n), lat["inv_tau"], lat["velocity"][0], storage=a.storage, device=local,
                         fused_multiply_add=a.fma) as s:
        assert s.info()["fast_path"] == 1
        if a.variant >= 0:
            s.set_fast_variant(a.variant)
        # warm-up (also captures the run graph)
        s.run(max(a.warmup, 3), stream=stream)
        stream.synchronize()
        barrier(world)
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = kernel_launches()
        with ClockSampler(dev_id) as clocks:
            torch.cuda.synchronize()
            ev0.record(stream)
            s.run(a.steps, stream=stream)
            ev1.record(stream)
            ev1.synchronize()
        launches = kernel_launches() - l0
        torch.cuda.synchronize()
        ms, lups_per_s = combine_ranks(ev0.elapsed_time(ev1), float(n) ** 3 * a.steps, world, device="cuda")
        barrier(world)
        value = lups_per_s / 1e6

        # per-kernel durations (CUDA events on the launching stream)
        per = {"alpha": [], "beta": []}
        for i in range(20):
            kind = "beta" if s.info()["last_step_was_alpha"] else "alpha"
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            (s.simulationStepBeta if kind == "beta" else s.simulationStepAlpha)(stream=stream)
            e1.record(stream)
            e1.synchronize()
            per[kind].append(e0.elapsed_time(e1))
        avg = {k: statistics.mean(v) for k, v in per.items() if v}
        dom = max(avg, key=avg.get)
        peak, peak_kind = measured_peaks()
        algo = bytes_per_lup * float(n) ** 3
        achieved = algo / (avg[dom] / 1e3) / 1e9
        info = s.info()
        kname = f"{dom}_fast" + ({1: "_blk", 2: "_direct", 3: "_pk"}.get(info["beta_block_exchange"], "")
                                 if dom == "beta" else "")
        if info["fast_variant"] >= s._lib.lbm_register_variant_count():  # the bulk-copy variants follow
            kname = "step_tma"
        traffic = profile_traffic(a, kname)
        roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic, "kernel": f"{kname}<{a.storage}>",
                "launch_variant": info["fast_variant"],
                "algorithmic_bytes_per_launch": algo, "peak_source": f"{peak_kind} hbm_gbs (copy)",
                "per_kernel_ms": {k: round(v, 4) for k, v in avg.items()},
                "per_kernel_frac": {k: round(algo / (v / 1e3) / 1e9 / peak, 4) for k, v in avg.items()}}

        # end to end through the C ABI with pinned host buffers
        e2e = None
        if not a.no_e2e:
            state = torch.empty((19, n + 2, n + 2, n + 2), dtype=torch.float64 if a.storage == "f64" else torch.float32,
                                pin_memory=True)
            s.getDensityDistributions((0, 0, 0), (n + 2, n + 2, n + 2), out=state.numpy())
            macro = torch.empty((4, n, n, n), dtype=state.dtype, pin_memory=True)
            mnp = macro.numpy()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s.setDensityDistributions(state.numpy(), (0, 0, 0), (n + 2, n + 2, n + 2), stream=stream)
            s.run(a.steps, stream=stream)
            stream.synchronize()
            s.getDensities(out=mnp[0])
            s.getVelocities(out=mnp[1:])
            t_e2e = time.perf_counter() - t0
            e2e = {"value": round(float(n) ** 3 * a.steps / t_e2e / 1e6 * world, 1), "unit": "MLUPS",
                   "h2d_bytes_per_step": int(state.numel() * state.element_size() / a.steps),
                   "d2h_bytes_per_step": int(macro.numel() * macro.element_size() / a.steps),
                   "how": "pinned host -> setDensityDistributions (full state), run(K), getDensities + "
                          "getVelocities -> pinned host; host wall clock"}

    cpu = None
    if rank == 0 and not a.no_cpu:
        cpu = cpu_baseline(a)

    ext = extensions(a) if (rank == 0 and world == 1 and not a.no_extensions) else None

    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 1), "unit": "MLUPS", "n_gpus": world, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": round(ms / a.steps, 5), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": DTYPE_NAME[a.storage], "data": "synthetic",
                "config": config_dict(a, world), "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
                "clocks": clocks.summary(), "gpu_launches": int(launches)}
        if ext is not None:
            line["extensions"] = ext
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
