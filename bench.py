#!/usr/bin/env python3
"""Benchmark of the fused mass-spring step on one GB300 (or N replicas).

Workload: the single large lattice -- 100^3 = 1,000,000 masses and
12,731,796 springs (k log-uniform [1e3, 1e5], damping 0.1, 20% actuated),
frictional plane and a fixed ball, dt = 1e-4 (titan_gb300.workloads.actuated_lattice).
A step is one time step of the whole lattice; its working set (~0.4-0.6 GB)
is larger than L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

ours:      FP32-compensated fused step (headline), CUDA-graph replay, CUDA
           events on the engine's stream; plus an FP64 drop-in figure, an
           end-to-end figure through the C ABI with host buffers, and the
           CPU oracle timed on the host cores.
reference: the reference's per-spring / per-mass update functions restated
           on the host (the CPU oracle, OpenMP with atomics as the reference's
           kernels use) on all host threads, same workload and metric.
Prints one JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "spring-updates/s"
UNIT = "spring-updates/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3000)
    p.add_argument("--warmup", type=int, default=20)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--precision", default="f32c", choices=["f32c", "f64", "f32"])
    p.add_argument("--side", type=int, default=100)
    p.add_argument("--fp64-steps", type=int, default=200)
    p.add_argument("--e2e-chunk", type=int, default=100)
    p.add_argument("--e2e-calls", type=int, default=5)
    p.add_argument("--cpu-steps", type=int, default=8)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-fp64", action="store_true")
    p.add_argument("--tile", type=int, default=0)
    p.add_argument("--threads", type=int, default=0)
    p.add_argument("--kernel", type=int, default=0, help="0 auto, 1 per-tile, 2 pipelined")
    p.add_argument("--suite", action="store_true",
                   help="instead of the headline line: one JSON line per workload of the baseline table "
                        "(5^3, 100^3, 4096 bodies; engine FP64/FP32C, the reference's CUDA kernels, the CPU port)")
    p.add_argument("--precision-study", action="store_true",
                   help="instead of the headline line: 64^3 lattice at dt=1e-5, FP32 and FP32C against FP64")
    p.add_argument("--study-steps", type=int, default=20000)
    p.add_argument("--study-every", type=int, default=10000, help="steps between checkpoints of the precision study")
    p.add_argument("--study-ref-steps", type=int, default=100000,
                   help="steps of the reference's own CUDA kernels run beside the study's FP64 form")
    p.add_argument("--serving", action="store_true",
                   help="instead of the headline line: rollout serving, Poisson arrivals (p50/p99 latency)")
    p.add_argument("--serve-requests", type=int, default=400)
    p.add_argument("--serve-rate", type=float, default=200.0)
    p.add_argument("--serve-max-masses", type=int, default=200000)
    p.add_argument("--serve-small-masses", type=int, default=50000,
                   help="streams engine: requests below this many masses run the per-tile kernel (0: all automatic)")
    p.add_argument("--serve-rates", default="100,300,1000,3000,5000",
                   help="comma-separated arrival rates (req/s) to sweep, one JSON line each")
    p.add_argument("--serve-engine", default="device", choices=["device", "streams"],
                   help="device: the persistent request-server kernel; streams: one engine per request on its "
                        "own CUDA stream")
    p.add_argument("--serve-stream-masses", type=int, default=0,
                   help="device engine: requests of at least this many masses run on their own stream (0: none)")
    p.add_argument("--serve-prewarm", type=int, default=1,
                   help="device engine: build the engines the requests need before the clock starts (1) or not (0)")
    p.add_argument("--serve-bodies", type=int, default=0,
                   help="instead of the rate sweep: this many single-body robot rollouts (3-12 masses per side, "
                        "5000 steps) submitted at once")
    p.add_argument("--ref-gpu-steps", type=int, default=50,
                   help="steps of the reference's own CUDA kernels timed beside ours (0: skip)")
    return p.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def max_over_ranks(x: float, world: int, device="cuda") -> float:
    """The slowest rank's time: replicas report the whole job by it."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_rank: float, world: int, max_seconds: float) -> float:
    """Whole-job throughput of weak-scaled replicas: every rank processes
    units_per_rank; the job takes as long as its slowest rank."""
    return units_per_rank * world / max_seconds


def peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(precision: str):
    """DRAM bytes per launch of the step kernel from the committed ncu summary."""
    f = ROOT / "profiles" / "traffic.json"
    if not f.exists():
        return None
    try:
        d = json.loads(f.read_text())
        return d.get(precision, {}).get("dram_bytes_per_launch")
    except Exception:
        return None


KERNEL_NAMES = {"warp-specialised": "k_step_ws", "per-tile": "k_step",
                "per-tile-async": "k_step_async", "pull": "k_step_pull"}


class ClockSampler:
    """SM clocks and throttle reasons sampled while the timed region runs.

    NVML is read through ctypes (libnvidia-ml.so.1) every millisecond from a
    host thread, so that even a region of a few milliseconds is sampled (the
    engine's calls release the interpreter lock while they wait); without
    NVML, nvidia-smi polls every 10 ms.  Read-only queries: no GPU setting
    is changed."""

    # nvmlClocksEventReasons bits (nvml.h)
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.thread = None
        self.samples = []  # (sm_mhz, max_mhz, reasons set)
        self.source = None

    def _nvml_handle(self):
        import ctypes
        nv = ctypes.CDLL("libnvidia-ml.so.1")
        if nv.nvmlInit_v2() != 0:
            return None, None
        h = ctypes.c_void_p()
        bus = None
        try:
            import torch
            pr = torch.cuda.get_device_properties(self.device)
            dom, b, d = getattr(pr, "pci_domain_id", None), getattr(pr, "pci_bus_id", None), getattr(pr, "pci_device_id", None)
            if b is not None:
                bus = f"{dom or 0:08x}:{b:02x}:{d or 0:02x}.0".encode()
        except Exception:
            bus = None
        if bus is None or nv.nvmlDeviceGetHandleByPciBusId_v2(bus, ctypes.byref(h)) != 0:
            if nv.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(self.device), ctypes.byref(h)) != 0:
                return None, None
        return nv, h

    def _poll_nvml(self, nv, h):
        import ctypes
        clk, mx, rs = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
        get_reasons = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            nv.nvmlDeviceGetCurrentClocksThrottleReasons
        nv.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx))  # NVML_CLOCK_SM
        while not self._stop.is_set():
            if nv.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(clk)) == 0 and get_reasons(h, ctypes.byref(rs)) == 0:
                self.samples.append((float(clk.value), float(mx.value),
                                     {v for b, v in self.REASONS.items() if rs.value & b}))
            self._stop.wait(0.001)

    def __enter__(self):
        import threading
        self._stop = threading.Event()
        try:
            nv, h = self._nvml_handle()
        except Exception:
            nv, h = None, None
        if nv is not None:
            self.source = "nvml, 1 ms"
            self.thread = threading.Thread(target=self._poll_nvml, args=(nv, h), daemon=True)
            self.thread.start()
            return self
        try:
            self.source = "nvidia-smi, 10 ms"
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "10"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.thread is not None:
            self._stop.set()
            self.thread.join(timeout=5)
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            for ln in out.splitlines():
                parts = [x.strip() for x in ln.split(",")]
                if len(parts) < 7:
                    continue
                try:
                    sm, mx = float(parts[0]), float(parts[1])
                except ValueError:
                    continue
                self.samples.append((sm, mx, {nm for nm, v in zip(names, parts[3:7]) if v.lower().startswith("active")}))

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0, "source": self.source}
        reasons = set()
        for _, _, r in self.samples:
            reasons |= r
        return {"sm_mhz": statistics.median(x[0] for x in self.samples),
                "sm_max_mhz": max(x[1] for x in self.samples), "reasons": sorted(reasons),
                "samples": len(self.samples), "source": self.source}


def workload_config(side, nm, ns, world):
    """The `config` of the JSON line: the workload only, identical in both
    arms (engine details go under "engine")."""
    return {"workload": f"single {side}^3 lattice, {nm} masses, {ns} springs, 20% actuated, plane + ball, dt=1e-4",
            "masses": nm, "springs": ns, "step": "one time step of the whole lattice",
            "parallelism": "replicas" if world > 1 else "single GPU",
            "l2": "per-step working set larger than L2 (no flush)"}


def mapped_repo_libraries():
    """Shared libraries of this repository mapped into this process."""
    try:
        maps = Path("/proc/self/maps").read_text().splitlines()
    except OSError:
        return None
    libs = {ln.split()[-1] for ln in maps if ln.rstrip().endswith(".so") and str(ROOT) in ln}
    return sorted(str(Path(x).relative_to(ROOT)) for x in libs)


def cpu_oracle_rate(sc, steps, threads):
    from oracle import pyoracle as po
    o = po.OracleSim(sc)
    o.step(1, po.ATOMIC_OMP, threads)  # warm
    t0 = time.perf_counter()
    o.step(steps, po.ATOMIC_OMP, threads)
    dt = time.perf_counter() - t0
    return sc["left"].size * steps / dt, dt


def reference_kernels(sc, steps, device, value, fp64):
    """The reference's own CUDA kernels (computeSpringForces +
    massForcesAndUpdate, compiled from its sources) on the same scene and
    GPU: back to back (kernel-only) and with execute()'s per-step device
    synchronisation."""
    from oracle import refgpu
    why = refgpu.available()
    if why:
        return {"unavailable": why}
    ns = sc["left"].size
    r = refgpu.RefGpuSim(sc, device)
    try:
        r.step(3)
        ms = r.time_steps(steps)
        ms_sync = r.time_steps(max(1, steps // 2), sync_each=True) / max(1, steps // 2) * steps
    finally:
        r.close()
    out = {"value": ns * steps / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / steps,
           "ms_per_step_with_step_sync": ms_sync / steps, "steps": steps, "dtype": "f64",
           "speedup_of_headline": value / (ns * steps / (ms / 1e3)),
           "note": "reference src/sim.cu kernels, 1024-thread blocks, FP64 atomics; actuation at the reference's "
                   "fixed 0.2 amplitude (same actuated springs and omegas)"}
    if fp64:
        out["speedup_of_fp64"] = fp64["value"] / out["value"]
    return out


def run_ours(a, rank, world, local):
    import numpy as np
    import torch

    import titan_gb300 as tg
    from titan_gb300 import workloads as wl

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()


    prec = {"f32c": tg.FP32C, "f64": tg.FP64, "f32": tg.FP32}[a.precision]
    sc = wl.actuated_lattice(a.side)
    ns, nm = sc["left"].size, sc["pos"].shape[0]
    peak, peak_kind = peaks()

    def timed(sim, steps):
        stream = torch.cuda.ExternalStream(sim.stream, device=local)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        sim.step(steps)
        e1.record(stream)
        sim.synchronize()
        torch.cuda.synchronize()
        barrier()
        return e0.elapsed_time(e1)

    sim = wl.make_sim(sc, prec, a.tile, device=local, threads=a.threads, kernel=a.kernel)
    info = sim.plan_info()
    kinfo = sim.kernel_info()
    sim.step(a.warmup)
    # the graphs step(a.steps) replays are built before the timed region
    sim.prepare_steps(a.steps)
    sim.synchronize()
    with ClockSampler(local) as clk:
        ms = timed(sim, a.steps)
    ms_max = max_over_ranks(ms, world)
    st = sim.get_state(pos=True, vel=False)
    finite = bool(np.all(np.isfinite(st["pos"])))
    per_launch_s = ms / a.steps / 1e3
    alg = info["algorithmic_bytes_per_step"]
    achieved = alg / per_launch_s / 1e9
    value = replica_value(ns * a.steps, world, ms_max / 1e3)
    traffic = profiled_traffic(a.precision)

    def e2e(sim, chunk, calls):
        """Same metric end to end through the C ABI with host buffers: upload
        of positions and velocities from page-locked host arrays (moved by
        DMA, no staging copy), step(chunk), download of positions."""
        pos_h = tg.pinned_empty(sc["pos"].shape)
        pos_h[:] = sc["pos"]
        vel_h = tg.pinned_empty(sc["pos"].shape)
        vel_h[:] = 0.0
        out = {"pos": tg.pinned_empty(sc["pos"].shape)}
        sim.set_mass_state(None, pos=pos_h, vel=vel_h)
        sim.step(chunk)
        sim.get_state(pos=True, vel=False, out=out)
        barrier()
        t0 = time.perf_counter()
        for _ in range(calls):
            sim.set_mass_state(None, pos=pos_h, vel=vel_h)
            sim.step(chunk)
            sim.get_state(pos=True, vel=False, out=out)
        secs = max_over_ranks(time.perf_counter() - t0, world)
        barrier()
        return {"value": ns * chunk * calls * world / secs, "unit": UNIT, "h2d_bytes_per_step": 6 * nm * 8 / chunk,
                "d2h_bytes_per_step": 3 * nm * 8 / chunk, "steps_per_call": chunk, "calls": calls,
                "path": "C ABI: set_mass_state(page-locked host pos+vel) -> step(chunk) -> "
                        "get_state(page-locked host pos)"}

    e2e_main = e2e(sim, a.e2e_chunk, a.e2e_calls)
    sim.close()

    fp64 = None
    if not a.no_fp64 and prec != tg.FP64:
        s64 = wl.make_sim(sc, tg.FP64, 0, device=local)
        i64 = s64.plan_info()
        s64.step(3)
        s64.prepare_steps(a.fp64_steps)
        s64.synchronize()
        ms64 = timed(s64, a.fp64_steps)
        t = ms64 / a.fp64_steps / 1e3
        fp64 = {"value": ns / t, "unit": UNIT, "ms_per_step": ms64 / a.fp64_steps, "steps": a.fp64_steps,
                "mass_updates_per_s": nm / t, "algorithmic_gbs": i64["algorithmic_bytes_per_step"] / t / 1e9,
                "kernel": s64.kernel_info()["kernel"],
                "e2e": e2e(s64, a.e2e_chunk, max(1, a.e2e_calls // 2)),
                "note": "FP64 drop-in (bit-identical to the CPU oracle); FP64-ALU bound on GB300"}
        s64.close()

    ref_gpu = None
    if rank == 0 and world == 1 and a.ref_gpu_steps > 0:
        ref_gpu = reference_kernels(sc, a.ref_gpu_steps, local, value, fp64)

    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, secs = cpu_oracle_rate(sc, a.cpu_steps, threads)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{a.cpu_steps} full steps of the same 100^3 lattice, FP64, OpenMP with atomics "
                         f"({secs:.1f} s wall)"}

    if rank != 0:
        return None
    res = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms_max / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": a.precision, "data": "synthetic (seeded actuated lattice on a frictional plane)",
        "config": workload_config(a.side, nm, ns, world),
        "engine": {"precision": a.precision, "tiles": info["tiles"], "kernel": kinfo["kernel"], "ctas": kinfo["ctas"],
                   "threads_per_cta": kinfo["threads"], "smem_bytes": kinfo["smem_bytes"],
                   "graphs": "built before the timed region (prepare_steps)"},
        "mass_updates_per_s": nm * a.steps * world / (ms_max / 1e3),
        "hbm_algorithmic_gbs": achieved,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_kind": peak_kind, "algorithmic_bytes_per_launch": alg,
                     "implementation_bytes_per_launch": info["implementation_bytes_per_step"],
                     "kernel": KERNEL_NAMES.get(kinfo["kernel"], kinfo["kernel"])
                     + " (fused spring forces + mass update, one launch per step)"},
        "e2e": e2e_main,
        "gpu_launches": a.steps,
        "clocks": clk.summary(),
        "finite": finite,
        "native_libraries": mapped_repo_libraries(),
    }
    if fp64:
        res["fp64"] = fp64
    if ref_gpu:
        res["reference_kernels"] = ref_gpu
    if cpu:
        res["cpu_baseline"] = cpu
    return res


def run_reference(a, rank, world):
    """The reference arm: the reference's per-spring / per-mass functions
    restated on the host (the oracle port, OpenMP, FP64 atomics as the
    reference's kernels use), on all host threads, on the same workload.  The
    scene is built with the oracle's own lattice builder, so no library of
    the engine is loaded into this process."""
    if rank != 0:
        return None
    from oracle import pyoracle as po
    from titan_gb300 import workloads as wl
    sc = wl.actuated_lattice(a.side, lattice_fn=po.lattice)
    ns, nm = sc["left"].size, sc["pos"].shape[0]
    threads = os.cpu_count() or 1
    o = po.OracleSim(sc)
    o.step(min(a.warmup, 3), po.ATOMIC_OMP, threads)
    k = max(1, min(a.steps, 60))
    t0 = time.perf_counter()
    o.step(k, po.ATOMIC_OMP, threads)
    dt = time.perf_counter() - t0
    val = ns * k / dt
    return {"metric": METRIC, "value": val, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": dt / k * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded actuated lattice on a frictional plane)",
            "config": workload_config(a.side, nm, ns, world),
            "impl": "reference",
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{k} of the {a.steps} requested full steps (each the whole lattice), "
                                       "reference per-spring/per-mass functions restated in C, OpenMP atomics"},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "native_libraries": mapped_repo_libraries()}


def _event_ms(sim, steps, local):
    import torch
    stream = torch.cuda.ExternalStream(sim.stream, device=local)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    sim.step(steps)
    e1.record(stream)
    sim.synchronize()
    return e0.elapsed_time(e1)


def run_suite(a, local):
    """Rows of the baseline table: each workload timed with the engine (FP64
    and FP32C, automatic kernel), the reference's own CUDA kernels on the same
    GPU (back to back and with execute()'s per-step synchronisation) and the
    CPU port of the reference on all host cores.  Every value is
    spring-updates/s over a bounded sample of the workload's steps."""
    import torch

    import titan_gb300 as tg
    from oracle import pyoracle as po
    from oracle import refgpu
    from titan_gb300 import workloads as wl

    torch.cuda.set_device(local)
    threads = os.cpu_count() or 1
    rows = [
        ("5^3 lattice, contact + friction (config 1 contact variant)", wl.falling_cube(contact=True), 10000, 2000,
         5000, 2000),
        ("100^3 lattice, 20% actuated, plane + ball (config 2)", wl.actuated_lattice(), 1000, 200, 50, 4),
        ("4096 bodies, 3-12 masses per side, own planes (config 3)", wl.robot_batch(nbodies=4096), 5000, 200, 20, 4),
    ]
    for name, sc, steps, eng_steps, ref_steps, cpu_steps in rows:
        ns, nm = sc["left"].size, sc["pos"].shape[0]
        out = {"workload": name, "masses": nm, "springs": ns, "steps_of_workload": steps, "unit": UNIT}
        for prec, key in ((tg.FP32C, "engine_f32c"), (tg.FP64, "engine_f64")):
            sim = wl.make_sim(sc, prec, 0, device=local)
            k = eng_steps if prec != tg.FP64 else max(1, eng_steps // 4)
            sim.step(3)
            ms = _event_ms(sim, k, local)
            out[key] = {"value": ns * k / (ms / 1e3), "ms_per_step": ms / k, "steps_timed": k,
                        "kernel": sim.kernel_info()["kernel"]}
            sim.close()
        why = refgpu.available()
        if why:
            out["reference_cuda_kernels"] = {"unavailable": why}
        else:
            rsc = dict(sc)
            note = "reference src/sim.cu kernels, 1024-thread blocks, FP64 atomics"
            if "body_ptr" in sc:  # the reference has no per-body planes: one global plane does the same work
                rsc["planes"] = sc["planes"] + [((0.0, 0.0, 1.0), 0.0, 0.5, 0.5)]
                note += "; per-body planes replaced by one global plane (same per-mass work)"
            r = refgpu.RefGpuSim(rsc, local)
            try:
                r.step(3)
                ms = r.time_steps(ref_steps)
                ms_sync = r.time_steps(ref_steps, sync_each=True)
            finally:
                r.close()
            out["reference_cuda_kernels"] = {"value": ns * ref_steps / (ms / 1e3), "ms_per_step": ms / ref_steps,
                                             "ms_per_step_with_step_sync": ms_sync / ref_steps,
                                             "steps_timed": ref_steps, "note": note}
        o = po.OracleSim(sc)
        t0 = time.perf_counter()
        o.step(cpu_steps, po.ATOMIC_OMP, threads)
        dt = time.perf_counter() - t0
        out["reference_cpu_port"] = {"value": ns * cpu_steps / dt, "ms_per_step": dt / cpu_steps * 1e3,
                                     "steps_timed": cpu_steps, "cores": threads}
        rv = out["reference_cuda_kernels"].get("value")
        if rv:
            out["speedup_f32c_vs_reference_kernels"] = out["engine_f32c"]["value"] / rv
            out["speedup_f64_vs_reference_kernels"] = out["engine_f64"]["value"] / rv
        print(json.dumps(out), flush=True)


def run_precision_study(a, local):
    """Long-horizon precision study: 64^3 lattice dropped on a frictional
    plane, dt = 1e-5, --study-steps steps in FP64, FP32 and FP32C, a
    checkpoint every --study-every steps: each mode's total energy and its
    drift from the start, linear momentum, and FP32 / FP32C position error
    against the FP64 form (the study's oracle, itself pinned to the CPU
    oracle and to the reference's kernels by the tests); beside it, for the
    first --study-ref-steps steps, the reference's own CUDA kernels from the
    same start, whose distance from the FP64 form is the reference's own
    run-to-run spread (float atomics).  One JSON line per checkpoint, then a
    summary line."""
    import numpy as np
    import torch

    import titan_gb300 as tg
    from titan_gb300 import workloads as wl

    torch.cuda.set_device(local)
    sc = wl.settling_lattice()
    n = sc["pos"].shape[0]
    sims = {p: wl.make_sim(sc, p, 0, device=local) for p in (tg.FP64, tg.FP32, tg.FP32C)}
    names = {tg.FP64: "f64", tg.FP32: "f32", tg.FP32C: "f32c"}
    g = float(abs(sc["g"][2]))
    from oracle import refgpu
    ref = None
    if a.study_ref_steps > 0 and refgpu.available() is None:
        ref = refgpu.RefGpuSim(sc, local)
    e0 = {p: float(s.diagnostics(g)["total"]) for p, s in sims.items()}
    rows = []
    done = 0
    t0 = time.perf_counter()
    while done < a.study_steps:
        k = min(a.study_every, a.study_steps - done)
        for s in sims.values():
            s.step(k)
        if ref is not None:
            if done + k <= a.study_ref_steps:
                ref.step(k)
            else:
                ref.close()
                ref = None
        done += k
        st = {p: s.get_state(pos=True, vel=False) for p, s in sims.items()}
        row = {"steps": done, "t": done * sc["dt"]}
        for p, s in sims.items():
            d = s.diagnostics(g)
            row[names[p] + "_energy_j"] = float(d["total"])
            row[names[p] + "_energy_drift_rel"] = (float(d["total"]) - e0[p]) / abs(e0[p])
            row[names[p] + "_momentum"] = [float(x) for x in d["linear"]]
        for p in (tg.FP32, tg.FP32C):
            dd = st[p]["pos"] - st[tg.FP64]["pos"]
            row[names[p] + "_max_pos_err_m"] = float(np.max(np.abs(dd)))
            row[names[p] + "_rms_pos_err_m"] = float(np.sqrt(np.mean(dd * dd)))
        if ref is not None and done <= a.study_ref_steps:
            dr = ref.state()["pos"] - st[tg.FP64]["pos"]
            row["reference_kernels_max_pos_diff_m"] = float(np.max(np.abs(dr)))
            row["reference_kernels_rms_pos_diff_m"] = float(np.sqrt(np.mean(dr * dr)))
        row["wall_s"] = time.perf_counter() - t0
        rows.append(row)
        print(json.dumps(row), flush=True)
    for s in sims.values():
        s.close()
    if ref is not None:
        ref.close()
    print(json.dumps({"study": "64^3 lattice dropped 0.05 m on a frictional plane (mu 0.5), damping 0.1, dt=1e-5",
                      "masses": n, "steps": a.study_steps, "every": a.study_every,
                      "reference_kernel_steps": min(a.study_ref_steps, a.study_steps), "final": rows[-1]}), flush=True)


def run_serving(a, local):
    """Rollout serving.  Rate sweep: requests with Poisson arrivals at each
    rate of --serve-rates, masses log-uniform in [27, --serve-max-masses]
    (cube side = round(cbrt)), horizon U[100, 5000] steps, 120 GB HBM budget
    (the same requests at every rate; only arrival times scale).  Bodies:
    --serve-bodies single-body robots (3-12 masses per side, 5% of springs
    removed, 30% actuated) submitted together for 5000 steps.  Latency runs
    from arrival to the final positions on the host; one JSON line per rate."""
    import torch

    import titan_gb300 as tg
    from titan_gb300 import serving
    from titan_gb300 import workloads as wl

    torch.cuda.set_device(local)
    prec = {"f32c": tg.FP32C, "f64": tg.FP64, "f32": tg.FP32}[a.precision]
    if a.serve_engine == "device":
        srv = serving.DeviceRolloutServer(prec, device=local, stream_masses=a.serve_stream_masses)
        engine = f"device-resident request loop (one persistent kernel, per-tile arithmetic, tiles of {srv.tile} masses)"
        engine += (f" for requests under {a.serve_stream_masses} masses, own stream and automatic kernel above"
                   if a.serve_stream_masses > 0 else " for every request")
    else:
        srv = serving.RolloutServer(prec, device=local, small_masses=a.serve_small_masses)
        engine = "one engine per request on its own CUDA stream"
    if a.serve_bodies:
        rng = np.random.default_rng(11)
        reqs = [{"id": i, "arrival_s": 0.0, "side": int(rng.integers(3, 13)), "steps": 5000, "seed": 7000 + i}
                for i in range(a.serve_bodies)]
        runs = [("bodies", reqs)]
    else:
        runs = [(float(r), wl.request_stream(a.serve_requests, float(r), mass_range=(27, a.serve_max_masses)))
                for r in a.serve_rates.split(",")]
    # scenes built before the clock starts (request payloads arrive ready)
    scenes = {}
    for _, reqs in runs:
        for r in reqs:
            scenes.setdefault((r["side"], r["seed"]), None)
    for key in scenes:
        scenes[key] = wl.rollout_request(*key)
    scene_of = lambda r: scenes[(r["side"], r["seed"])]
    # warm-up: one short request per design, so that the served runs measure
    # steady state (plans and pooled engines exist)
    warm = {}
    for _, reqs in runs:
        for r in reqs:
            warm.setdefault(r["side"], dict(r, arrival_s=0.0, steps=100))
    srv.run(list(warm.values()), scene_of=scene_of)
    prewarmed = 0
    if a.serve_engine == "device" and a.serve_prewarm:
        # as many engines per design as any run has requests of it
        counts = {}
        for _, reqs in runs:
            c = {}
            for r in reqs:
                c[r["side"]] = c.get(r["side"], 0) + 1
            for side, k in c.items():
                counts[side] = max(counts.get(side, 0), k)
        by_side = {}
        for r in warm.values():
            by_side[r["side"]] = scene_of(r)
        before = srv.engines_built
        srv.prewarm(counts, lambda side: by_side[side])
        prewarmed = srv.engines_built - before
    for rate, reqs in runs:
        recs, stats = srv.run(reqs, scene_of=scene_of)
        masses = sum(rec["masses"] for rec in recs.values())
        print(json.dumps({"workload": "rollout serving", "engine": engine, "requests": len(reqs),
                          "rate_per_s": rate, "mean_masses": masses / len(recs), "precision": a.precision,
                          "engines_prebuilt": prewarmed, **stats,
                          "unit": UNIT}), flush=True)
    srv.close()


def main():
    a = parse()
    rank, world, local = dist_env()
    if a.serving:
        if rank == 0:
            run_serving(a, local)
        return
    if a.suite:
        if rank == 0:
            run_suite(a, local)
        return
    if a.precision_study:
        if rank == 0:
            run_precision_study(a, local)
        return
    if a.impl == "reference":
        res = run_reference(a, rank, world)
    else:
        res = run_ours(a, rank, world, local)
    if res is not None:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
