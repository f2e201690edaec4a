"""Launch-shape autotuner: times the step of a given scene with each
candidate (kernel form, tile size, threads per CTA) on the current GPU and
caches the fastest per (GPU, precision, scene size).

All candidates compute the same bits (the kernel forms and tile sizes are
bit-identical by construction), so tuning changes speed only.
"""
from __future__ import annotations

import hashlib
import json
import os
import time
from pathlib import Path

from . import FP64, Sim
from . import workloads as wl

# (kernel form, tile masses, threads per CTA); form 6 = pull (threads =
# consumer threads: a team of one warp per 32 tile masses per tile in
# flight; 0 = two teams), 4 = warp-specialised (threads = consumer
# threads), 3 = per-tile with asynchronous staging, 1 = per-tile
CANDIDATES_F32 = [(6, 256, 0), (6, 192, 0), (6, 128, 0), (6, 128, 384), (4, 208, 448), (4, 192, 448),
                  (4, 160, 448), (3, 256, 256), (1, 256, 256), (1, 128, 128)]
CANDIDATES_F64 = [(1, 128, 128), (1, 64, 128), (3, 128, 128), (1, 128, 256)]


def _default_cache() -> Path:
    base = os.environ.get("TITAN_GB300_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "titan_gb300")
    return Path(base) / "autotune.json"


def _gpu_name(device: int) -> str:
    try:
        import torch
        return torch.cuda.get_device_name(device)
    except Exception:
        return "cuda"


def scene_key(sc: dict, precision: int, device: int = 0) -> str:
    n, ns = sc["pos"].shape[0], sc["left"].size
    nb = len(sc["body_ptr"]) - 1 if "body_ptr" in sc else 1
    h = hashlib.sha1(f"{_gpu_name(device)}|{precision}|{n}|{ns}|{nb}".encode()).hexdigest()[:16]
    return h


def _time_candidate(sc, precision, cand, steps, device):
    kern, tile, threads = cand
    s = wl.make_sim(sc, precision, tile, device=device, threads=threads, kernel=kern)
    try:
        s.step(5)
        s.synchronize()
        t0 = time.perf_counter()
        s.step(steps)
        s.synchronize()
        return (time.perf_counter() - t0) / steps * 1e3, s.kernel_info()["kernel"]
    finally:
        s.close()


def autotune(sc: dict, precision: int, steps: int = 60, candidates=None, cache_path=None, device: int = 0,
             refresh: bool = False) -> dict:
    """Fastest launch configuration for scene sc; cached on disk."""
    cache = Path(cache_path) if cache_path else _default_cache()
    key = scene_key(sc, precision, device)
    table = {}
    if cache.exists():
        try:
            table = json.loads(cache.read_text())
        except ValueError:
            table = {}
    if key in table and not refresh:
        return table[key]
    cands = candidates or (CANDIDATES_F64 if precision == FP64 else CANDIDATES_F32)
    results = []
    for cand in cands:
        try:
            ms, form = _time_candidate(sc, precision, cand, steps, device)
        except Exception as ex:  # a candidate that does not fit this scene
            results.append({"candidate": list(cand), "error": str(ex)})
            continue
        results.append({"candidate": list(cand), "ms_per_step": ms, "form": form})
    ok = [r for r in results if "ms_per_step" in r]
    if not ok:
        raise RuntimeError("no launch configuration ran: " + "; ".join(r.get("error", "") for r in results))
    best = min(ok, key=lambda r: r["ms_per_step"])
    kern, tile, threads = best["candidate"]
    entry = {"kernel": kern, "tile": tile, "threads": threads, "ms_per_step": best["ms_per_step"],
             "form": best["form"], "tried": results}
    table[key] = entry
    cache.parent.mkdir(parents=True, exist_ok=True)
    cache.write_text(json.dumps(table, indent=1))
    return entry


def make_tuned_sim(sc: dict, precision: int, device: int = 0, **kw) -> Sim:
    cfg = autotune(sc, precision, device=device, **kw)
    return wl.make_sim(sc, precision, cfg["tile"], device=device, threads=cfg["threads"], kernel=cfg["kernel"])
