"""Rollout serving over the engine: many independent scenes (requests) on
one GPU, each rolled out for its own number of steps and returned to the host.

Design (GB300-first, no reference counterpart -- the reference runs one scene
per process):
  * every active request runs on its own engine handle and CUDA stream, so
    the GPU executes the steps of all active requests concurrently (kernels
    from different streams overlap); step() is asynchronous and completion is
    detected with poll(), so one host thread keeps many rollouts in flight;
  * admission control: a request starts only while the device bytes of all
    active requests stay within the HBM budget (default 120 GB), and at most
    max_active run at once; the rest wait in arrival order;
  * engines are pooled per design (identical topology): a finished engine is
    reused for the next request of its design by uploading that request's
    state, spring parameters and clock (no reallocation, no replanning, the
    CUDA graphs stay cached), and the first engine of a design takes its
    plan from a host-planned template (adopt_plan);
  * a new design is planned on a host thread (the planner is native code
    and runs without the interpreter lock), so rollouts of planned designs
    keep being admitted and polled meanwhile; among arrived requests, those
    whose design is planned start in arrival order;
  * a design small enough for one CTA's shared memory runs as one tile of
    its own size: a halo-free tile, stepped for the whole rollout by one
    resident-tile launch (one CTA, no per-step launches);
  * a request's result is the same bits whether it runs alone or among
    others: its engine's arithmetic depends only on its own scene.
"""
from __future__ import annotations

import collections
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import FP32, FP32C, FP64, Server, Sim
from . import workloads as wl

_SMEM_PER_CTA = 227 * 1024


def resident_tile_fits(precision, masses, springs):
    """Whether a body of this size fits one resident tile: launch parameters,
    two state records per mass and a force slot per spring (plus the zero
    slot) in one CTA's shared memory."""
    rec = 32 if precision == FP32 else 48
    slot = 32 if precision == FP64 else 16
    return 2016 + 2 * masses * rec + (springs + 1) * slot + 64 <= _SMEM_PER_CTA and masses <= 2048


class RolloutServer:
    def __init__(self, precision=FP32C, device=0, hbm_budget_bytes=120e9, max_active=256, pool_per_design=64,
                 small_masses=50000, resident_tiles=True):
        """Designs that fit one CTA's shared memory run as one resident tile;
        small_masses: larger scenes below this size run the per-tile kernel
        with 128-mass tiles (a few CTAs per SM, so that many small rollouts
        share the SMs); larger ones the automatic kernel (one persistent CTA
        per SM).  0 disables the split.  resident_tiles=False keeps every
        design on the per-step kernels."""
        self.precision = precision
        self.resident_tiles = resident_tiles
        self.small_masses = small_masses
        self.device = device
        self.budget = float(hbm_budget_bytes)
        self.max_active = max_active
        self.pool_per_design = pool_per_design
        self.templates = {}                          # side -> planned host-only Sim
        self.planning = {}                           # side -> (host-only Sim, Future of its plan)
        self._planner = None                         # host threads for planning, during run()
        self.pool = collections.defaultdict(list)    # side -> idle started engines
        self.bytes_of = {}                           # side -> device bytes of one engine
        self.used = 0.0
        self.engines_built = 0

    # -- engines ---------------------------------------------------------
    def _estimate(self, side, sc):
        if side in self.bytes_of:
            return self.bytes_of[side]
        n, ns = sc["pos"].shape[0], sc["left"].size
        return 400.0 * n + 96.0 * ns + (8 << 20)

    def _choice(self, n, ns):
        """(kernel, tile) for a design of n masses and ns springs."""
        if self.resident_tiles and resident_tile_fits(self.precision, n, ns):
            return 0, max(32, n)  # one halo-free tile: a resident-tile launch per rollout
        if n < self.small_masses:
            return 1, 128
        return 0, 0

    def _template(self, side, sc):
        """A host-only handle of design `side`, loaded (not yet planned)."""
        kernel, _ = self._choice(sc["pos"].shape[0], sc["left"].size)
        t = Sim(self.precision, self.device)
        wl.load(t, sc, start=False, kernel=kernel)
        return t

    def _plan_async(self, side, sc):
        """Start planning design `side` on a host thread (once)."""
        if side in self.templates or side in self.planning:
            return
        t = self._template(side, sc)
        _, tile = self._choice(sc["pos"].shape[0], sc["left"].size)
        if self._planner is None:
            self._planner = ThreadPoolExecutor(max_workers=2, thread_name_prefix="titan-plan")
        self.planning[side] = (t, self._planner.submit(t.plan_host, tile))

    def _collect_plans(self):
        """Move finished plans to the templates; a planning error is raised
        here.  Returns whether one finished."""
        done = [side for side, (_, f) in self.planning.items() if f.done()]
        for side in done:
            t, f = self.planning.pop(side)
            try:
                f.result()
            except BaseException:
                t.close()
                raise
            self.templates[side] = t
        return bool(done)

    def _planned(self, side):
        return side in self.templates or bool(self.pool[side])

    def _engine(self, side, sc):
        """An engine loaded with scene sc, ready at time 0 (planning the
        design here if no template exists yet)."""
        if self.pool[side]:
            e = self.pool[side].pop()
            n = e.n
            e.set_mass_state(None, pos=sc["pos"], vel=sc["vel"], T=np.zeros(n))
            e.set_spring_params(None, k=sc["k"], rest=sc["rest"], damping=sc["damping"], type=sc["type"],
                                omega=sc["omega"], amp=sc["amp"], phase=sc["phase"])
            e.set_time(0.0)
            return e
        kernel, tile = self._choice(sc["pos"].shape[0], sc["left"].size)
        if side not in self.templates:
            t = self._template(side, sc)
            t.plan_host(tile)
            self.templates[side] = t
        e = Sim(self.precision, self.device)
        wl.load(e, sc, start=False, kernel=kernel)
        e.adopt_plan(self.templates[side])
        e.start(tile)
        self.engines_built += 1
        if side not in self.bytes_of:
            self.bytes_of[side] = float(e.device_bytes())
        return e

    def _launch(self, e, steps):
        e.step(steps)

    def _done(self, e):
        return e.poll()

    def _release(self, side, e):
        if len(self.pool[side]) < self.pool_per_design:
            self.pool[side].append(e)
        else:
            e.close()

    # -- serving loop ----------------------------------------------------
    def run(self, requests, scene_of=None, keep_results=False, time_scale=1.0):
        """Serve requests (dicts with id, arrival_s, side, steps, seed) with
        arrivals replayed in wall-clock time (arrival_s * time_scale).
        Returns per-request records and summary statistics."""
        scene_of = scene_of or (lambda r: wl.rollout_request(r["side"], r["seed"]))
        pending = collections.deque(sorted(requests, key=lambda r: r["arrival_s"]))
        scenes = {}  # id -> scene, built once per arrived request
        active = []
        records = {}
        springs_done = 0
        max_active = 0
        host = {"engine_s": 0.0, "launch_s": 0.0, "collect_s": 0.0}  # host time in each part of the loop
        self._host = host
        t0 = time.perf_counter()
        try:
            while pending or active:
                now = time.perf_counter() - t0
                # plans of new designs finish on host threads
                progressed = self._collect_plans()
                idx = 0
                while idx < len(pending) and len(active) < self.max_active:
                    r = pending[idx]
                    if r["arrival_s"] * time_scale > now:
                        break
                    if r["id"] not in scenes:
                        scenes[r["id"]] = scene_of(r)
                    sc = scenes[r["id"]]
                    if not self._planned(r["side"]):
                        self._plan_async(r["side"], sc)  # admitted once its design is planned
                        idx += 1
                        continue
                    need = self._estimate(r["side"], sc)
                    if active and self.used + need > self.budget:
                        break  # admission by HBM budget: wait for a rollout to finish
                    del pending[idx]
                    del scenes[r["id"]]
                    th = time.perf_counter()
                    e = self._engine(r["side"], sc)
                    tl = time.perf_counter()
                    self._launch(e, r["steps"])
                    host["engine_s"] += tl - th
                    host["launch_s"] += time.perf_counter() - tl
                    self.used += need
                    active.append((r, e, need, time.perf_counter() - t0, sc["left"].size))
                    max_active = max(max_active, len(active))
                    progressed = True
                tc = time.perf_counter()
                finished, springs = self._poll(active, records, keep_results, t0, time_scale)
                host["collect_s"] += time.perf_counter() - tc
                springs_done += springs
                if not (progressed or finished):
                    time.sleep(50e-6)
        finally:
            if self._planner is not None:
                self._planner.shutdown(wait=True)
                self._planner = None
            self._collect_finished_quietly()
        wall = time.perf_counter() - t0
        lat = np.array([rec["latency_ms"] for rec in records.values()])
        stats = {"requests": len(records), "wall_s": wall, "p50_ms": float(np.percentile(lat, 50)),
                 "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()),
                 "spring_updates_per_s": springs_done / wall, "engines_built": self.engines_built,
                 "max_concurrent": max_active, "host_s": host}
        return records, stats

    def _collect_finished_quietly(self):
        """After run(): keep finished plans as templates, drop failed ones."""
        for side, (t, f) in list(self.planning.items()):
            if f.done() and f.exception() is None:
                self.templates[side] = t
            else:
                t.close()
        self.planning.clear()

    def _poll(self, active, records, keep_results, t0, time_scale):
        """Retire finished rollouts from `active` (in place) into records.
        Returns (whether one finished, their spring updates)."""
        still = []
        finished, springs = False, 0
        for r, e, need, started, ns in active:
            if not self._done(e):
                still.append((r, e, need, started, ns))
                continue
            pos = e.get_state(pos=True, vel=False)["pos"]
            done = time.perf_counter() - t0
            rec = {"id": r["id"], "arrival_s": r["arrival_s"] * time_scale, "start_s": started,
                   "done_s": done, "latency_ms": (done - r["arrival_s"] * time_scale) * 1e3,
                   "steps": r["steps"], "masses": pos.shape[0], "springs": ns}
            if keep_results:
                rec["pos"] = pos
            records[r["id"]] = rec
            springs += ns * r["steps"]
            self.used -= need
            self._release(r["side"], e)
            finished = True
        active[:] = still
        return finished, springs

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def close(self):
        for lst in self.pool.values():
            for e in lst:
                e.close()
        self.pool.clear()
        for t in self.templates.values():
            t.close()
        self.templates.clear()


class DeviceRolloutServer(RolloutServer):
    """The same serving layer (arrival replay, HBM-budget admission, design
    pooling, host-thread planning, latency records) over the device-resident
    request loop (titan_gb300_server_*): a rollout below stream_masses masses
    is not launched on its own stream but submitted to one persistent
    kernel, which admits it at its next step boundary as slots free up,
    steps every active rollout's tiles each step and reports finished ones
    through page-locked memory -- thousands of small rollouts share one
    kernel, with no launch per rollout or step.  Those designs run the
    per-tile arithmetic with tiles of `tile` masses (resident tiles off), so
    results are bit-identical to a rollout's own step() with the per-tile
    kernel, alone or in any mix.  Rollouts of at least stream_masses masses
    (0, the default: none) run on their own engine and stream with the
    automatic kernel, where a large scene steps fastest (measured on GB300,
    100^3 lattice: 0.121 ms per step there against 0.336 ms in the request
    loop) -- but that kernel takes a whole SM's shared memory, so it runs
    only while the request loop's kernel is not resident (it leaves one
    second after its last rollout): mixing the two serialises them."""

    def __init__(self, precision=FP32C, device=0, hbm_budget_bytes=120e9, max_slots=4096, pool_per_design=4096,
                 tile=None, tile_smem_bytes=0, stream_masses=0):
        super().__init__(precision, device, hbm_budget_bytes, max_active=max_slots, pool_per_design=pool_per_design,
                         small_masses=0, resident_tiles=True)
        # tiles of 208 masses fit the loop's default tile memory in FP32 and
        # FP32C (0.305 ms per 100^3 step against 0.331 with 128); FP64
        # records are larger
        self.tile = tile if tile is not None else (128 if precision == FP64 else 208)
        self.stream_masses = stream_masses
        self.server = Server(precision, device, max_slots, tile_smem_bytes)
        self._ticket = {}  # id(engine) -> ticket (request-loop rollouts)

    def _in_loop(self, n):
        return not self.stream_masses or n < self.stream_masses

    def _choice(self, n, ns):
        return (1, self.tile) if self._in_loop(n) else (0, 0)

    def _template(self, side, sc):
        if not self._in_loop(sc["pos"].shape[0]):
            return super()._template(side, sc)
        t = Sim(self.precision, self.device)
        wl.load(t, sc, start=False, kernel=1, resident=(0, 0, 0))
        return t

    def _engine(self, side, sc):
        if self.pool[side] or not self._in_loop(sc["pos"].shape[0]):
            return super()._engine(side, sc)
        if side not in self.templates:
            t = self._template(side, sc)
            t.plan_host(self.tile)
            self.templates[side] = t
        e = Sim(self.precision, self.device)
        wl.load(e, sc, start=False, kernel=1, resident=(0, 0, 0))
        e.adopt_plan(self.templates[side])
        e.start(self.tile)
        self.engines_built += 1
        if side not in self.bytes_of:
            self.bytes_of[side] = float(e.device_bytes())
        return e

    def prewarm(self, counts, scene_of):
        """Build engines ahead of serving: counts maps a design (side) to how
        many engines its pool should hold; scene_of(side) gives a scene of
        that design.  Building an engine costs host time (allocations,
        uploads); a server that knows its designs does it before requests
        arrive."""
        built = []
        for side, k in counts.items():
            sc = scene_of(side)
            while len(self.pool[side]) + sum(1 for s2, _ in built if s2 == side) < k:
                built.append((side, self._engine(side, sc)))
        for side, e in built:
            self.pool[side].append(e)

    def _launch(self, e, steps):
        if not self._in_loop(e.n):
            e.step(steps)
            return
        t = self.server.submit(e, steps)
        if t is None:
            raise RuntimeError("no free server slot (admission allows at most max_slots rollouts)")
        self._ticket[id(e)] = t

    def _done(self, e):
        t = self._ticket.get(id(e))
        if t is None:
            return e.poll()
        if not self.server.poll(t):
            return False
        del self._ticket[id(e)]
        return True

    def close(self):
        super().close()
        self.server.close()
