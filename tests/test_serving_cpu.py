"""Host logic of the rollout server (titan_gb300/serving.py) on the CPU:
admission by the HBM budget and by max_active, engine pooling per design,
complete per-request records, and planning of new designs on host threads.
The engine is a stand-in that finishes a rollout after a fixed number of
polls; the GPU tests cover the real one."""
import time

import numpy as np
import pytest

from titan_gb300 import serving
from titan_gb300 import workloads as wl


class FakeEngine:
    """The calls the server and workloads.load make on an engine handle."""

    live = 0        # engines with a rollout in flight
    max_live = 0
    built = 0

    def __init__(self, precision, device=0):
        self.precision, self.device = precision, device
        self.n = 0
        self.polls_left = 0
        self.started = False
        self.tile = None
        self.kernel = 0

    # scene upload (workloads.load)
    def set_time_step(self, dt): self.dt = dt
    def set_global_acc(self, g): self.g = g
    def set_integrator(self, k): pass
    def set_masses(self, pos, m, **kw): self.n = pos.shape[0]; self.pos = np.array(pos)
    def set_springs(self, left, right, k, rest, **kw): self.ns = len(left)
    def set_local_constraints(self, *a): pass
    def add_plane(self, *a): pass
    def add_ball(self, *a): pass
    def set_bodies(self, *a): pass
    def set_body_plane(self, *a): pass
    def set_launch(self, t): pass
    def set_kernel(self, k): self.kernel = k
    def set_resident(self, *a): pass
    def set_occupancy(self, o): pass

    # planning and start
    def plan_host(self, tile): self.tile = tile
    def adopt_plan(self, src): self.adopted = src
    def start(self, tile=0):
        assert not self.started
        self.started, self.tile = True, tile
        FakeEngine.built += 1
    def device_bytes(self): return 1000 * self.n

    # a rollout: done after steps // 100 + 1 polls
    def step(self, k):
        assert self.started and self.polls_left == 0
        self.polls_left = k // 100 + 1
        FakeEngine.live += 1
        FakeEngine.max_live = max(FakeEngine.max_live, FakeEngine.live)
    def poll(self):
        self.polls_left -= 1
        if self.polls_left <= 0:
            FakeEngine.live -= 1
            return True
        return False
    def get_state(self, pos=True, vel=False):
        return {"pos": self.pos.copy()}

    # reuse from the pool
    def set_mass_state(self, idx, pos=None, vel=None, T=None): self.pos = np.array(pos)
    def set_spring_params(self, idx, **kw): pass
    def set_time(self, t): pass
    def close(self): pass


@pytest.fixture
def fake(monkeypatch):
    monkeypatch.setattr(serving, "Sim", FakeEngine)
    FakeEngine.live = FakeEngine.max_live = FakeEngine.built = 0
    return FakeEngine


def requests(sides, steps=300):
    return [{"id": i, "arrival_s": 0.0, "side": s, "steps": steps, "seed": 100 + i} for i, s in enumerate(sides)]


def test_all_requests_complete_with_their_results(fake):
    reqs = requests([4, 6, 4, 5, 6, 4, 3, 5])
    srv = serving.RolloutServer(hbm_budget_bytes=1e12)
    recs, stats = srv.run(reqs, keep_results=True)
    assert stats["requests"] == len(reqs) and set(recs) == {r["id"] for r in reqs}
    for r in reqs:
        rec = recs[r["id"]]
        sc = wl.rollout_request(r["side"], r["seed"])
        assert rec["masses"] == sc["pos"].shape[0] and rec["springs"] == sc["left"].size
        assert rec["steps"] == r["steps"] and rec["latency_ms"] >= 0 and rec["done_s"] >= rec["start_s"]
        assert np.array_equal(rec["pos"], sc["pos"])  # the stand-in returns the uploaded pose
    assert stats["p50_ms"] <= stats["p99_ms"]


def test_engines_are_pooled_per_design(fake):
    reqs = requests([4] * 6 + [5] * 4)
    srv = serving.RolloutServer(hbm_budget_bytes=1e12, max_active=2, pool_per_design=4)
    _, stats = srv.run(reqs)
    # at most two in flight: each design needs at most two engines
    assert stats["engines_built"] <= 4 and fake.built == stats["engines_built"]
    assert fake.max_live <= 2


def test_admission_respects_the_budget(fake):
    # every side-6 engine reports 216,000 bytes: a budget of 500,000 admits two at a time
    reqs = requests([6] * 7)
    srv = serving.RolloutServer(hbm_budget_bytes=500_000, max_active=64)
    _, stats = srv.run(reqs)
    assert stats["requests"] == 7
    assert fake.max_live == 2


def test_small_designs_are_planned_as_one_tile(fake):
    reqs = requests([3, 7, 12])
    srv = serving.RolloutServer(hbm_budget_bytes=1e12)
    srv.run(reqs)
    tiles = {side: eng[0].tile for side, eng in srv.pool.items()}
    n7 = wl.rollout_request(7, 0)["pos"].shape[0]
    assert tiles[3] == 32 and tiles[7] == n7  # one resident tile each (at least 32 masses)
    assert tiles[12] == 128                    # larger: the per-tile kernel with 128-mass tiles


class SlowPlanEngine(FakeEngine):
    """Planning a design of side 12 takes 0.3 s; side 13 fails to plan."""

    def plan_host(self, tile):
        if self.n == wl.rollout_request(12, 0)["pos"].shape[0]:
            time.sleep(0.3)
        if self.n == wl.rollout_request(13, 0)["pos"].shape[0]:
            raise RuntimeError("plan_host: planning failed")
        super().plan_host(tile)


def test_planning_a_new_design_does_not_hold_up_others(monkeypatch):
    monkeypatch.setattr(serving, "Sim", SlowPlanEngine)
    FakeEngine.live = FakeEngine.max_live = FakeEngine.built = 0
    reqs = [{"id": 0, "arrival_s": 0.0, "side": 12, "steps": 100, "seed": 1}]
    reqs += [{"id": i, "arrival_s": 0.001 * i, "side": 4, "steps": 100, "seed": i} for i in range(1, 6)]
    recs, stats = serving.RolloutServer(hbm_budget_bytes=1e12).run(reqs)
    assert stats["requests"] == 6
    # the side-4 requests arrive later but finish while side 12 is still planning
    assert max(recs[i]["done_s"] for i in range(1, 6)) < recs[0]["start_s"]
    assert recs[0]["start_s"] >= 0.3


def test_a_planning_error_reaches_the_caller(monkeypatch):
    monkeypatch.setattr(serving, "Sim", SlowPlanEngine)
    reqs = [{"id": 0, "arrival_s": 0.0, "side": 13, "steps": 100, "seed": 1},
            {"id": 1, "arrival_s": 0.0, "side": 4, "steps": 100, "seed": 2}]
    srv = serving.RolloutServer(hbm_budget_bytes=1e12)
    with pytest.raises(RuntimeError, match="planning failed"):
        srv.run(reqs)
    assert not srv.planning and 13 not in srv.templates
