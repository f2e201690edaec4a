"""Rollout serving (titan_gb300/serving.py): a request's result does not
depend on what else is being served (bit-identical to running it alone),
pooled engines are reused correctly, and admission respects the HBM
budget."""
import numpy as np
import pytest

import titan_gb300 as tg
from titan_gb300 import serving
from titan_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def alone(side, seed, steps, precision):
    s = wl.make_sim(wl.rollout_request(side, seed), precision)
    s.step(steps)
    pos = s.get_state(pos=True, vel=False)["pos"]
    s.close()
    return pos


@pytest.mark.parametrize("precision", [tg.FP32C, tg.FP64])
def test_results_same_alone_and_in_mix(precision):
    reqs = [{"id": i, "arrival_s": 0.0, "side": side, "steps": steps, "seed": 7000 + i}
            for i, (side, steps) in enumerate([(4, 150), (6, 90), (4, 301), (3, 64), (8, 120), (4, 77), (6, 200),
                                               (5, 128), (4, 33), (3, 250), (6, 65), (7, 99)])]
    srv = serving.RolloutServer(precision, max_active=3, pool_per_design=4)
    recs, stats = srv.run(reqs, keep_results=True)
    srv.close()
    assert stats["requests"] == len(reqs)
    assert stats["engines_built"] < len(reqs)  # pooled engines were reused
    for r in reqs:
        got = recs[r["id"]]["pos"]
        want = alone(r["side"], r["seed"], r["steps"], precision)
        assert np.array_equal(got, want), r


def test_admission_by_budget_serialises():
    reqs = [{"id": i, "arrival_s": 0.0, "side": 4 + i % 3, "steps": 200, "seed": 11 + i} for i in range(6)]
    srv = serving.RolloutServer(tg.FP32C, hbm_budget_bytes=1.0)  # every request alone
    recs, stats = srv.run(reqs)
    srv.close()
    spans = sorted((rec["start_s"], rec["done_s"]) for rec in recs.values())
    for (s0, d0), (s1, _) in zip(spans, spans[1:]):
        assert s1 >= d0 - 1e-9
    assert stats["p50_ms"] <= stats["p99_ms"]


def test_poisson_arrivals_complete():
    reqs = wl.request_stream(40, rate=400.0, mass_range=(27, 3000), horizon=(100, 400))
    srv = serving.RolloutServer(tg.FP32C)
    recs, stats = srv.run(reqs)
    srv.close()
    assert stats["requests"] == 40
    assert all(rec["latency_ms"] > 0 for rec in recs.values())


def test_small_designs_run_as_one_resident_tile():
    """A design that fits one CTA's shared memory is served as one
    halo-free tile (resident-tile launches); a larger one on the per-step
    kernels; results as when run alone."""
    reqs = [{"id": 0, "arrival_s": 0.0, "side": 7, "steps": 120, "seed": 5},
            {"id": 1, "arrival_s": 0.0, "side": 12, "steps": 60, "seed": 6}]
    srv = serving.RolloutServer(tg.FP32C)
    recs, _ = srv.run(reqs, keep_results=True)
    (e7,), (e12,) = srv.pool[7], srv.pool[12]
    assert e7.resident_info()["active"] == 2 and e7.plan_info()["tiles"] == 1
    assert e12.resident_info()["active"] == 0
    for r in reqs:
        assert np.array_equal(recs[r["id"]]["pos"], alone(r["side"], r["seed"], r["steps"], tg.FP32C))
    srv.close()


@pytest.mark.parametrize("precision", [tg.FP32C, tg.FP64])
def test_device_server_result_is_the_same_alone_and_in_a_mix(precision):
    """The same through the device-resident request loop (its default tiles:
    208 masses in FP32C, 128 in FP64): every request of a Poisson stream
    (designs of 27 to 1000 masses, horizons 100 to 600 steps) gives the bits
    it gives alone, and the bits of its own step() with other tiles."""
    reqs = wl.request_stream(24, 400.0, seed=8, mass_range=(27, 1000), horizon=(100, 600))
    with serving.DeviceRolloutServer(precision) as srv:
        alone = {}
        for r in reqs[:5]:
            recs, _ = srv.run([dict(r, arrival_s=0.0)], keep_results=True)
            alone[r["id"]] = recs[r["id"]]["pos"]
        recs, stats = srv.run(reqs, keep_results=True)
    assert stats["requests"] == len(reqs) and stats["max_concurrent"] > 1
    for rid, pos in alone.items():
        assert np.array_equal(recs[rid]["pos"], pos), rid
    for r in reqs:
        s = wl.make_sim(wl.rollout_request(r["side"], r["seed"]), precision, 96, kernel=1, resident=(0, 0, 0))
        s.step(r["steps"])
        assert np.array_equal(recs[r["id"]]["pos"], s.get_state(pos=True, vel=False)["pos"]), r["id"]
        s.close()
