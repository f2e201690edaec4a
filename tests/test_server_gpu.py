"""The device-resident request server (titan_gb300_server_*).

Bar: a request's result (positions, velocities, accelerations, per-mass
time) is bit-identical to the same scene stepped by its own step() on the
per-tile kernel, whether it runs alone on the server or among thousands of
other resident bodies, and whether it was admitted at once or later, as
slots freed up; the FP64 form is also bit-identical to the oracle."""
import numpy as np
import pytest

import titan_gb300 as tg
from oracle import pyoracle as po
from titan_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

KEYS = ("pos", "vel", "acc", "T")


def make(sc, precision, tile=128):
    return wl.make_sim(sc, precision, tile, kernel=1, resident=(0, 0, 0))


def requests():
    """64 batches of 64 small bodies (4096 bodies), a 20^3 lattice cut into
    tiles with halos, and the 5^3 contact lattice, with uneven horizons."""
    out = []
    for b in range(64):
        sc = wl.robot_batch(nbodies=64, seed=100 + b, side_range=(3, 5))
        out.append((sc, 150 + 7 * b))
    out.append((wl.actuated_lattice(20), 400))
    cube = wl.falling_cube(contact=True)
    cube["vel"] = np.random.default_rng(2).normal(scale=0.3, size=cube["pos"].shape)
    out.append((cube, 333))
    return out


def reference(sc, steps, precision):
    s = make(sc, precision)
    s.step(steps)
    st = s.get_state(acc=True, T=True)
    t = s.time
    s.close()
    return st, t


def test_server_results_equal_step_alone_and_in_a_4096_body_mix():
    reqs = requests()
    assert sum(np.diff(sc["body_ptr"]).size for sc, _ in reqs if "body_ptr" in sc) == 4096
    want = [reference(sc, n, tg.FP32C) for sc, n in reqs]
    with tg.Server(tg.FP32C, max_slots=len(reqs)) as srv:
        # alone: the 20^3 lattice and one batch, one at a time
        for i in (64, 3):
            sc, n = reqs[i]
            s = make(sc, tg.FP32C)
            t = srv.submit(s, n)
            srv.wait(t)
            st = s.get_state(acc=True, T=True)
            for k in KEYS:
                assert np.array_equal(st[k], want[i][0][k]), (i, k)
            assert s.time == want[i][1] and s.steps == n
        # the mix: every request at once (4096 bodies resident together)
        sims = [make(sc, tg.FP32C) for sc, _ in reqs]
        tickets = [srv.submit(s, n) for s, (_, n) in zip(sims, reqs)]
        assert srv.info()["busy_slots"] == len(reqs)
        for t in tickets:
            srv.wait(t)
        for i, s in enumerate(sims):
            st = s.get_state(acc=True, T=True)
            for k in KEYS:
                assert np.array_equal(st[k], want[i][0][k]), (i, k)
            assert s.time == want[i][1]
        # a served scene steps on by itself afterwards
        sims[-1].step(10)
        assert sims[-1].steps == reqs[-1][1] + 10


def test_server_admits_as_slots_free_up():
    """Eight slots, 24 requests: the rest are submitted as requests finish,
    while others run; every result equals its own step() run."""
    reqs = [(wl.robot_batch(nbodies=8, seed=300 + i, side_range=(3, 6)), 100 + 31 * i) for i in range(24)]
    want = [reference(sc, n, tg.FP32C) for sc, n in reqs]
    with tg.Server(tg.FP32C, max_slots=8) as srv:
        sims = [make(sc, tg.FP32C) for sc, _ in reqs]
        pending = list(range(len(reqs)))
        running = {}
        while pending or running:
            while pending:
                t = srv.submit(sims[pending[0]], reqs[pending[0]][1])
                if t is None:
                    break
                running[t] = pending.pop(0)
            assert len(running) <= 8
            for t in [t for t in running if srv.poll(t)]:
                i = running.pop(t)
                st = sims[i].get_state(acc=True, T=True)
                for k in KEYS:
                    assert np.array_equal(st[k], want[i][0][k]), (i, k)
        assert srv.info()["busy_slots"] == 0


def test_server_fp64_bitwise_vs_oracle_and_refusals():
    sc = wl.falling_cube(contact=True)
    sc["vel"] = np.random.default_rng(3).normal(scale=0.3, size=sc["pos"].shape)
    with tg.Server(tg.FP64, max_slots=4) as srv:
        s = wl.make_sim(sc, tg.FP64, 32, kernel=1, resident=(0, 0, 0))
        t = srv.submit(s, 1500)
        with pytest.raises(tg.TitanError, match="ESTATE"):
            s.step(1)  # the server holds the scene
        srv.wait(t)
        st = s.get_state(acc=True, T=True)
        o = po.OracleSim(sc)
        o.step(1500)
        for k, v in (("pos", o.pos), ("vel", o.vel), ("acc", o.acc), ("T", o.T)):
            assert np.array_equal(st[k], v), k
        # scenes the server cannot step are refused
        r = wl.make_sim(sc, tg.FP64, 128, resident=(2, 0, 0))  # one halo-free tile, run resident
        assert r.resident_info()["active"] == 2
        with pytest.raises(tg.TitanError, match="EINVAL"):
            srv.submit(r, 10)
        f = wl.make_sim(sc, tg.FP32C, 32, kernel=1, resident=(0, 0, 0))
        with pytest.raises(tg.TitanError, match="EINVAL"):
            srv.submit(f, 10)  # another precision
