"""VERLET and RK2 integrators (the reference's -DVERLET / -DRK2 builds of
massForcesAndUpdate, src/sim.cu:1141-1159, with RK2's two force evaluations
per step, src/sim.cu:1572-1583).

Bar: FP64 bit-identical to the oracle's ascending order (passive springs,
contact with friction, ball, damping) in every kernel form, including a
switch of integrator between steps; FP32C within 1e-6 m of FP64 over 5000
free-flight steps; all FP32C kernel forms bit-identical."""
import numpy as np
import pytest

import titan_gb300 as tg
from oracle import pyoracle as po
from titan_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def contact_scene():
    rng = np.random.default_rng(21)
    sc = wl.lattice_scene((0, 0, 0.55), (1.0, 0.8, 0.9), 9, 7, 8, k=2e3, damping=0.2)
    sc["vel"] = rng.normal(scale=0.5, size=sc["pos"].shape)
    sc["planes"].append(((0.0, 0.1, 1.0), 0.0, 0.4, 0.6))
    sc["balls"].append(((0.3, 0.0, -0.1), 0.35))
    return sc


@pytest.mark.parametrize("integ", [tg.VERLET, tg.RK2])
@pytest.mark.parametrize("kernel", [1, 3, 4])
def test_fp64_bitwise_vs_oracle(integ, kernel):
    sc = dict(contact_scene(), integrator=integ)
    s = wl.make_sim(sc, tg.FP64, 64, kernel=kernel)
    for c in (1, 63, 64, 372):
        s.step(c)
    st = s.get_state(acc=True, T=True)
    o = po.OracleSim(sc)
    o.step(500)
    for k, v in (("pos", o.pos), ("vel", o.vel), ("acc", o.acc), ("T", o.T)):
        assert np.array_equal(st[k], v), (k, np.max(np.abs(st[k] - v)))
    assert s.time == o.time


def test_switch_integrator_between_steps_bitwise():
    sc = contact_scene()
    s = wl.make_sim(sc, tg.FP64, 64)
    o = po.OracleSim(sc)
    for integ, n in ((tg.EULER, 120), (tg.RK2, 77), (tg.VERLET, 130), (tg.EULER, 50)):
        s.set_integrator(integ)
        s.step(n)
        o.s.integrator = integ
        o.step(n)
    st = s.get_state(acc=True, T=True)
    for k, v in (("pos", o.pos), ("vel", o.vel), ("T", o.T)):
        assert np.array_equal(st[k], v), k
    assert s.time == o.time


@pytest.mark.parametrize("integ", [tg.VERLET, tg.RK2])
def test_fp32c_free_flight_error_and_forms(integ):
    rng = np.random.default_rng(22)
    sc = wl.lattice_scene((0, 0, 5.0), (1, 1, 1), 8, 8, 8, k=3e3, damping=0.05)
    wl.actuate(sc, rng, 0.3, 0.1)
    sc["vel"] = rng.normal(scale=0.1, size=sc["pos"].shape)
    sc["integrator"] = integ
    ref = wl.make_sim(sc, tg.FP64)
    ref.step(5000)
    want = ref.get_state()["pos"]
    got = {}
    for kernel in (1, 3, 4, 6):
        s = wl.make_sim(sc, tg.FP32C, 0, kernel=kernel)
        s.step(5000)
        got[kernel] = s.get_state(acc=True)
    assert np.max(np.abs(got[1]["pos"] - want)) < 1e-6
    for kernel in (3, 4, 6):
        for k in ("pos", "vel", "acc"):
            assert np.array_equal(got[1][k], got[kernel][k]), (kernel, k)
