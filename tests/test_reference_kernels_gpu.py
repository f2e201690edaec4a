"""The engine against the reference's own CUDA kernels (src/sim.cu
computeSpringForces / massForcesAndUpdate compiled from the reference
sources, run by oracle/ref_gpu_harness.cpp exactly as execute() launches
them).

Bar: FP64 per step within 1e-9 relative (positions against the scene's
extent, velocities and accelerations against their largest magnitude).  The
reference's float atomics add each mass's spring forces in a scheduling-
dependent order and its kernels are compiled with FMA contraction, so its
own results move in the last bits from run to run; the engine's FP64 form is
the oracle's ascending order without contraction."""
import numpy as np
import pytest

import titan_gb300 as tg
from oracle import refgpu
from titan_gb300 import workloads as wl

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(refgpu.available() is not None, reason=str(refgpu.available()))]


def reference_actuation(sc):
    """The reference's actuation: amplitude 0.2, no phase."""
    if "amp" in sc:
        sc["amp"] = np.full(sc["left"].size, 0.2)
        sc["phase"] = np.zeros(sc["left"].size)
    return sc


def rel(a, b, scale):
    return float(np.max(np.abs(a - b)) / scale)


def compare(sc, nsteps, bound):
    r = refgpu.RefGpuSim(sc)
    try:
        r.step(nsteps)
        ref = r.state()
        T = r.time
    finally:
        r.close()
    s = wl.make_sim(sc, tg.FP64)
    s.step(nsteps)
    st = s.get_state(acc=True, T=True)
    ext = np.max(np.ptp(sc["pos"], axis=0))
    errs = {"pos": rel(st["pos"], ref["pos"], ext),
            "vel": rel(st["vel"], ref["vel"], max(np.max(np.abs(ref["vel"])), 1e-30)),
            "acc": rel(st["acc"], ref["acc"], max(np.max(np.abs(ref["acc"])), 1e-30))}
    assert max(errs.values()) <= bound, errs
    assert np.array_equal(st["T"], ref["T"])
    assert s.time == T
    return errs


def test_contact_friction_lattice_per_step():
    sc = wl.falling_cube(contact=True)
    sc["vel"] = np.random.default_rng(1).normal(scale=0.3, size=sc["pos"].shape)
    compare(sc, 1, 1e-9)


def test_actuated_damped_lattice_ball_fixed_ext_per_step():
    rng = np.random.default_rng(7)
    sc = wl.lattice_scene((0, 0, 0.55), (1.0, 0.8, 0.9), 9, 7, 8, k=2e3, damping=0.2)
    wl.actuate(sc, rng, 0.3, 0.2)
    reference_actuation(sc)
    n = sc["pos"].shape[0]
    sc["vel"] = rng.normal(scale=0.5, size=(n, 3))
    sc["fixed"] = (rng.random(n) < 0.05).astype(np.uint8)
    sc["ext"] = rng.normal(scale=0.2, size=(n, 3))
    sc["planes"].append(((0.0, 0.1, 1.0), 0.0, 0.4, 0.6))
    sc["balls"].append(((0.3, 0.0, -0.1), 0.35))
    compare(sc, 1, 1e-9)


def test_free_flight_1000_steps():
    """No contact (no chaos): the per-step bar holds over 1000 steps."""
    rng = np.random.default_rng(8)
    sc = wl.lattice_scene((0, 0, 5.0), (1, 1, 1), 6, 6, 6, k=3e3, damping=0.05)
    wl.actuate(sc, rng, 0.3, 0.2)
    reference_actuation(sc)
    sc["vel"] = rng.normal(scale=0.1, size=sc["pos"].shape)
    compare(sc, 1000, 1e-9)


def test_full_size_single_lattice_three_steps():
    """100^3 lattice (1,000,000 masses, 12,731,796 springs), plane and ball,
    20% actuated at the reference's amplitude."""
    sc = reference_actuation(wl.actuated_lattice())
    compare(sc, 3, 1e-9)
