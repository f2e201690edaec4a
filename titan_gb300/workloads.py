"""Synthetic scenes for the measured configurations (no datasets involved).

A scene is a plain dict of numpy arrays in creation order:
    pos (n,3) vel (n,3) m (n) [ext (n,3)] [fixed (n)] [drag (n)]
    left right k rest damping type omega amp phase  (per spring)
    planes: list of (normal, offset, friction_k, friction_s)
    balls:  list of (center, radius)
    g (3,), dt, [body_ptr (nb+1)], [body_planes: list of (normal, offset, fk, fs)]

Geometry follows Titan's createLattice (src/object.cu:232-293): masses in i,j,k
order, 13 forward springs of the 26-neighbourhood per mass, rest = initial
length.  Where the measured configurations leave a value open, the value
chosen here is written beside it.
"""
from __future__ import annotations

import math

import numpy as np

from . import FP64, Sim, lattice

TWO_PI = 2.0 * math.pi


def empty_scene(dt=1e-4, g=(0.0, 0.0, -9.81)):
    return {"planes": [], "balls": [], "g": np.array(g, float), "dt": float(dt)}


def lattice_scene(center, dims, nx, ny, nz, m=0.1, k=1e4, damping=0.0, dt=1e-4, g=(0.0, 0.0, -9.81),
                  lattice_fn=None):
    """lattice_fn(center, dims, nx, ny, nz) -> (pos, left, right, rest): the
    geometry builder (default: the engine's titan_gb300.lattice; any builder
    that reproduces createLattice gives the same scene)."""
    pos, left, right, rest = (lattice_fn or lattice)(center, dims, nx, ny, nz)
    n, ns = pos.shape[0], left.size
    sc = empty_scene(dt, g)
    sc.update(pos=pos, vel=np.zeros_like(pos), m=np.full(n, m), left=left, right=right,
              k=np.full(ns, float(k)), rest=rest, damping=np.full(ns, float(damping)),
              type=np.zeros(ns, np.int32), omega=np.zeros(ns), amp=np.full(ns, 0.2), phase=np.zeros(ns))
    return sc


def falling_cube(contact=False):
    """5x5x5 lattice of 0.1 kg masses spanning 5 m, centre (0,0,10), k=1e4,
    no damping, g=(0,0,-9.81), plane z=0 with friction (mu_k = mu_s = 0.5, the
    friction values are not given by the configuration), dt=1e-4.
    contact=True moves the centre to z=2.6 so the lattice reaches the plane
    within 10^4 steps (at z=10 it never does)."""
    sc = lattice_scene((0.0, 0.0, 2.6 if contact else 10.0), (5.0, 5.0, 5.0), 5, 5, 5)
    sc["planes"].append(((0.0, 0.0, 1.0), 0.0, 0.5, 0.5))
    return sc


def actuate(sc, rng, fraction, amp, period=(0.1, 1.0), kinds=(2, 3)):
    """Sinusoidal rest-length actuation on a random fraction of springs:
    type 2/3 (contract-then-expand / expand-then-contract), amplitude amp,
    phase U[0, 2pi), omega = 2pi / U[period]."""
    ns = sc["left"].size
    act = rng.random(ns) < fraction
    na = int(act.sum())
    sc["type"][act] = rng.choice(np.array(kinds, np.int32), size=na)
    sc["amp"][act] = amp
    sc["phase"][act] = rng.uniform(0.0, TWO_PI, na)
    sc["omega"][act] = TWO_PI / rng.uniform(period[0], period[1], na)
    return sc


def actuated_lattice(n_side=100, seed=20261203, lattice_fn=None):
    """Single large lattice: n_side^3 masses (100^3 = 1,000,000 masses,
    12,731,796 springs), 5 m cube centred at (0,0,2.6) so its bottom face
    starts 0.1 m above the plane, m = 0.1 kg; k log-uniform in [1e3, 1e5],
    damping 0.1; 20% of springs actuated (amplitude 0.1, random phase, period
    U[0.1, 1] s); plane z=0 with friction 0.5; a fixed ball of radius 2 m at
    (0,0,-2.5), below the plane, so every mass evaluates it every step but none
    is pushed by its constant 20 kN force (contact with that ball ejects a
    0.1 kg mass at ~20 m/s per step, which would make precision comparisons
    measure chaos, not arithmetic); dt = 1e-4."""
    rng = np.random.default_rng(seed)
    sc = lattice_scene((0.0, 0.0, 2.6), (5.0, 5.0, 5.0), n_side, n_side, n_side, m=0.1, damping=0.1,
                       lattice_fn=lattice_fn)
    ns = sc["left"].size
    sc["k"] = np.exp(rng.uniform(math.log(1e3), math.log(1e5), ns))
    actuate(sc, rng, 0.2, 0.1)
    sc["planes"].append(((0.0, 0.0, 1.0), 0.0, 0.5, 0.5))
    sc["balls"].append(((0.0, 0.0, -2.5), 2.0))
    return sc


def settling_lattice(n_side=64, seed=7):
    """Long-horizon study scene: n_side^3 lattice (64^3 = 262,144 masses) of
    0.1 kg masses spanning 3 m, dropped from 0.05 m onto a frictional plane
    (mu 0.5), k = 1e4, damping 0.1, dt = 1e-5."""
    sc = lattice_scene((0.0, 0.0, 1.55), (3.0, 3.0, 3.0), n_side, n_side, n_side, m=0.1, damping=0.1, dt=1e-5)
    sc["planes"].append(((0.0, 0.0, 1.0), 0.0, 0.5, 0.5))
    return sc


def body_lattice(side, spacing, center, rng, drop=0.05, act_fraction=0.3, amp=0.1):
    pos, left, right, rest = lattice(center, (spacing * (side - 1),) * 3, side, side, side)
    ns = left.size
    keep = rng.random(ns) >= drop
    left, right, rest = left[keep], right[keep], rest[keep]
    ns = left.size
    k = np.exp(rng.uniform(math.log(1e3), math.log(1e5), ns))
    typ = np.zeros(ns, np.int32)
    ampa = np.full(ns, 0.2)
    ph = np.zeros(ns)
    om = np.zeros(ns)
    act = rng.random(ns) < act_fraction
    na = int(act.sum())
    typ[act] = rng.choice(np.array([2, 3], np.int32), size=na)
    ampa[act] = amp
    ph[act] = rng.uniform(0, TWO_PI, na)
    om[act] = TWO_PI / rng.uniform(0.1, 1.0, na)
    return pos, left, right, rest, k, typ, ampa, ph, om


def robot_batch(nbodies=4096, seed=3, side_range=(3, 12), spacing=0.1, pitch=2.0):
    """Batch of independent soft-body robots: side ~ U{3..12} masses per axis
    (0.1 m spacing, 0.1 kg masses), 5% of springs removed per body, k
    log-uniform in [1e3, 1e5], damping 0.1, 30% actuated (amplitude 0.1,
    random phase, period U[0.1, 1] s); each body has its own ground plane
    z = 0 with friction U[0.3, 0.8]; bodies start 0.05 m above it on a
    2 m grid; dt = 1e-4."""
    rng = np.random.default_rng(seed)
    grid = int(math.ceil(math.sqrt(nbodies)))
    P, L, R, RS, K, TY, AM, PH, OM = ([] for _ in range(9))
    body_ptr = [0]
    body_planes = []
    off = 0
    for b in range(nbodies):
        side = int(rng.integers(side_range[0], side_range[1] + 1))
        cx, cy = (b % grid) * pitch, (b // grid) * pitch
        h = spacing * (side - 1)
        pos, left, right, rest, k, typ, ampa, ph, om = body_lattice(side, spacing, (cx, cy, 0.05 + h / 2), rng)
        P.append(pos)
        L.append(left + off)
        R.append(right + off)
        RS.append(rest)
        K.append(k)
        TY.append(typ)
        AM.append(ampa)
        PH.append(ph)
        OM.append(om)
        off += pos.shape[0]
        body_ptr.append(off)
        mu = float(rng.uniform(0.3, 0.8))
        body_planes.append(((0.0, 0.0, 1.0), 0.0, mu, mu))
    pos = np.concatenate(P)
    ns = sum(x.size for x in L)
    sc = empty_scene(1e-4)
    sc.update(pos=pos, vel=np.zeros_like(pos), m=np.full(pos.shape[0], 0.1), left=np.concatenate(L),
              right=np.concatenate(R), rest=np.concatenate(RS), k=np.concatenate(K),
              damping=np.full(ns, 0.1), type=np.concatenate(TY), amp=np.concatenate(AM),
              phase=np.concatenate(PH), omega=np.concatenate(OM), body_ptr=np.array(body_ptr, np.int64),
              body_planes=body_planes)
    return sc


def load(sim: Sim, sc: dict, start=True, tile_masses=0, threads=0, kernel=0, resident=None, occupancy=0):
    """Upload a scene into a Sim handle (and start it).  resident: None for
    the default, else (mode, bin_masses, threads) for set_resident."""
    sim.set_time_step(sc["dt"])
    sim.set_global_acc(sc["g"])
    if sc.get("integrator", 0):
        sim.set_integrator(sc["integrator"])
    sim.set_masses(sc["pos"], sc["m"], vel=sc.get("vel"), ext=sc.get("ext"), fixed=sc.get("fixed"),
                   drag=sc.get("drag"))
    sim.set_springs(sc["left"], sc["right"], sc["k"], sc["rest"], damping=sc.get("damping"),
                    type=sc.get("type"), omega=sc.get("omega"), amp=sc.get("amp"), phase=sc.get("phase"))
    if "lc_ptr" in sc:
        sim.set_local_constraints(sc["lc_ptr"], sc["lc_type"], sc["lc_vec"], sc["lc_num"])
    for n, off, fk, fs in sc["planes"]:
        sim.add_plane(n, off, fk, fs)
    for c, r in sc["balls"]:
        sim.add_ball(c, r)
    if "body_ptr" in sc:
        sim.set_bodies(sc["body_ptr"])
        for b, (n, off, fk, fs) in enumerate(sc.get("body_planes", [])):
            if n is not None:
                sim.set_body_plane(b, n, off, fk, fs)
    if threads:
        sim.set_launch(threads)
    if kernel:
        sim.set_kernel(kernel)
    if resident is not None:
        sim.set_resident(*resident)
    if occupancy:
        sim.set_occupancy(occupancy)
    if start:
        sim.start(tile_masses)
    return sim


def make_sim(sc: dict, precision=FP64, tile_masses=0, device=0, threads=0, kernel=0, resident=None,
             occupancy=0) -> Sim:
    return load(Sim(precision, device), sc, True, tile_masses, threads, kernel, resident, occupancy)


def robot_design(side, spacing=0.1, design_seed=None):
    """Topology of one soft-robot design of side^3 masses: a lattice with 5% of
    springs removed and 30% of the rest actuated (type 2 or 3), chosen by a
    seed derived from the side, so every rollout of a design shares one tile
    plan.  Returns (pos, left, right, rest, actuated type)."""
    rng = np.random.default_rng(1000003 + side if design_seed is None else design_seed)
    pos, left, right, rest = lattice((0.0, 0.0, 0.05 + spacing * (side - 1) / 2), (spacing * (side - 1),) * 3,
                                     side, side, side)
    keep = rng.random(left.size) >= 0.05
    left, right, rest = left[keep], right[keep], rest[keep]
    typ = np.zeros(left.size, np.int32)
    act = rng.random(left.size) < 0.3
    typ[act] = rng.choice(np.array([2, 3], np.int32), size=int(act.sum()))
    return pos, left, right, rest, typ


_DESIGNS = {}


def rollout_request(side, seed, dt=1e-4):
    """One rollout request on design `side`: per-request spring constants
    (log-uniform [1e3, 1e5]), actuation (amplitude 0.1, random phase, period
    U[0.1, 1] s), initial velocity jitter; ground plane z = 0, friction 0.5,
    damping 0.1."""
    if side not in _DESIGNS:
        _DESIGNS[side] = robot_design(side)
    pos, left, right, rest, typ = _DESIGNS[side]
    rng = np.random.default_rng(seed)
    ns = left.size
    act = typ >= 2
    na = int(act.sum())
    amp = np.full(ns, 0.2)
    ph = np.zeros(ns)
    om = np.zeros(ns)
    amp[act] = 0.1
    ph[act] = rng.uniform(0, TWO_PI, na)
    om[act] = TWO_PI / rng.uniform(0.1, 1.0, na)
    sc = empty_scene(dt)
    sc.update(pos=pos.copy(), vel=rng.normal(scale=0.01, size=pos.shape), m=np.full(pos.shape[0], 0.1), left=left,
              right=right, rest=rest, k=np.exp(rng.uniform(math.log(1e3), math.log(1e5), ns)),
              damping=np.full(ns, 0.1), type=typ, omega=om, amp=amp, phase=ph)
    sc["planes"].append(((0.0, 0.0, 1.0), 0.0, 0.5, 0.5))
    return sc


def request_stream(nreq, rate, seed=5, mass_range=(27, 200000), horizon=(100, 5000)):
    """Serving workload: nreq rollout requests with Poisson arrivals at `rate`
    per second, masses log-uniform in mass_range (cube side =
    round(cbrt(masses))), horizon U[horizon] steps.  Returns a list of dicts
    (id, arrival_s, side, steps, seed); scenes are built on demand by
    rollout_request(side, seed)."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, nreq))
    m = np.exp(rng.uniform(math.log(mass_range[0]), math.log(mass_range[1]), nreq))
    sides = np.maximum(2, np.round(np.cbrt(m))).astype(int)
    steps = rng.integers(horizon[0], horizon[1] + 1, nreq)
    return [{"id": i, "arrival_s": float(t[i]), "side": int(sides[i]), "steps": int(steps[i]),
             "seed": int(seed * 1000003 + i)} for i in range(nreq)]
