"""The CPU oracle, pinned against the reference's own code and its tests.

1. Golden vectors produced by the reference's host-callable functions
   (tests/golden/make_golden.py): Lattice, ContactPlane/Ball/ConstraintPlane/
   Direction applyForce, plane normalisation -- compared bit for bit.
2. Known answers of the discrete dynamics (free fall, springs at rest, ...).
3. The tolerances of the reference's own tests (test/physics/*.cpp).
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import pyoracle as po

GOLD = np.load(Path(__file__).parent / "golden" / "reference_host.npz")


def _lattice_keys():
    return sorted({k.rsplit("_", 1)[0] for k in GOLD.files if k.startswith("lattice_")})


@pytest.mark.parametrize("key", _lattice_keys())
def test_lattice_matches_reference(key):
    dims = tuple(int(x) for x in key.split("_")[1:4])
    pos, left, right, rest = po.lattice(GOLD[key + "_center"], GOLD[key + "_dims"], *dims)
    assert np.array_equal(pos, GOLD[key + "_pos"])
    assert np.array_equal(left, GOLD[key + "_left"])
    assert np.array_equal(right, GOLD[key + "_right"])
    assert np.array_equal(rest, GOLD[key + "_rest"])


@pytest.mark.parametrize("key", _lattice_keys())
def test_product_lattice_matches_reference(key):
    import titan_gb300 as tg
    dims = tuple(int(x) for x in key.split("_")[1:4])
    pos, left, right, rest = tg.lattice(GOLD[key + "_center"], GOLD[key + "_dims"], *dims)
    assert np.array_equal(pos, GOLD[key + "_pos"])
    assert np.array_equal(left, GOLD[key + "_left"])
    assert np.array_equal(right, GOLD[key + "_right"])
    assert np.array_equal(rest, GOLD[key + "_rest"])


def test_lattice_counts():
    L = po.lib()
    assert L.to_lattice_springs(5, 5, 5) == 1036
    assert L.to_lattice_springs(64, 64, 64) == 3298428
    assert L.to_lattice_springs(100, 100, 100) == 12731796


def test_normalize_matches_reference():
    for v, ref in zip(GOLD["norm_in"], GOLD["norm_out"]):
        assert np.array_equal(po.normalize(v), ref)


def _call(fn, *args):
    import ctypes
    conv = []
    for a in args:
        if isinstance(a, np.ndarray):
            conv.append(a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        else:
            conv.append(float(a))
    fn(*conv)


def test_plane_matches_reference():
    L = po.lib()
    for row, ref in zip(GOLD["plane_in"], GOLD["plane_out"]):
        n, off, fk, fs = row[0:3], row[3], row[4], row[5]
        pos, vel, force = row[6:9].copy(), row[9:12].copy(), row[12:15].copy()
        _call(L.to_plane_apply, po.normalize(n), off, fk, fs, pos, vel, force)
        assert np.array_equal(force, ref), (row, force, ref)


def test_ball_matches_reference():
    L = po.lib()
    for row, ref in zip(GOLD["ball_in"], GOLD["ball_out"]):
        c, r, pos, force = row[0:3].copy(), row[3], row[4:7].copy(), row[7:10].copy()
        _call(L.to_ball_apply, c, r, pos, force)
        assert np.array_equal(force, ref)


@pytest.mark.parametrize("name", ["cplane", "dir"])
def test_local_constraints_match_reference(name):
    L = po.lib()
    fn = L.to_constraint_plane_apply if name == "cplane" else L.to_direction_apply
    for row, ref in zip(GOLD[name + "_in"], GOLD[name + "_out"]):
        v, fr, vel, force = po.normalize(row[0:3]), row[3], row[7:10].copy(), row[10:13].copy()
        _call(fn, v, fr, vel, force)
        assert np.array_equal(vel, ref[:3]) and np.array_equal(force, ref[3:])


# ---------------------------------------------------------------- KATs -----
def one_mass(pos=(1.0, 0.0, 1.0), g=(0.0, 0.0, -9.81), dt=1e-4, m=0.1):
    return {"pos": np.array([pos], float), "vel": np.zeros((1, 3)), "m": np.array([m]),
            "left": np.zeros(0, np.int32), "right": np.zeros(0, np.int32), "k": np.zeros(0),
            "rest": np.zeros(0), "planes": [], "balls": [], "g": np.array(g, float), "dt": dt}


def test_free_fall_discrete():
    """Symplectic Euler: v_n = -g n dt, z_n = z0 - g dt^2 n(n+1)/2."""
    n, dt, g = 1000, 1e-4, 9.81
    o = po.OracleSim(one_mass(g=(0, 0, -g), dt=dt))
    o.step(n)
    assert abs(o.vel[0, 2] - (-g * n * dt)) < 1e-12
    assert abs(o.pos[0, 2] - (1.0 - g * dt * dt * n * (n + 1) / 2)) < 1e-12
    assert o.pos[0, 0] == 1.0 and o.pos[0, 1] == 0.0
    assert abs(o.time - n * dt) < 1e-12
    assert abs(o.T[0] - o.time) == 0.0


def test_spring_at_rest_is_exactly_static():
    pos = np.array([[0.0, 0.0, 0.0], [0.3, 0.1, -0.2]])
    rest = np.array([np.sqrt(0.3 ** 2 + 0.1 ** 2 + 0.2 ** 2)])
    sc = {"pos": pos, "vel": np.zeros((2, 3)), "m": np.array([0.1, 0.2]), "left": np.array([0], np.int32),
          "right": np.array([1], np.int32), "k": np.array([1e4]), "rest": rest, "planes": [], "balls": [],
          "g": np.zeros(3), "dt": 1e-4}
    o = po.OracleSim(sc)
    o.step(50)
    assert np.array_equal(o.pos, pos)


def test_hooke_force():
    import ctypes
    L = po.lib()
    pl, pr = np.array([0.0, 0.0, 0.0]), np.array([0.0, 0.0, 1.5])
    z = np.zeros(3)
    out = np.zeros(3)
    D = ctypes.POINTER(ctypes.c_double)
    L.to_spring_force(pl.ctypes.data_as(D), pr.ctypes.data_as(D), z.ctypes.data_as(D), z.ctypes.data_as(D),
                      1000.0, 1.0, 0.0, 0, 0.0, 0.2, 0.0, 0.0, out.ctypes.data_as(D))
    # stretched by 0.5: right mass pulled back toward the left with 500 N
    assert np.allclose(out, [0, 0, -500.0], rtol=0, atol=1e-12)
    # actuated: rest * (1 - 0.2 sin(omega t)) at omega t = pi/2 -> rest 0.8
    L.to_spring_force(pl.ctypes.data_as(D), pr.ctypes.data_as(D), z.ctypes.data_as(D), z.ctypes.data_as(D),
                      1000.0, 1.0, 0.0, 2, np.pi / 2, 0.2, 0.0, 1.0, out.ctypes.data_as(D))
    assert abs(out[2] - (-700.0)) < 1e-9


def test_constraint_plane_keeps_height():
    sc = one_mass()
    sc["lc_ptr"] = np.array([0, 1], np.int64)
    sc["lc_type"] = np.array([0], np.int32)
    sc["lc_vec"] = np.array([[0.0, 0.0, 2.0]])
    sc["lc_num"] = np.array([0.0])
    o = po.OracleSim(sc)
    o.step(100)
    assert o.pos[0, 2] == 1.0


def test_fixed_mass_never_moves():
    sc = one_mass()
    sc["fixed"] = np.array([1], np.uint8)
    o = po.OracleSim(sc)
    o.step(100)
    assert np.array_equal(o.pos, sc["pos"]) and o.T[0] == 0.0


def test_drag_is_truncated_to_int():
    """The device struct stores the drag coefficient as int (object.h:213)."""
    sc = one_mass()
    a = po.OracleSim(dict(sc, drag=np.array([0.9])))
    b = po.OracleSim(sc)
    a.step(200)
    b.step(200)
    assert np.array_equal(a.pos, b.pos)
    c = po.OracleSim(dict(sc, drag=np.array([1.7])))
    c.step(200)
    assert c.vel[0, 2] > b.vel[0, 2]  # drag 1 slows the fall


# ------------------------------------------- reference test tolerances -----
def energy_util(o, plane_z=None):
    """test/testutil/utils.h:12-30 (hard-coded 9.8 for gravity PE).  With
    plane_z, the penalty energy 20000 disp^2 / 2 of masses inside the plane is
    added: the reference's util leaves it out, so a sample taken inside a
    ~7 ms contact under-reads by up to the whole kinetic energy, and the
    reference test passes only when its free-running sampling misses those
    windows."""
    e = o.energy(9.8)[3]
    if plane_z is not None:
        d = np.minimum(o.pos[:, 2] - plane_z, 0.0)
        e += float(np.sum(0.5 * 20000.0 * d * d))
    return e


def test_reference_external_force():
    """test/physics/external_unittest.cpp:17-35: x,y within 1e-6, z within 0.1
    of 1 - 4.9 t^2, sampled every 0.1 s up to 5 s."""
    sc = one_mass(g=(0, 0, 0.0))
    sc["ext"] = np.array([[0.0, 0.0, -9.8 * 0.1]])
    o = po.OracleSim(sc)
    while o.time < 5:
        o.step(1000)
        assert abs(o.pos[0, 0] - 1) < 1e-6 and abs(o.pos[0, 1]) < 1e-6
        assert abs(o.pos[0, 2] - (1 + 0.5 * -9.8 * o.time ** 2)) < 0.1


def test_reference_simple_energy():
    """test/physics/simple_unittest.cpp:15-34: EMA(0.9) of total energy
    within 1% of the initial energy every 0.1 s for 5 s."""
    sc = one_mass(g=(0, 0, -9.8))
    sc["planes"].append(((0.0, 0.0, 1.0), 0.0, 0.0, 0.0))
    o = po.OracleSim(sc)
    e0 = energy_util(o, 0.0)
    avg = e0
    while o.time < 5:
        o.step(1000)
        avg = 0.1 * energy_util(o, 0.0) + 0.9 * avg
        assert abs(avg - e0) <= 0.01 * e0


def test_reference_lattice_energy_small():
    """test/physics/energy_unittest.cpp:14-40 at reduced size for the CPU
    (6^3 lattice for 1 s instead of 20^3 for 5 s; the full case runs on the GPU)."""
    from titan_gb300 import workloads as wl
    sc = wl.lattice_scene((0, 0, 5), (4, 4, 4), 6, 6, 6, k=1000, g=(0, 0, -9.8))
    sc["planes"].append(((0.0, 0.0, 1.0), 0.0, 0.0, 0.0))
    o = po.OracleSim(sc)
    e0 = energy_util(o, 0.0)
    avg = e0
    while o.time < 1:
        o.step(1000)
        avg = 0.3 * energy_util(o, 0.0) + 0.7 * avg
        assert abs(avg - e0) <= 0.01 * e0


# ------------------------------------------------- accumulation orders -----
def test_orders_differ_only_by_rounding():
    """Ascending and descending spring orders are two legal serialisations of
    the reference's atomics: per step they agree to rounding and stay within
    1e-12 m for 1000 free steps.  Once the lattice slides on the frictional
    plane (after ~0.14 s) the static/kinetic friction switch amplifies the
    rounding difference to ~1e-5 m within 0.1 s: that spread is the
    reference's own run-to-run nondeterminism in contact."""
    from titan_gb300 import workloads as wl
    sc = wl.falling_cube(contact=True)
    sc["vel"] = np.random.default_rng(1).normal(scale=0.3, size=sc["pos"].shape)
    a, b = po.OracleSim(sc), po.OracleSim(sc)
    a.step(1, po.ASCENDING)
    b.step(1, po.DESCENDING)
    assert np.max(np.abs(a.pos - b.pos)) <= 1e-15 * np.max(np.abs(a.pos))
    a.step(999, po.ASCENDING)
    b.step(999, po.DESCENDING)
    assert np.max(np.abs(a.pos - b.pos)) < 1e-12
    a.step(1000, po.ASCENDING)
    b.step(1000, po.DESCENDING)
    assert 0 < np.max(np.abs(a.pos - b.pos)) < 1e-3


def test_device_order_is_ascending_without_heavy_masses():
    from titan_gb300 import workloads as wl
    sc = wl.falling_cube(contact=True)
    a, b = po.OracleSim(sc), po.OracleSim(sc)
    a.step(300, po.ASCENDING)
    b.step(300, po.DEVICE, nthreads=2)
    assert np.array_equal(a.pos, b.pos) and np.array_equal(a.vel, b.vel)


def hub_scene(degree=200, seed=5):
    rng = np.random.default_rng(seed)
    n = degree + 1
    pos = np.vstack([[0, 0, 1.0], rng.normal(size=(degree, 3)) + [0, 0, 3.0]])
    left = np.zeros(degree, np.int32)
    right = np.arange(1, n, dtype=np.int32)
    rest = np.linalg.norm(pos[right] - pos[left], axis=1) * rng.uniform(0.9, 1.1, degree)
    return {"pos": pos, "vel": np.zeros((n, 3)), "m": np.full(n, 0.1), "left": left, "right": right,
            "k": np.full(degree, 50.0), "rest": rest, "damping": np.full(degree, 0.05), "planes": [],
            "balls": [], "g": np.array([0, 0, -9.81]), "dt": 1e-4}


def test_heavy_order_close_to_ascending():
    sc = hub_scene()
    a, b = po.OracleSim(sc), po.OracleSim(sc, heavy_threshold=96)
    a.step(1, po.ASCENDING)
    b.step(1, po.DEVICE)
    assert np.max(np.abs(a.vel - b.vel)) <= 1e-12 * np.max(np.abs(a.vel))


def test_integrator_free_fall_known_answers():
    """Constant gravity, no springs: the reference's VERLET starts with a = 0,
    which makes its positions the discrete Euler sum z0 - g dt^2 n(n+1)/2;
    its RK2 (half step, then full step from the saved state) integrates a
    constant acceleration exactly: z0 - g (n dt)^2 / 2."""
    n_steps, dt, g = 2000, 1e-4, 9.81
    sc = {"pos": np.array([[0.0, 0.0, 10.0], [1.0, 2.0, 3.0]]), "m": np.array([0.1, 0.2]),
          "left": np.zeros(0, np.int32), "right": np.zeros(0, np.int32), "k": np.zeros(0), "rest": np.zeros(0),
          "planes": [], "balls": [], "g": np.array([0.0, 0.0, -g]), "dt": dt}
    for integ, want in ((1, lambda z0, n: z0 - g * dt * dt * n * (n + 1) / 2),
                        (2, lambda z0, n: z0 - 0.5 * g * (n * dt) ** 2)):
        o = po.OracleSim(dict(sc, integrator=integ))
        o.step(n_steps)
        for i, z0 in ((0, 10.0), (1, 3.0)):
            assert abs(o.pos[i, 2] - want(z0, n_steps)) < 1e-12
        assert np.array_equal(o.pos[:, :2], sc["pos"][:, :2])
        assert abs(o.time - n_steps * dt) < 1e-12


def test_integrators_agree_on_a_smooth_oscillation():
    """A stiff pair of masses: the three integrators are first/second order
    schemes of the same ODE and agree to O(dt) over one period."""
    rng = np.random.default_rng(2)
    from titan_gb300 import workloads as wl
    sc = wl.lattice_scene((0, 0, 5.0), (0.5, 0.5, 0.5), 3, 3, 3, k=2e3, damping=0.0)
    sc["g"] = np.zeros(3)
    sc["vel"] = rng.normal(scale=0.05, size=sc["pos"].shape)
    pos = []
    for integ in (0, 1, 2):
        o = po.OracleSim(dict(sc, integrator=integ))
        o.step(2000)
        pos.append(o.pos.copy())
    assert np.max(np.abs(pos[1] - pos[0])) < 2e-3
    assert np.max(np.abs(pos[2] - pos[0])) < 2e-3


def test_stl_inside_oracle_cube_and_sphere():
    from tests import meshes
    rng = np.random.default_rng(3)
    pts = rng.uniform(-1.5, 1.5, size=(3000, 3))
    for mesh, truth in ((meshes.cube(), np.all(np.abs(pts) < 1.0, axis=1)),
                        (meshes.icosphere(1.0, levels=2), np.linalg.norm(pts, axis=1) < 0.95)):
        got = po.stl_inside(mesh, pts, num_rays=7, seed=11)
        # away from the surface the classification is exact
        if mesh.shape[0] == 12:
            far = np.min(np.abs(np.abs(pts) - 1.0), axis=1) > 1e-3
        else:
            r = np.linalg.norm(pts, axis=1)
            far = (r < 0.95) | (r > 1.0)
        assert np.array_equal(got[far], truth[far])
        # the same seed reproduces; another seed may differ only at the surface
        assert np.array_equal(got, po.stl_inside(mesh, pts, num_rays=7, seed=11))
