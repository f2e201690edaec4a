"""GPU parity: the fused sm_103a step against the CPU oracle.

Bar (stated per test):
  * FP64, passive springs: bit-identical to the oracle's ascending-spring
    order (one legal serialisation of the reference's atomics) for any number
    of steps -- max |diff| == 0 on positions, velocities and accelerations.
  * FP64, actuated springs: CUDA's sin and the host libm's sin may differ in
    the last bits, so the bar is 1e-12 relative per step and the oracle's own
    order spread over N steps.
  * FP32C: position error against FP64 stated in each test.
"""
import numpy as np
import pytest

import titan_gb300 as tg
from oracle import pyoracle as po
from titan_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def gpu_run(sc, nsteps, precision=tg.FP64, tile=0, chunks=None, kernel=0, threads=0, resident=None):
    s = wl.make_sim(sc, precision, tile, kernel=kernel, threads=threads, resident=resident)
    if chunks:
        for c in chunks:
            s.step(c)
    else:
        s.step(nsteps)
    st = s.get_state(acc=True, T=True)
    return s, st


def oracle_run(sc, nsteps, order=po.ASCENDING, threads=1):
    o = po.OracleSim(sc)
    o.step(nsteps, order, threads)
    return o


def assert_bitwise(st, o):
    assert np.array_equal(st["pos"], o.pos), np.max(np.abs(st["pos"] - o.pos))
    assert np.array_equal(st["vel"], o.vel), np.max(np.abs(st["vel"] - o.vel))
    assert np.array_equal(st["acc"], o.acc), np.max(np.abs(st["acc"] - o.acc))
    assert np.array_equal(st["T"], o.T)


def test_falling_cube_free_fall_10k_steps_bitwise():
    sc = wl.falling_cube()
    s, st = gpu_run(sc, 10000)
    o = oracle_run(sc, 10000)
    assert_bitwise(st, o)
    assert s.time == o.time


def test_falling_cube_contact_friction_10k_steps_bitwise():
    sc = wl.falling_cube(contact=True)
    sc["vel"] = np.random.default_rng(1).normal(scale=0.3, size=sc["pos"].shape)
    _, st = gpu_run(sc, 10000)
    o = oracle_run(sc, 10000)
    assert_bitwise(st, o)
    assert np.min(o.pos[:, 2]) < 0.0  # the plane and friction were exercised


@pytest.mark.parametrize("tile", [32, 64, 256])
def test_many_tiles_halo_damping_ball_bitwise(tile):
    rng = np.random.default_rng(3)
    sc = wl.lattice_scene((0, 0, 0.55), (1.0, 0.8, 0.9), 9, 7, 8, k=2e3, damping=0.2)
    sc["k"] = np.exp(rng.uniform(np.log(1e3), np.log(1e4), sc["k"].size))
    sc["vel"] = rng.normal(scale=0.5, size=sc["pos"].shape)
    sc["planes"].append(((0.0, 0.1, 1.0), 0.0, 0.4, 0.6))
    sc["balls"].append(((0.3, 0.0, -0.1), 0.35))  # the lattice's bottom corner sits inside it
    _, st = gpu_run(sc, 2000, tile=tile)
    o = oracle_run(sc, 2000)
    assert_bitwise(st, o)


def test_fixed_ext_drag_local_constraints_bitwise():
    rng = np.random.default_rng(4)
    sc = wl.lattice_scene((0, 0, 1.0), (1, 1, 1), 5, 5, 5, k=5e3, damping=0.1)
    n = sc["pos"].shape[0]
    sc["vel"] = rng.normal(scale=0.2, size=(n, 3))
    sc["fixed"] = np.zeros(n, np.uint8)
    sc["fixed"][:25] = 1  # a Beam-like fixed face
    sc["ext"] = np.zeros((n, 3))
    sc["ext"][60] = [0.5, -0.2, 3.0]
    sc["drag"] = np.zeros(n)
    sc["drag"][[70, 71]] = [2.7, 0.5]
    ptr = np.zeros(n + 1, np.int64)
    types, vecs, nums = [], [], []
    special = {80: [(0, (0, 0, 1), 0.3)], 81: [(3, (1, 1, 0), 0.2)], 82: [(1, (0, 0, 1), 0.9)],
               83: [(2, (0.2, 0.2, 1.0), 0.5), (0, (1, 0, 0), 0.1)]}
    for i in range(n):
        for t, v, num in special.get(i, []):
            types.append(t)
            vecs.append(v)
            nums.append(num)
        ptr[i + 1] = len(types)
    sc.update(lc_ptr=ptr, lc_type=np.array(types, np.int32), lc_vec=np.array(vecs, float),
              lc_num=np.array(nums, float))
    _, st = gpu_run(sc, 1500, tile=64)
    o = oracle_run(sc, 1500)
    assert_bitwise(st, o)
    assert np.array_equal(st["pos"][:25], sc["pos"][:25])


def test_heavy_hub_device_order_bitwise():
    from tests.test_oracle import hub_scene
    sc = hub_scene(degree=300)
    _, st = gpu_run(sc, 500, tile=64)
    o = oracle_run(sc, 500, po.DEVICE)
    assert_bitwise(st, o)


def test_bodies_with_own_planes_bitwise():
    sc = wl.robot_batch(nbodies=24, seed=9, side_range=(3, 7))
    for key in ("type",):
        sc[key][:] = 0  # passive: bitwise bar
    _, st = gpu_run(sc, 3000, tile=128, resident=(0, 0, 0))
    o = oracle_run(sc, 3000)
    assert_bitwise(st, o)


def test_actuated_springs_tolerance():
    """Reference actuation (amp 0.2, no phase) and the amplitude/phase
    extension: 1e-12 relative after one step; after 2000 steps within the
    spread between two legal atomic orders of the oracle (plus 1e-12)."""
    rng = np.random.default_rng(5)
    sc = wl.lattice_scene((0, 0, 0.8), (1, 1, 1), 6, 6, 6, k=3e3, damping=0.05)
    wl.actuate(sc, rng, 0.5, 0.2)
    sc["amp"][::2] = 0.2
    sc["phase"][::2] = 0.0  # the reference's own actuation on half the springs
    sc["planes"].append(((0.0, 0.0, 1.0), 0.0, 0.5, 0.5))
    _, st1 = gpu_run(sc, 1)
    o1 = oracle_run(sc, 1)
    scale = np.max(np.abs(o1.vel))
    assert np.max(np.abs(st1["vel"] - o1.vel)) <= 1e-12 * scale
    _, st = gpu_run(sc, 2000)
    oa, od = oracle_run(sc, 2000), oracle_run(sc, 2000, po.DESCENDING)
    spread = np.max(np.abs(oa.pos - od.pos))
    assert np.max(np.abs(st["pos"] - oa.pos)) <= spread + 1e-12


def kernel_scenes():
    from tests.test_oracle import hub_scene
    rng = np.random.default_rng(11)
    lat = wl.lattice_scene((0, 0, 0.55), (1.0, 0.8, 0.9), 9, 7, 8, k=2e3, damping=0.2)
    lat["vel"] = rng.normal(scale=0.5, size=lat["pos"].shape)
    wl.actuate(lat, rng, 0.3, 0.1)
    lat["planes"].append(((0.0, 0.1, 1.0), 0.0, 0.4, 0.6))
    lat["balls"].append(((0.3, 0.0, -0.1), 0.35))
    # damping that differs between springs (the pull form's per-column path)
    var = wl.lattice_scene((0, 0, 0.55), (1.0, 0.8, 0.9), 9, 7, 8, k=2e3, damping=0.2)
    var["vel"] = rng.normal(scale=0.5, size=var["pos"].shape)
    var["damping"] = rng.uniform(0.0, 0.4, var["damping"].size)
    var["damping"][::5] = 0.0
    wl.actuate(var, rng, 0.3, 0.1)
    var["planes"].append(((0.0, 0.0, 1.0), 0.0, 0.5, 0.5))
    return {"lattice": lat, "hub": hub_scene(degree=300), "bodies": wl.robot_batch(nbodies=24, seed=9, side_range=(3, 7)),
            "damping": var}


@pytest.mark.parametrize("precision", [tg.FP64, tg.FP32, tg.FP32C])
@pytest.mark.parametrize("scene", ["lattice", "hub", "bodies", "damping"])
@pytest.mark.parametrize("tile", [32, 96])
def test_kernel_forms_bitwise_identical(precision, scene, tile):
    """The per-tile kernel, the per-tile kernel with asynchronous staging,
    the warp-specialised kernel and (FP32 and FP32C) the pull kernel give
    identical bits; the pull kernel refuses a scene with a heavy mass."""
    sc = kernel_scenes()[scene]
    s1, a = gpu_run(sc, 700, precision, tile=tile, kernel=1, resident=(0, 0, 0))
    s3, c = gpu_run(sc, 700, precision, tile=tile, kernel=3, resident=(0, 0, 0))
    s4, d = gpu_run(sc, 700, precision, tile=tile, kernel=4, resident=(0, 0, 0))
    assert s1.kernel_info()["kernel"] == "per-tile" and s3.kernel_info()["kernel"] == "per-tile-async"
    assert s4.kernel_info()["kernel"] == "warp-specialised"
    others = [c, d]
    if precision != tg.FP64:
        if scene == "hub":
            with pytest.raises(tg.TitanError, match="ELIMIT"):
                gpu_run(sc, 1, precision, tile=tile, kernel=6, resident=(0, 0, 0))
        else:
            s6, e = gpu_run(sc, 700, precision, tile=tile, kernel=6, resident=(0, 0, 0))
            assert s6.kernel_info()["kernel"] == "pull"
            others.append(e)
    for k in ("pos", "vel", "acc", "T"):
        for o in others:
            assert np.array_equal(a[k], o[k]), k


@pytest.mark.parametrize("precision", [tg.FP64, tg.FP32C])
def test_persistent_kernels_with_more_tiles_than_ctas(precision):
    """Tiles walked by a persistent grid (warp-specialised and pull forms):
    more tiles than CTAs, odd counts, partial units."""
    sc = wl.lattice_scene((0, 0, 1.0), (2, 2, 2), 41, 39, 37, k=3e3, damping=0.1)
    sc["planes"].append(((0.0, 0.0, 1.0), 0.0, 0.5, 0.5))
    _, a = gpu_run(sc, 300, precision, tile=48, kernel=1)
    for form in ((4, 6) if precision != tg.FP64 else (4,)):
        s, b = gpu_run(sc, 300, precision, tile=48, kernel=form)
        info = s.kernel_info()
        assert info["ctas"] < s.plan_info()["tiles"]
        assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["vel"], b["vel"])


def test_graph_chunks_equal_single_steps_and_repeatable():
    sc = wl.falling_cube(contact=True)
    _, a = gpu_run(sc, 777)
    _, b = gpu_run(sc, 777, chunks=[1] * 77 + [100, 600])
    _, c = gpu_run(sc, 777)
    for k in ("pos", "vel", "acc", "T"):
        assert np.array_equal(a[k], b[k]) and np.array_equal(a[k], c[k])


def test_state_roundtrip_and_partial_set():
    sc = wl.falling_cube(contact=True)
    s = wl.make_sim(sc)
    s.step(500)
    st = s.get_state(acc=True, T=True)
    idx = np.array([3, 17, 99])
    sub = s.get_masses(idx, acc=True, T=True)
    for k in ("pos", "vel", "acc", "T"):
        assert np.array_equal(sub[k], st[k][idx])
    # set a few masses, as set(Mass*) does, and mirror it in the oracle
    o = oracle_run(sc, 500)
    newp = st["pos"][idx] + [0.0, 0.0, 0.01]
    s.set_mass_state(idx, pos=newp)
    o.pos[idx] = newp
    s.step(300)
    o.step(300)
    st2 = s.get_state()
    assert np.array_equal(st2["pos"], o.pos)


def test_fix_after_start_rebuilds_plan():
    sc = wl.falling_cube(contact=True)
    s = wl.make_sim(sc)
    o = po.OracleSim(sc)
    s.step(200)
    o.step(200)
    fixed = np.zeros(125, np.uint8)
    fixed[:10] = 1
    s.set_mass_state(None, fixed=fixed)
    o._keep["fixed"] = fixed
    o.s.fixed = o._keep["fixed"].ctypes.data_as(po.ctypes.POINTER(po.ctypes.c_uint8))
    s.step(300)
    o.step(300)
    st = s.get_state()
    assert np.array_equal(st["pos"], o.pos)


def test_spring_param_update():
    sc = wl.falling_cube(contact=True)
    s = wl.make_sim(sc)
    s.step(100)
    o = oracle_run(sc, 100)
    k2 = sc["k"] * 1.5
    s.set_spring_params(k=k2)
    o._keep["k"][:] = k2
    s.step(200)
    o.step(200)
    assert np.array_equal(s.get_state()["pos"], o.pos)


def test_diagnostics_match_oracle():
    sc = wl.falling_cube(contact=True)
    s, st = gpu_run(sc, 3000)
    o = oracle_run(sc, 3000)
    d = s.diagnostics(9.8)
    e = o.energy(9.8)
    lin, ang = o.momentum()
    np.testing.assert_allclose([d["spring_pe"], d["kinetic"], d["gravity_pe"], d["total"]], e, rtol=1e-12)
    np.testing.assert_allclose(d["linear"], lin, rtol=1e-11, atol=1e-13)
    np.testing.assert_allclose(d["angular"], ang, rtol=1e-11, atol=1e-13)


def fp_errors(sc, nsteps):
    _, ref = gpu_run(sc, nsteps, tg.FP64)
    _, c = gpu_run(sc, nsteps, tg.FP32C)
    _, f = gpu_run(sc, nsteps, tg.FP32)
    return np.max(np.abs(c["pos"] - ref["pos"])), np.max(np.abs(f["pos"] - ref["pos"]))


def test_fp32c_error_free_flight_10k_steps():
    """No contact (config 1 as given: the lattice never reaches the plane):
    FP32C stays under 1e-5 m of FP64 after 10^4 steps; plain FP32 does not
    need to."""
    sc = wl.falling_cube()
    err_c, err_f = fp_errors(sc, 10000)
    print(f"free flight 10^4 steps: fp32c {err_c:.3e} m, fp32 {err_f:.3e} m")
    assert err_c < 1e-5
    assert err_c < err_f


def test_fp32c_contact_statistics_against_fp64():
    """Frictional contact is chaotic: two legal FP64 atomic orders of the
    reference already diverge by millimetres within 10^4 steps, so a pointwise
    bound is meaningless there.  FP32C must agree with FP64 in the
    statistics: total energy within 0.5% after 10^4 steps of the contact
    scene.  The pointwise errors are printed for the record."""
    sc = wl.falling_cube(contact=True)
    s64, ref = gpu_run(sc, 10000, tg.FP64)
    s32, c = gpu_run(sc, 10000, tg.FP32C)
    oa, od = oracle_run(sc, 10000), oracle_run(sc, 10000, po.DESCENDING)
    spread = np.max(np.abs(oa.pos - od.pos))
    err_c = np.max(np.abs(c["pos"] - ref["pos"]))
    e64, e32 = s64.diagnostics(9.81)["total"], s32.diagnostics(9.81)["total"]
    print(f"contact 10^4 steps: fp32c {err_c:.3e} m vs fp64; fp64 order spread {spread:.3e} m; "
          f"energy fp64 {e64:.6f} fp32c {e32:.6f}")
    assert abs(e32 - e64) <= 5e-3 * abs(e64)


def test_full_size_actuated_lattice_fp64_matches_oracle_three_steps():
    """The single-lattice workload at full size (100^3 masses, 12.7M
    springs, 20% actuated): three FP64 steps against the oracle (parallel,
    device order), 1e-12 relative on velocities; positions finite."""
    sc = wl.actuated_lattice()
    s = wl.make_sim(sc, tg.FP64)
    s.step(3)
    st = s.get_state()
    o = po.OracleSim(sc)
    o.step(3, po.DEVICE, po.host_threads())
    dv = np.max(np.abs(st["vel"] - o.vel))
    assert dv <= 1e-12 * max(1.0, np.max(np.abs(o.vel))), dv
    assert np.max(np.abs(st["pos"] - o.pos)) <= 1e-12 * np.max(np.abs(o.pos))


def test_full_size_actuated_lattice_fp32c_vs_fp64_200_steps():
    sc = wl.actuated_lattice()
    _, a = gpu_run(sc, 200, tg.FP64)
    _, b = gpu_run(sc, 200, tg.FP32C)
    assert np.all(np.isfinite(b["pos"]))
    err = np.max(np.abs(a["pos"] - b["pos"]))
    print(f"100^3 fp32c vs fp64 after 200 steps: {err:.3e} m")
    assert err < 1e-6


@pytest.mark.parametrize("precision", [tg.FP32, tg.FP32C])
@pytest.mark.parametrize("occupancy", [3, 4])
def test_register_capped_variants_bitwise_identical(precision, occupancy):
    """Launch-bound variants of the per-tile kernel compute the same bits."""
    sc = kernel_scenes()["lattice"]
    _, a = gpu_run(sc, 500, precision, tile=64, threads=128, kernel=1)
    s = wl.make_sim(sc, precision, 64, threads=128, kernel=1, occupancy=occupancy)
    s.step(500)
    b = s.get_state(acc=True, T=True)
    for k in ("pos", "vel", "acc", "T"):
        assert np.array_equal(a[k], b[k]), k
