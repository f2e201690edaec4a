"""GPU parity of the resident launches: bins of whole bodies (resident.cu)
and halo-free tiles (resident_tiles.cu).

Bar: bit-identical to the per-step kernels in every precision, and in FP64
(passive springs) to the oracle's ascending order -- max |diff| == 0 on
positions, velocities, accelerations and per-mass time, across step() calls
of any length and with per-step tiles running beside the bins."""
import numpy as np
import pytest

import titan_gb300 as tg
from oracle import pyoracle as po
from titan_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def batch(nbodies=40, seed=12, side_range=(3, 7), passive=True):
    sc = wl.robot_batch(nbodies=nbodies, seed=seed, side_range=side_range)
    rng = np.random.default_rng(seed)
    n = sc["pos"].shape[0]
    if passive:
        sc["type"][:] = 0
    sc["fixed"] = (rng.random(n) < 0.03).astype(np.uint8)
    ext = np.zeros((n, 3))
    pick = rng.random(n) < 0.1
    ext[pick] = rng.normal(scale=0.5, size=(pick.sum(), 3))
    sc["ext"] = ext
    sc["vel"] = rng.normal(scale=0.3, size=(n, 3))
    sc["planes"].append(((0.0, 0.0, 1.0), -0.02, 0.5, 0.5))  # a global plane under the bodies' own planes
    return sc


def run(sc, chunks, precision=tg.FP64, resident=(1, 0, 0), tile=128, edit=None):
    # tile 128: every body of up to 128 masses is one tile in every precision
    # (default FP64 tiles of small scenes are smaller, to spread over SMs)
    s = wl.make_sim(sc, precision, tile, resident=resident)
    for q, c in enumerate(chunks):
        s.step(c)
        if edit is not None and q == 0:
            edit(s)
    return s, s.get_state(acc=True, T=True)


def assert_same(a, b):
    for k in ("pos", "vel", "acc", "T"):
        assert np.array_equal(a[k], b[k]), (k, np.max(np.abs(a[k] - b[k])))


def test_resident_fp64_bitwise_vs_oracle():
    sc = batch()
    chunks = [1, 7, 64, 300, 128]
    s, st = run(sc, chunks)
    info = s.resident_info()
    assert info["active"] and info["bodies"] == 40 and info["masses"] == sc["pos"].shape[0]
    assert s.plan_info()["tiles"] > 0
    o = po.OracleSim(sc)
    o.step(sum(chunks), po.ASCENDING, 1)
    assert np.array_equal(st["pos"], o.pos), np.max(np.abs(st["pos"] - o.pos))
    assert np.array_equal(st["vel"], o.vel)
    assert np.array_equal(st["acc"], o.acc)
    assert np.array_equal(st["T"], o.T)
    assert s.time == o.time


def test_resident_bins_beside_per_step_tiles_bitwise():
    """Bins of 128 masses: larger bodies, and two bodies joined by a spring,
    run on the per-step kernels in the same step() calls."""
    sc = batch(nbodies=20, seed=13, side_range=(3, 8))
    bp = sc["body_ptr"]
    for key, val in (("left", bp[0]), ("right", bp[1]), ("k", 500.0), ("rest", 1.0), ("damping", 0.0), ("type", 0),
                     ("omega", 0.0), ("amp", 0.2), ("phase", 0.0)):
        sc[key] = np.concatenate([sc[key], [val]]).astype(sc[key].dtype)
    chunks = [3, 250, 1, 146]
    s, st = run(sc, chunks, resident=(1, 128, 64))
    info = s.resident_info()
    sizes = np.diff(bp)
    assert info["active"] and info["cap"] == 128
    assert info["bodies"] == int(np.sum(sizes[2:] <= 128))
    # the per-step kernels launch only the tiles of the other bodies
    assert 0 < s.kernel_info()["ctas"] < s.plan_info()["tiles"]
    o = po.OracleSim(sc)
    o.step(sum(chunks), po.ASCENDING, 1)
    for k, v in (("pos", o.pos), ("vel", o.vel), ("acc", o.acc), ("T", o.T)):
        assert np.array_equal(st[k], v), k


@pytest.mark.parametrize("precision", [tg.FP64, tg.FP32, tg.FP32C])
@pytest.mark.parametrize("shape", [(1, 0, 0), (1, 256, 64), (1, 512, 128), (2, 0, 0), (2, 0, 64)])
def test_resident_equals_per_step_kernels(precision, shape):
    """Actuated bodies, a mid-run state upload: resident bins and resident
    tiles (several CTA shapes, 1 to 4 masses per thread) and the per-step
    kernels agree bit for bit."""
    sc = batch(nbodies=30, seed=14, side_range=(3, 8), passive=False)
    n = sc["pos"].shape[0]
    idx = np.arange(0, n, 7, dtype=np.int64)
    newpos = sc["pos"][idx] + 0.01

    def edit(s):
        s.set_mass_state(idx, pos=newpos)

    chunks = [1, 299, 64, 236]
    sr, a = run(sc, chunks, precision, resident=shape, edit=edit)
    assert sr.resident_info()["active"]
    sp, b = run(sc, chunks, precision, resident=(0, 0, 0), edit=edit)
    assert not sp.resident_info()["active"]
    assert_same(a, b)


def test_resident_only_scene_time_and_repeat():
    """Every body resident: no per-step tile runs, the device time record
    advances through the resident launch alone."""
    sc = batch(nbodies=12, seed=15, side_range=(3, 5))
    s, a = run(sc, [5, 1, 94])
    assert s.plan_info()["tiles"] > 0 and s.resident_info()["bodies"] == 12
    o = po.OracleSim(sc)
    o.step(100, po.ASCENDING, 1)
    assert np.array_equal(a["pos"], o.pos) and np.array_equal(a["T"], o.T)
    s2, b = run(sc, [100])
    assert_same(a, b)


def test_resident_tiles_fp64_bitwise_vs_oracle():
    """Every body in one halo-free tile: the resident tiles carry the whole
    scene, bit-identical to the oracle's ascending order in FP64."""
    sc = batch(nbodies=40, seed=16, side_range=(3, 5))  # at most 125 masses: one FP64 tile (128) each
    chunks = [1, 7, 64, 300, 128]
    s, st = run(sc, chunks, resident=(2, 0, 0))
    info = s.resident_info()
    assert info["active"] == 2 and info["bodies"] == 40 and info["masses"] == sc["pos"].shape[0]
    o = po.OracleSim(sc)
    o.step(sum(chunks), po.ASCENDING, 1)
    for k, v in (("pos", o.pos), ("vel", o.vel), ("acc", o.acc), ("T", o.T)):
        assert np.array_equal(st[k], v), k
    assert s.time == o.time


def test_resident_tiles_beside_per_step_tiles_bitwise():
    """Tiles of 64 masses: bodies larger than a tile (tiles with halos), and
    two bodies joined by a spring, run on the per-step kernels in the same
    step() calls as the halo-free tiles."""
    sc = batch(nbodies=20, seed=17, side_range=(3, 8))
    bp = sc["body_ptr"]
    for key, val in (("left", bp[0]), ("right", bp[1]), ("k", 500.0), ("rest", 1.0), ("damping", 0.0), ("type", 0),
                     ("omega", 0.0), ("amp", 0.2), ("phase", 0.0)):
        sc[key] = np.concatenate([sc[key], [val]]).astype(sc[key].dtype)
    chunks = [3, 250, 1, 146]
    s, st = run(sc, chunks, resident=(2, 0, 0), tile=64)
    info = s.resident_info()
    sizes = np.diff(bp)
    assert info["active"] == 2 and info["cap"] <= 64
    assert info["bodies"] == int(np.sum(sizes[2:] <= 64))
    assert 0 < s.kernel_info()["ctas"] < s.plan_info()["tiles"]
    o = po.OracleSim(sc)
    o.step(sum(chunks), po.ASCENDING, 1)
    for k, v in (("pos", o.pos), ("vel", o.vel), ("acc", o.acc), ("T", o.T)):
        assert np.array_equal(st[k], v), k


@pytest.mark.parametrize("precision", [tg.FP64, tg.FP32, tg.FP32C])
def test_resident_tiles_single_body_with_contact(precision):
    """The small-robot scene (one actuated 125-mass lattice on a friction
    plane): one resident tile with its records staged in shared memory,
    bit-identical to the per-step kernels over calls of any length."""
    sc = wl.actuate(wl.falling_cube(contact=True), np.random.default_rng(7), 0.3, 0.1)
    chunks = [1, 63, 200, 2000]
    s1, a = run(sc, chunks, precision, resident=(2, 0, 0))
    i1 = s1.resident_info()
    assert i1["active"] == 2 and i1["bins"] == 1 and i1["masses"] == 125
    s2, b = run(sc, chunks, precision, resident=(0, 0, 0))
    assert_same(a, b)


def test_resident_tiles_heavy_hub_bitwise():
    """A hub mass of degree 300 (warp-cooperative heavy sum) in a resident
    tile: bit-identical to the oracle's device order in FP64."""
    from tests.test_oracle import hub_scene
    sc = hub_scene(degree=300)
    s, st = run(sc, [1, 99, 400], resident=(2, 0, 0), tile=512)
    assert s.resident_info()["active"] == 2
    o = po.OracleSim(sc, heavy_threshold=96)
    o.step(500, po.DEVICE, 1)
    for k, v in (("pos", o.pos), ("vel", o.vel), ("acc", o.acc)):
        assert np.array_equal(st[k], v), k


def test_automatic_resident_tiles_choice():
    """By default resident tiles carry the halo-free tiles (symplectic
    Euler, automatic kernel form): a whole small scene, the small bodies of
    a batch beside the per-step kernels, nothing of a single large lattice."""
    small = wl.falling_cube(contact=True)
    s = wl.make_sim(small, tg.FP32C)
    assert s.resident_info()["active"] == 2 and s.plan_info()["tiles"] == 1
    assert s.kernel_info()["kernel"] == "resident-tiles" and s.kernel_info()["ctas"] == 1
    s.close()
    s = wl.make_sim(small, tg.FP32C, kernel=1)  # an explicit kernel form: per-step kernels
    assert s.resident_info()["active"] == 0
    s.close()
    s = wl.make_sim(wl.actuated_lattice(n_side=20), tg.FP32C)  # tiles with halos
    assert s.resident_info()["active"] == 0
    s.close()
    mixed = batch(nbodies=24, seed=21, side_range=(3, 9), passive=False)  # 9^3 bodies span several tiles
    s = wl.make_sim(mixed, tg.FP32C)
    info = s.resident_info()
    assert info["active"] == 2 and 0 < info["bins"] < s.plan_info()["tiles"]
    assert s.kernel_info()["kernel"] == "warp-specialised"
    s.step(1)
    s.step(299)
    a = s.get_state(acc=True, T=True)
    s.close()
    _, b = run(mixed, [1, 299], tg.FP32C, resident=(0, 0, 0))
    assert_same(a, b)
    sc = dict(small, integrator=tg.VERLET)
    s = wl.make_sim(sc, tg.FP64)
    assert s.resident_info()["active"] == 0
    s.close()


def test_set_integrator_leaves_resident_tiles_bitwise():
    """A switch to RK2 after some Euler steps rebuilds the scene on the
    per-step kernels: same bits as a run that never had resident tiles."""
    sc = wl.actuate(wl.falling_cube(contact=True), np.random.default_rng(8), 0.3, 0.1)
    out = []
    for res in ((2, 0, 0), (0, 0, 0)):
        s = wl.make_sim(sc, tg.FP64, 128, resident=res)  # the body in one tile
        s.step(300)
        s.set_integrator(tg.RK2)
        s.step(200)
        assert s.resident_info()["active"] == 0
        out.append(s.get_state(acc=True, T=True))
    assert_same(*out)


@pytest.mark.parametrize("precision", [tg.FP64, tg.FP32C])
def test_resident_tiles_many_tiles_bitwise(precision):
    """More halo-free tiles than SMs (unstaged records, CTAs of 128
    threads) and fewer (staged records, wider CTAs): both bit-identical to
    the per-step kernels."""
    sc = batch(nbodies=200, seed=18, side_range=(3, 5), passive=False)
    chunks = [2, 97, 101]
    s1, a = run(sc, chunks, precision, resident=(2, 0, 0))
    assert s1.resident_info()["bins"] == 200
    s2, b = run(sc, chunks, precision, resident=(0, 0, 0))
    assert_same(a, b)
    few = batch(nbodies=8, seed=19, side_range=(3, 5), passive=False)
    s3, c = run(few, chunks, precision, resident=(2, 0, 0))
    s4, d = run(few, chunks, precision, resident=(0, 0, 0))
    assert_same(c, d)
