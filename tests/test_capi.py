"""C ABI checks that need no GPU: the library loads, exports every entry point
include/titan_gb300.h declares, and the host tile plan satisfies every
invariant the step kernel relies on."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

import titan_gb300 as tg
from titan_gb300 import workloads as wl

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include" / "titan_gb300.h").read_text()
    return sorted(set(re.findall(r"\b(titan_gb300_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = ctypes.CDLL(str(tg.library_path()))
    syms = declared_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing


def test_version_and_host_helpers():
    assert b"sm_103a" in tg.lib().titan_gb300_version()
    assert tg.lattice_springs(5, 5, 5) == 1036


def test_create_needs_no_gpu_and_validates():
    s = tg.Sim(tg.FP64)
    with pytest.raises(tg.TitanError):
        s.set_time_step(0.0)
    with pytest.raises(tg.TitanError):
        s.step(1)  # not started
    s.close()


# ------------------------------------------------------- plan validation ---
T = {name: i for i, name in enumerate(
    ["new2old", "tile_mass_off", "tile_halo_off", "halo", "tile_ent_off", "tile_nact", "ent_ends", "ent_spring",
     "tile_warp_off", "warp_inc_off", "deg", "inc", "tile_heavy_off", "heavy_local", "heavy_inc_off", "heavy_inc",
     "body_of_tile", "tile_nh"])}
DT = {"new2old": np.int32, "tile_mass_off": np.int64, "tile_halo_off": np.int64, "halo": np.int32,
      "tile_ent_off": np.int64, "tile_nact": np.int32, "ent_ends": np.uint32, "ent_spring": np.int64,
      "tile_warp_off": np.int64, "warp_inc_off": np.uint32, "deg": np.uint8, "inc": np.uint16,
      "tile_heavy_off": np.int64, "heavy_local": np.uint16, "heavy_inc_off": np.uint32, "heavy_inc": np.uint16,
      "body_of_tile": np.int32, "tile_nh": np.int32}


def plan_tables(sc, tile, precision=tg.FP32C, kernel=0):
    s = tg.Sim(precision)
    wl.load(s, sc, start=False, kernel=kernel)
    rc = s._L.titan_gb300_plan_host(s._h, tile)
    s._check(rc, "plan_host")
    out = {}
    for name, idx in T.items():
        n = s._L.titan_gb300_plan_table(s._h, idx, None)
        a = np.zeros(max(n, 0), DT[name])
        s._L.titan_gb300_plan_table(s._h, idx, a.ctypes.data_as(ctypes.c_void_p))
        out[name] = a
    s.close()
    return out


def validate(sc, P, heavy_threshold=96):
    n = sc["pos"].shape[0]
    left, right = sc["left"], sc["right"]
    ns = left.size
    fixed = sc.get("fixed")
    fixed = np.zeros(n, bool) if fixed is None else np.asarray(fixed, bool)
    typ = sc.get("type")
    new2old = P["new2old"]
    assert sorted(new2old.tolist()) == list(range(n))
    old2new = np.empty(n, np.int64)
    old2new[new2old] = np.arange(n)
    tmo = P["tile_mass_off"]
    ntiles = tmo.size - 1
    tile_of = np.empty(n, np.int64)
    for t in range(ntiles):
        tile_of[tmo[t]:tmo[t + 1]] = t
    if "body_ptr" in sc:
        bp = sc["body_ptr"]
        body_of_old = np.searchsorted(bp, np.arange(n), side="right") - 1
        for t in range(ntiles):
            bodies = set(body_of_old[new2old[tmo[t]:tmo[t + 1]]].tolist())
            assert bodies == {P["body_of_tile"][t]}
    valid = (left >= 0) & (right >= 0) & (left < n) & (right < n)
    # expected incidence per new mass: ascending springs, right before left
    expect = [[] for _ in range(n)]
    for s in range(ns):
        if not valid[s]:
            continue
        r, l = old2new[right[s]], old2new[left[s]]
        if not fixed[right[s]]:
            expect[r].append((s, 1))
        if not fixed[left[s]]:
            expect[l].append((s, -1))
    seen_in_tile = {}
    heavy_seen = 0
    for t in range(ntiles):
        m0, m1 = tmo[t], tmo[t + 1]
        nm = m1 - m0
        h0 = P["tile_halo_off"][t]
        assert h0 % 4 == 0 and P["tile_halo_off"][t + 1] - h0 == (P["tile_nh"][t] + 3) // 4 * 4
        halo = P["halo"][h0:h0 + P["tile_nh"][t]]
        assert np.all(np.diff(halo) > 0)
        assert not np.any((halo >= m0) & (halo < m1))
        slot2g = np.concatenate([np.arange(m0, m1), halo])
        e0, e1 = P["tile_ent_off"][t], P["tile_ent_off"][t + 1]
        ends = P["ent_ends"][e0:e1]
        sp = P["ent_spring"][e0:e1]
        nact = P["tile_nact"][t]
        if typ is not None:
            assert np.all(np.isin(typ[sp[:nact]], [2, 3])) and not np.any(np.isin(typ[sp[nact:]], [2, 3]))
        a, b, ty = ends & 0xFFF, (ends >> 12) & 0xFFF, (ends >> 24) & 3
        assert np.all(a < nm + halo.size) and np.all(b < nm + halo.size)
        assert np.array_equal(new2old[slot2g[a]], left[sp])
        assert np.array_equal(new2old[slot2g[b]], right[sp])
        if typ is not None:
            assert np.array_equal(ty, typ[sp] & 3)
        remote = set(slot2g[a][a >= nm].tolist()) | set(slot2g[b][b >= nm].tolist())
        assert remote == set(halo.tolist())
        for s in sp.tolist():
            seen_in_tile.setdefault(s, set()).add(t)
        # incidence
        w0 = P["tile_warp_off"][t]
        hl = P["heavy_local"][P["tile_heavy_off"][t]:P["tile_heavy_off"][t + 1]].tolist()
        for i in range(nm):
            g = m0 + i
            d = int(P["deg"][g])
            if d == 255:
                h = P["tile_heavy_off"][t] + hl.index(i)
                codes = P["heavy_inc"][P["heavy_inc_off"][h]:P["heavy_inc_off"][h + 1]]
                heavy_seen += 1
                assert len(expect[g]) > heavy_threshold
            else:
                off = int(P["warp_inc_off"][w0 + i // 32])
                assert off % 128 == 0  # 8-byte aligned groups of four codes
                j = np.arange(d)
                codes = P["inc"][off + (j // 4) * 128 + 4 * (i % 32) + (j % 4)]
            got = [(int(sp[c & 0x7FFF]), -1 if c & 0x8000 else 1) for c in codes.tolist()]
            assert got == expect[g], (t, i)
    assert heavy_seen == sum(1 for e in expect if len(e) > heavy_threshold)
    # each valid spring with a free end sits in the tile of every free end
    for s in range(ns):
        if not valid[s]:
            continue
        want = {tile_of[old2new[x]] for x in (left[s], right[s]) if not fixed[x]}
        assert seen_in_tile.get(s, set()) == want, s


@pytest.mark.parametrize("tile", [32, 64, 512])
def test_plan_lattice(tile):
    sc = wl.lattice_scene((0, 0, 1), (1, 1, 1), 9, 7, 8)
    validate(sc, plan_tables(sc, tile))


def test_plan_actuated_fixed_and_loops():
    rng = np.random.default_rng(2)
    sc = wl.lattice_scene((0, 0, 1), (1, 1, 1), 6, 6, 6)
    wl.actuate(sc, rng, 0.3, 0.1)
    sc["fixed"] = (rng.random(216) < 0.1).astype(np.uint8)
    # a self-loop, a dangling spring and a duplicate
    sc["left"] = np.concatenate([sc["left"], [5, -1, 3]]).astype(np.int32)
    sc["right"] = np.concatenate([sc["right"], [5, 7, 4]]).astype(np.int32)
    for key, val in (("k", 1e3), ("rest", 0.1), ("damping", 0.0), ("omega", 0.0), ("amp", 0.2), ("phase", 0.0)):
        sc[key] = np.concatenate([sc[key], [val] * 3])
    sc["type"] = np.concatenate([sc["type"], [0, 0, 0]]).astype(np.int32)
    validate(sc, plan_tables(sc, 64))


def test_plan_tiles_are_compact_blocks():
    """Recursive coordinate bisection: every tile of a 24^3 lattice is a
    near-cubic block of lattice sites (no side more than twice another),
    and the halos are those of blocks, not of runs of a space-filling
    curve."""
    n = 24
    sc = wl.lattice_scene((0, 0, 1), (1, 1, 1), n, n, n)
    P = plan_tables(sc, 192)
    validate(sc, P)
    tmo, new2old = P["tile_mass_off"], P["new2old"]
    ijk = np.stack(np.unravel_index(np.arange(n ** 3), (n, n, n)), 1)  # lattice builder order: i, j, k
    for t in range(tmo.size - 1):
        c = ijk[new2old[tmo[t]:tmo[t + 1]]]
        ext = c.max(0) - c.min(0) + 1
        assert ext.max() <= 2 * ext.min(), (t, ext)
        assert np.prod(ext) <= 2 * (tmo[t + 1] - tmo[t]), (t, ext)  # a block (cuts may split a layer)
    assert P["tile_nh"].mean() < 1.6 * np.diff(tmo).mean()


def test_plan_default_tile_adapts_and_keeps_small_bodies_whole():
    """Default tiles: a small lattice gets tiles small enough to cover the
    SMs; bodies that fit the large-scene tile (208 masses in FP32C, where
    the warp-specialised kernel runs) are one tile each even then; a large
    lattice gets the 208-mass tiles."""
    small = wl.lattice_scene((0, 0, 1), (1, 1, 1), 20, 20, 20)
    P = plan_tables(small, 0)
    nm = np.diff(P["tile_mass_off"])
    assert nm.max() <= 128 and P["tile_mass_off"].size - 1 >= 60
    sc = wl.robot_batch(nbodies=40, seed=3, side_range=(3, 7))
    P = plan_tables(sc, 0)
    bp = sc["body_ptr"]
    sizes = np.diff(bp)
    body_of_tile = P["body_of_tile"]
    for b in range(sizes.size):
        ntile = int(np.sum(body_of_tile == b))
        if sizes[b] <= 208:
            assert ntile == 1, (b, sizes[b], ntile)
    plain = wl.lattice_scene((0, 0, 1), (1, 1, 1), 64, 64, 64)
    d, p208 = plan_tables(plain, 0), plan_tables(plain, 208)
    assert all(np.array_equal(d[k], p208[k]) for k in d)


def denser_lattice(n, extra=1, seed=1):
    """A lattice plus `extra` springs per mass to random masses within three
    lattice steps (larger slabs and halos per tile than a plain lattice)."""
    sc = wl.lattice_scene((0, 0, 1), (1, 1, 1), n, n, n)
    pos = sc["pos"]
    N = pos.shape[0]
    rng = np.random.default_rng(seed)
    idx = np.arange(N)
    ijk = np.stack(np.unravel_index(idx, (n, n, n)), 1)
    L, R = [], []
    for _ in range(extra):
        tgt = np.clip(ijk + rng.integers(-3, 4, size=(N, 3)), 0, n - 1)
        j = np.ravel_multi_index(tgt.T, (n, n, n))
        keep = j != idx
        L.append(idx[keep])
        R.append(j[keep])
    L = np.concatenate(L).astype(np.int32)
    R = np.concatenate(R).astype(np.int32)
    for key, val in (("k", 1e3), ("damping", 0.0), ("omega", 0.0), ("amp", 0.2), ("phase", 0.0)):
        sc[key] = np.concatenate([sc[key], np.full(L.size, val)])
    sc["rest"] = np.concatenate([sc["rest"], np.linalg.norm(pos[L] - pos[R], axis=1)])
    sc["type"] = np.concatenate([sc["type"], np.zeros(L.size, np.int32)])
    sc["left"] = np.concatenate([sc["left"], L])
    sc["right"] = np.concatenate([sc["right"], R])
    return sc


def test_plan_default_tile_falls_back_when_two_stages_do_not_fit():
    """Large scenes plan 208-mass tiles for the warp-specialised kernel, or
    192 when two stages of the 208-mass tiles would not fit one SM's shared
    memory (checked on the host from the plan itself)."""
    plain = wl.lattice_scene((0, 0, 1), (1, 1, 1), 52, 52, 52)
    d, p208 = plan_tables(plain, 0, kernel=4), plan_tables(plain, 208, kernel=4)
    assert all(np.array_equal(d[k], p208[k]) for k in d)
    dense = denser_lattice(52)
    d, p192, p208 = plan_tables(dense, 0, kernel=4), plan_tables(dense, 192, kernel=4), plan_tables(dense, 208, kernel=4)
    assert all(np.array_equal(d[k], p192[k]) for k in d)
    assert p208["tile_mass_off"].size < p192["tile_mass_off"].size


def bank_wavefronts(P, rec_mod=8):
    """Mean 16-byte shared-memory wavefronts per quarter-warp endpoint load
    in phase B (1.0 = conflict-free)."""
    te, ends = P["tile_ent_off"], P["ent_ends"]
    tot = cnt = 0
    for t in range(te.size - 1):
        a = (ends[te[t]:te[t + 1]] & 0xFFF).astype(np.int64)
        b = ((ends[te[t]:te[t + 1]] >> 12) & 0xFFF).astype(np.int64)
        for g0 in range(0, a.size, 8):
            for arr in (a, b):
                xs = np.unique(arr[g0:g0 + 8])
                tot += np.bincount((3 * xs) % rec_mod, minlength=rec_mod).max()
                cnt += 1
    return tot / cnt


def test_plan_slab_groups_avoid_bank_conflicts():
    """The planner orders each tile's slab so that a quarter-warp's endpoint
    records mostly fall in distinct bank groups (spring order alone gives
    about 1.6-1.7 wavefronts per load on a lattice)."""
    sc = wl.actuated_lattice(n_side=16)
    P = plan_tables(sc, 192)
    assert bank_wavefronts(P) < 1.2


def gather_wavefronts(P):
    """Mean 16-byte shared-memory wavefronts per quarter-warp force gather
    (eight consecutive masses at one incidence position; codes past a
    mass's degree up to a whole word load the zero slot)."""
    tmo, two, wio, inc = P["tile_mass_off"], P["tile_warp_off"], P["warp_inc_off"], P["inc"]
    deg = np.where(P["deg"] == 255, 0, P["deg"]).astype(np.int64)
    tot = cnt = 0
    for t in range(tmo.size - 1):
        for w in range(two[t], two[t + 1]):
            m0 = tmo[t] + 32 * (w - two[t])
            m1 = min(m0 + 32, tmo[t + 1])
            d4 = (deg[m0:m1] + 3) // 4 * 4
            for q in range(0, m1 - m0, 8):
                lanes = np.arange(q, min(q + 8, m1 - m0))
                for j in range(int(d4[lanes].max())):
                    live = lanes[d4[lanes] > j]
                    slots = np.unique(inc[int(wio[w]) + (j // 4) * 128 + 4 * live + j % 4] & 0x7FFF)
                    tot += np.bincount(slots % 8, minlength=8).max()
                    cnt += 1
    return tot / cnt


def test_plan_slab_groups_spread_gathers():
    """Inside each slab group the planner places entries so that the force
    slots one quarter-warp gathers mostly fall in distinct bank groups
    (greedy placement alone: about 1.6 wavefronts per gather on a lattice)."""
    P = plan_tables(wl.actuated_lattice(n_side=16), 192)
    assert gather_wavefronts(P) < 1.45


def test_plan_is_deterministic():
    """The planner orders tile slabs on several host threads; two plans of
    the same scene are the same, table for table."""
    sc = wl.robot_batch(nbodies=48, seed=11, side_range=(3, 9))
    wl.actuate(sc, np.random.default_rng(4), 0.3, 0.1)
    a, b = plan_tables(sc, 0), plan_tables(sc, 0)
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    validate(sc, a)


def test_plan_heavy_hub():
    from tests.test_oracle import hub_scene
    sc = hub_scene(degree=300)
    validate(sc, plan_tables(sc, 64))


def test_plan_bodies():
    sc = wl.robot_batch(nbodies=12, seed=4, side_range=(3, 6))
    validate(sc, plan_tables(sc, 64))


def test_plan_rejects_hub_beyond_slab():
    n = 40000
    sc = {"pos": np.random.default_rng(0).normal(size=(n, 3)), "m": np.full(n, 0.1),
          "left": np.zeros(n - 1, np.int32), "right": np.arange(1, n, dtype=np.int32),
          "k": np.ones(n - 1), "rest": np.ones(n - 1), "planes": [], "balls": [], "g": np.zeros(3), "dt": 1e-4}
    with pytest.raises(tg.TitanError, match="ELIMIT"):
        plan_tables(sc, 64)


# ------------------------------------------------- resident bin plan -------
RT = {"bin_mass_off": (18, np.int64), "bin_warp_off": (19, np.int64), "mass": (20, np.int32),
      "body": (21, np.int32), "deg": (22, np.uint8), "act_mask": (23, np.uint64), "warp_rec_off": (24, np.uint32),
      "words": (25, np.uint32), "rec_spring": (26, np.int64), "resident": (27, np.uint8)}


def resident_tables(sc, resident, precision=tg.FP32C):
    s = tg.Sim(precision)
    wl.load(s, sc, start=False, resident=resident)
    s._check(s._L.titan_gb300_plan_host(s._h, 64), "plan_host")
    out = {}
    for name, (idx, dt) in list(RT.items()) + [("new2old", (0, np.int32))]:
        n = s._L.titan_gb300_plan_table(s._h, idx, None)
        a = np.zeros(max(n, 0), dt)
        s._L.titan_gb300_plan_table(s._h, idx, a.ctypes.data_as(ctypes.c_void_p))
        out[name] = a
    s.close()
    return out


def validate_resident(sc, R, cap):
    n = sc["pos"].shape[0]
    left, right, typ = sc["left"], sc["right"], sc["type"]
    fixed = np.zeros(n, bool) if sc.get("fixed") is None else np.asarray(sc["fixed"], bool)
    bp = sc["body_ptr"]
    nb = bp.size - 1
    body_of = np.repeat(np.arange(nb), np.diff(bp))
    old2new = np.empty(n, np.int64)
    old2new[R["new2old"]] = np.arange(n)
    valid = (left >= 0) & (right >= 0) & (left < n) & (right < n)
    cross = np.zeros(nb, bool)
    for s in np.flatnonzero(valid):
        if body_of[left[s]] != body_of[right[s]]:
            cross[body_of[left[s]]] = cross[body_of[right[s]]] = True
    # expected incidence (ascending springs) of every free mass, creation order
    inc = [[] for _ in range(n)]
    for s in np.flatnonzero(valid):
        if not fixed[right[s]]:
            inc[right[s]].append((s, left[s], 1))
        if not fixed[left[s]]:
            inc[left[s]].append((s, right[s], 0))
    for b in range(nb):
        nm = bp[b + 1] - bp[b]
        fits = nm <= cap and not cross[b] and max(len(inc[i]) for i in range(bp[b], bp[b + 1])) <= 254
        assert bool(R["resident"][b]) == fits, b
    nbins = R["bin_mass_off"].size - 1
    seen = set()
    for k in range(nbins):
        m0, m1 = R["bin_mass_off"][k], R["bin_mass_off"][k + 1]
        assert 0 < m1 - m0 <= cap
        tiled = R["mass"][m0:m1]
        old = R["new2old"][tiled]
        bodies = set(body_of[old].tolist())
        assert all(R["resident"][b] for b in bodies)
        # whole bodies, each once
        assert sum(bp[b + 1] - bp[b] for b in bodies) == m1 - m0
        assert not (bodies & seen)
        seen |= bodies
        assert (R["body"][m0:m1] == body_of[old]).all()
        local = {int(g): q for q, g in enumerate(tiled)}
        w0 = R["bin_warp_off"][k]
        assert R["bin_warp_off"][k + 1] - w0 == (m1 - m0 + 31) // 32
        for q in range(m1 - m0):
            i = old[q]
            d = R["deg"][m0 + q]
            assert d == len(inc[i])
            mask = 0
            for j, (s, other, is_right) in enumerate(inc[i]):
                r = R["warp_rec_off"][w0 + q // 32] + 32 * j + q % 32
                assert R["rec_spring"][r] == s
                w = int(R["words"][r])
                assert w & 0x7FFF == local[int(old2new[other])]
                assert bool(w & 0x8000) == bool(is_right)
                assert (w >> 16) & 3 == typ[s] & 3
                if j < 64 and typ[s] >= 2:
                    mask |= 1 << j
            assert int(R["act_mask"][m0 + q]) == mask
    assert seen == set(np.flatnonzero(R["resident"]).tolist())
    # bins are ordered by decreasing work
    work = [R["deg"][R["bin_mass_off"][k]:R["bin_mass_off"][k + 1]].sum() + np.diff(R["bin_mass_off"])[k]
            for k in range(nbins)]
    assert all(work[k] >= work[k + 1] for k in range(nbins - 1))


def test_resident_plan_bins():
    sc = wl.robot_batch(nbodies=30, seed=5, side_range=(3, 7))
    rng = np.random.default_rng(1)
    sc["fixed"] = (rng.random(sc["pos"].shape[0]) < 0.05).astype(np.uint8)
    validate_resident(sc, resident_tables(sc, (1, 512, 0)), 512)


def test_resident_plan_excludes_large_and_coupled_bodies():
    sc = wl.robot_batch(nbodies=16, seed=6, side_range=(3, 8))
    bp = sc["body_ptr"]
    # a spring between bodies 0 and 1 keeps both on the per-step kernels
    for key, val in (("left", bp[0]), ("right", bp[1]), ("k", 1e3), ("rest", 1.0), ("damping", 0.0), ("type", 0),
                     ("omega", 0.0), ("amp", 0.2), ("phase", 0.0)):
        sc[key] = np.concatenate([sc[key], [val]]).astype(sc[key].dtype)
    R = resident_tables(sc, (1, 128, 64))  # 64 threads: bins of at most 4 * 64 masses
    cap = 128
    validate_resident(sc, R, cap)
    assert not R["resident"][0] and not R["resident"][1]
    sizes = np.diff(bp)
    assert (R["resident"][sizes > cap] == 0).all()


def test_set_resident_validates():
    s = tg.Sim(tg.FP32C)
    for args in ((3, 0, 0), (-2, 0, 0), (1, -5, 0), (1, 0, 100), (1, 0, 1024)):
        with pytest.raises(tg.TitanError, match="EINVAL"):
            s.set_resident(*args)
    s.set_resident(1, 512, 128)
    s.set_resident(2)
    s.set_resident(-1)
    s.set_resident(0)
    s.close()


def test_set_occupancy_validates():
    s = tg.Sim(tg.FP32C)
    for v in (-1, 2, 5):
        with pytest.raises(tg.TitanError, match="EINVAL"):
            s.set_occupancy(v)
    s.set_occupancy(4)
    s.set_occupancy(0)
    s.close()


def test_export_indices_on_host_before_start():
    sc = wl.lattice_scene((0, 0, 1), (1, 1, 1), 3, 3, 3)
    sc["left"] = np.concatenate([sc["left"], [-1, 5]]).astype(np.int32)
    sc["right"] = np.concatenate([sc["right"], [4, -1]]).astype(np.int32)
    for key, val in (("k", 1e3), ("rest", 0.1), ("damping", 0.0), ("omega", 0.0), ("amp", 0.2), ("phase", 0.0)):
        sc[key] = np.concatenate([sc[key], [val] * 2])
    sc["type"] = np.concatenate([sc["type"], [0, 0]]).astype(np.int32)
    s = tg.Sim(tg.FP32C)
    wl.load(s, sc, start=False)
    idx = s.export_indices()
    ns = sc["left"].size
    assert idx.shape == (ns, 2)
    assert (idx[:-2, 0] == sc["left"][:-2]).all() and (idx[:-2, 1] == sc["right"][:-2]).all()
    assert (idx[-2:] == 0).all()  # detached springs export (0, 0)
    s.close()


def test_set_integrator_validates():
    s = tg.Sim(tg.FP64)
    for v in (-1, 3):
        with pytest.raises(tg.TitanError, match="EINVAL"):
            s.set_integrator(v)
    s.set_integrator(tg.RK2)
    s.set_integrator(tg.VERLET)
    s.close()


def test_plan_does_not_depend_on_planner_threads(monkeypatch):
    """Every planner pass splits its work over host threads; one thread and
    many give the same tables (a lone body and a batch of bodies)."""
    scenes = [(wl.actuated_lattice(n_side=40), 0), (wl.robot_batch(nbodies=96, seed=2, side_range=(3, 10)), 0)]
    for sc, tile in scenes:
        monkeypatch.setenv("TITAN_GB300_PLAN_THREADS", "1")
        one = plan_tables(sc, tile)
        monkeypatch.setenv("TITAN_GB300_PLAN_THREADS", "13")
        many = plan_tables(sc, tile)
        for k in one:
            assert np.array_equal(one[k], many[k]), k


CHILD_OOM = r"""
import resource, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import titan_gb300 as tg
from titan_gb300 import workloads as wl

def limit_to_now_plus(extra):
    vm = next(int(l.split()[1]) for l in open("/proc/self/status") if l.startswith("VmSize:")) * 1024
    resource.setrlimit(resource.RLIMIT_AS, (vm + extra, resource.getrlimit(resource.RLIMIT_AS)[1]))

s = tg.Sim(tg.FP32C)
if sys.argv[2] == "plan":
    wl.load(s, wl.actuated_lattice(n_side=60), start=False)
    limit_to_now_plus(64 << 20)
    call = lambda: s.plan_host(208)
else:  # host copies of 4M masses: pos and vel alone are 192 MB
    n = 4 << 20
    pos, vel, m = np.zeros((n, 3)), np.zeros((n, 3)), np.full(n, 0.1)
    limit_to_now_plus(64 << 20)
    call = lambda: s.set_masses(pos, m, vel=vel)
try:
    call()
    print("DONE")
except tg.TitanError as e:
    print("ERROR", e.code, e)
"""


@pytest.mark.parametrize("what", ["plan", "masses"])
def test_out_of_host_memory_is_an_error_code(what):
    """A host allocation that fails inside an entry point (the planner's
    threads included) comes back as a status, not an abort: the C ABI
    throws nothing."""
    import subprocess
    import sys
    if not Path("/proc/self/status").exists():
        pytest.skip("needs /proc")
    r = subprocess.run([sys.executable, "-c", CHILD_OOM, str(ROOT), what], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.startswith("ERROR") and "memory" in r.stdout, r.stdout
