"""Host transfers through the C ABI (capi.cu get_masses / set_mass_state):
page-locked caller buffers move by DMA directly, pageable ones through the
handle's staging buffer, and partial requests download only what was asked
for.  Bar: identical bytes on both paths."""
import numpy as np
import pytest

import titan_gb300 as tg
from titan_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [tg.FP64, tg.FP32C])
def test_pinned_and_pageable_paths_agree(precision):
    sc = wl.actuated_lattice(n_side=24)
    n = sc["pos"].shape[0]
    rng = np.random.default_rng(3)
    pos = sc["pos"] + rng.normal(scale=1e-3, size=(n, 3))
    vel = rng.normal(scale=0.1, size=(n, 3))
    pos_p, vel_p = tg.pinned_empty((n, 3)), tg.pinned_empty((n, 3))
    pos_p[:] = pos
    vel_p[:] = vel
    got = []
    for pinned in (False, True):
        s = wl.make_sim(sc, precision)
        if pinned:
            s.set_mass_state(None, pos=pos_p, vel=vel_p)
        else:
            s.set_mass_state(None, pos=pos, vel=vel)
        s.step(50)
        if pinned:
            out = {k: tg.pinned_empty((n, 3)) for k in ("pos", "vel", "acc")}
            st = s.get_state(pos=True, vel=True, acc=True, out=out)
            assert st["pos"] is out["pos"]  # filled in place
        else:
            st = s.get_state(pos=True, vel=True, acc=True)
        only_vel = s.get_state(pos=False, vel=True)
        assert "pos" not in only_vel and np.array_equal(only_vel["vel"], st["vel"])
        idx = np.arange(0, n, 97)
        part = s.get_masses(idx, pos=True, vel=False, acc=True)
        assert np.array_equal(part["pos"], st["pos"][idx]) and np.array_equal(part["acc"], st["acc"][idx])
        got.append({k: np.array(v) for k, v in st.items()})
        s.close()
    for k in ("pos", "vel", "acc"):
        assert np.array_equal(got[0][k], got[1][k]), k
    assert np.all(np.isfinite(got[0]["pos"]))


def test_pinned_empty_is_writable_and_freed():
    a = tg.pinned_empty((1000, 3))
    a[:] = 1.5
    assert a.shape == (1000, 3) and a.dtype == np.float64 and float(a.sum()) == 4500.0
    del a  # freed with its last view
