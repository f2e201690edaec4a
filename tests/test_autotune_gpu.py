"""The autotuner times candidate launch shapes, caches the fastest, and the
tuned engine computes the same bits as the default one."""
import json

import numpy as np
import pytest

import titan_gb300 as tg
from titan_gb300 import autotune
from titan_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def test_autotune_caches_and_keeps_results(tmp_path):
    sc = wl.lattice_scene((0, 0, 1.0), (1, 1, 1), 14, 13, 12, k=3e3, damping=0.1)
    sc["planes"].append(((0.0, 0.0, 1.0), 0.0, 0.5, 0.5))
    cache = tmp_path / "tune.json"
    cfg = autotune.autotune(sc, tg.FP32C, steps=20, cache_path=cache)
    assert cfg["ms_per_step"] > 0 and len(cfg["tried"]) == len(autotune.CANDIDATES_F32)
    table = json.loads(cache.read_text())
    assert autotune.scene_key(sc, tg.FP32C) in table
    assert autotune.autotune(sc, tg.FP32C, cache_path=cache)["tile"] == cfg["tile"]  # from the cache
    s = autotune.make_tuned_sim(sc, tg.FP32C, cache_path=cache)
    s.step(300)
    a = s.get_state(acc=True)
    d = wl.make_sim(sc, tg.FP32C)
    d.step(300)
    b = d.get_state(acc=True)
    for k in ("pos", "vel", "acc"):
        assert np.array_equal(a[k], b[k])
