"""Host logic of the autotuner (titan_gb300/autotune.py) on the CPU: the
fastest candidate is chosen, failing candidates are recorded and skipped,
results are cached on disk per scene and reused, and refresh re-times.
Candidate timing is a stand-in here; the GPU tests time the real kernels."""
import json

import pytest

import titan_gb300 as tg
from titan_gb300 import autotune as at
from titan_gb300 import workloads as wl


@pytest.fixture
def timings(monkeypatch):
    calls = []
    table = {(4, 208, 448): 0.20, (4, 192, 448): 0.15, (1, 256, 256): 0.30}

    def fake_time(sc, precision, cand, steps, device):
        calls.append(tuple(cand))
        if tuple(cand) not in table:
            raise RuntimeError(f"candidate {cand} does not fit")
        return table[tuple(cand)], "warp-specialised" if cand[0] == 4 else "per-tile"

    monkeypatch.setattr(at, "_time_candidate", fake_time)
    monkeypatch.setattr(at, "_gpu_name", lambda device: "test-gpu")
    return calls


def test_fastest_candidate_is_chosen_and_cached(timings, tmp_path):
    sc = wl.actuated_lattice(n_side=10)
    cache = tmp_path / "tune.json"
    cands = [(4, 208, 448), (4, 192, 448), (3, 999, 256), (1, 256, 256)]
    best = at.autotune(sc, tg.FP32C, candidates=cands, cache_path=cache)
    assert (best["kernel"], best["tile"], best["threads"]) == (4, 192, 448)
    assert best["ms_per_step"] == pytest.approx(0.15)
    errors = [r for r in best["tried"] if "error" in r]
    assert len(errors) == 1 and errors[0]["candidate"] == [3, 999, 256]
    stored = json.loads(cache.read_text())
    assert stored[at.scene_key(sc, tg.FP32C)]["tile"] == 192
    n_calls = len(timings)
    again = at.autotune(sc, tg.FP32C, candidates=cands, cache_path=cache)  # from the cache
    assert again["tile"] == 192 and len(timings) == n_calls
    at.autotune(sc, tg.FP32C, candidates=cands, cache_path=cache, refresh=True)  # re-timed
    assert len(timings) == 2 * n_calls


def test_keys_separate_scenes_and_precisions(timings, tmp_path):
    a, b = wl.actuated_lattice(n_side=10), wl.actuated_lattice(n_side=12)
    assert at.scene_key(a, tg.FP32C) != at.scene_key(b, tg.FP32C)
    assert at.scene_key(a, tg.FP32C) != at.scene_key(a, tg.FP64)
    cache = tmp_path / "tune.json"
    at.autotune(a, tg.FP32C, candidates=[(4, 192, 448)], cache_path=cache)
    at.autotune(b, tg.FP32C, candidates=[(4, 208, 448)], cache_path=cache)
    stored = json.loads(cache.read_text())
    assert len(stored) == 2


def test_no_candidate_fits_raises(timings, tmp_path):
    with pytest.raises(RuntimeError, match="no launch configuration ran"):
        at.autotune(wl.actuated_lattice(n_side=8), tg.FP32C, candidates=[(2, 7, 7)], cache_path=tmp_path / "t.json")


def test_corrupt_cache_is_rebuilt(timings, tmp_path):
    cache = tmp_path / "tune.json"
    cache.write_text("{not json")
    best = at.autotune(wl.actuated_lattice(n_side=8), tg.FP32C, candidates=[(1, 256, 256)], cache_path=cache)
    assert best["kernel"] == 1 and json.loads(cache.read_text())
