"""The C++ drop-in: the reference's physics tests, written against
<Titan/sim.h>, compiled against this repository's headers and library.

Compiling needs no GPU (checks that user code written for the reference API
builds unchanged, with the reference's -Wall -Wextra -Werror, test/CMakeLists.txt:17);
running the physics tests needs one.  The misuse conventions before start()
touch no device and run on the CPU."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "cpp" / "reference_physics.cpp"
OUT = ROOT / "tests" / "cpp" / "_build" / "reference_physics"
PKG = ROOT / "titan_gb300"

TESTS = ["simple_test", "energy_test", "external_test", "external_acc_test", "multiagent_test", "rotate_test",
         "breakpoint_and_step_test", "beam_fixed_face_test", "topology_edit_test", "stl_import_test"]
DUMP_TESTS = ["delete_after_start_test"]
CPU_TESTS = ["errors_test"]


def compile_tests():
    OUT.parent.mkdir(parents=True, exist_ok=True)
    if OUT.exists() and OUT.stat().st_mtime > max(SRC.stat().st_mtime, (PKG / "libtitan_sim.so").stat().st_mtime):
        return OUT
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"), str(SRC),
           "-o", str(OUT), "-L", str(PKG), "-ltitan_sim", "-ltitan_gb300", f"-Wl,-rpath,{PKG}", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return OUT


def test_reference_tests_compile_against_dropin_headers():
    exe = compile_tests()
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0
    assert set(r.stdout.split()) == set(TESTS) | set(CPU_TESTS) | set(DUMP_TESTS)


@pytest.mark.parametrize("name", CPU_TESTS)
def test_misuse_before_start(name):
    exe = compile_tests()
    r = subprocess.run([str(exe), name], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "cannot be called before sim.start()" in r.stderr      # get(Mass*) before start
    assert "does nothing if called before the simulation has started" in r.stderr  # get(Container*)


@pytest.mark.gpu
@pytest.mark.parametrize("name", TESTS)
def test_reference_physics(name):
    exe = compile_tests()
    r = subprocess.run([str(exe), name], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]


@pytest.mark.gpu
def test_delete_after_start_matches_oracle(tmp_path):
    """deleteSpring / deleteMass / deleteContainer while paused, through the
    C++ drop-in, bit for bit against the oracle running the same deletions
    (a deleted spring, and every spring of a deleted mass, is skipped; a
    deleted mass is no longer stepped)."""
    import numpy as np

    from oracle import pyoracle as po

    exe = compile_tests()
    out = tmp_path / "state.bin"
    r = subprocess.run([str(exe), "delete_after_start_test", str(out)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    raw = out.read_bytes()
    n1, n2, nm = np.frombuffer(raw[:24], np.int64)
    got = np.frombuffer(raw[24:], np.float64).reshape(nm, 6)
    # the same scene for the oracle: createLattice twice (mass 0.1, k 1e4,
    # rest = initial length), a frictional plane
    pa, la, ra, sa = po.lattice((0, 0, 0.6), (1, 1, 1), 6, 6, 6)
    pb, lb, rb, sb = po.lattice((3, 0, 0.6), (1, 1, 1), 4, 4, 4)
    na = pa.shape[0]
    pos = np.concatenate([pa, pb])
    left = np.concatenate([la, lb + na]).astype(np.int32)
    right = np.concatenate([ra, rb + na]).astype(np.int32)
    rest = np.concatenate([sa, sb])
    n, ns = pos.shape[0], left.size
    sc = {"pos": pos, "vel": np.zeros_like(pos), "m": np.full(n, 0.1), "left": left, "right": right,
          "k": np.full(ns, 1e4), "rest": rest, "damping": np.zeros(ns), "type": np.zeros(ns, np.int32),
          "omega": np.zeros(ns), "amp": np.full(ns, 0.2), "phase": np.zeros(ns),
          "planes": [((0.0, 0.0, 1.0), 0.0, 0.5, 0.5)], "balls": [], "g": np.array([0.0, 0.0, -9.81]),
          "dt": 1e-4, "fixed": np.zeros(n, np.uint8)}
    o = po.OracleSim(sc)
    o.step(int(n1))
    gone_springs = [0, 7, 100, 333] + list(range(la.size, ns))
    gone_masses = [40] + list(range(na, n))
    o._keep["left"][gone_springs] = -1
    o._keep["right"][gone_springs] = -1
    for m in gone_masses:
        o._keep["left"][o._keep["left"] == m] = -1
        o._keep["right"][o._keep["right"] == m] = -1
    o._keep["fixed"][gone_masses] = 1
    o.step(int(n2))
    keep = np.setdiff1d(np.arange(n), gone_masses)
    assert nm == keep.size
    assert np.array_equal(got[:, :3], o.pos[keep]), np.max(np.abs(got[:, :3] - o.pos[keep]))
    assert np.array_equal(got[:, 3:], o.vel[keep]), np.max(np.abs(got[:, 3:] - o.vel[keep]))
    assert np.min(o.pos[keep, 2]) < 0.05  # the bottom face (at 0.1 m at the start) came down to the plane
