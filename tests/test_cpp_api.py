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
    assert set(r.stdout.split()) == set(TESTS) | set(CPU_TESTS)


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
