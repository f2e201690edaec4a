"""Build recipe for the in-tree native libraries (no cmake, no setuptools).

    python -m titan_gb300.build            # product library + oracle (+ reference pieces)

Products:
    titan_gb300/libtitan_gb300.so   C ABI of include/titan_gb300.h (sm_103a kernels)
    titan_gb300/libtitan_sim.so     C++ titan::Simulation drop-in over that C ABI
    oracle/libtitan_oracle.so       CPU oracle (test infrastructure only)
    oracle/_ref/...                 reference host code, when its sources are present

All host code is compiled with -ffp-contract=off so that x86_64 and aarch64
hosts round identically.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "titan_gb300"
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
ORACLE = ROOT / "oracle"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: every kernel rounds each product and sum separately, as the
# CPU oracle does (FP64 parity), and the two step-kernel forms stay
# bit-identical in every precision; explicit fmaf() calls are unaffected.
NVCC_COMMON = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
               "-I", str(ROOT / "include"), "-I", str(CSRC)]
NVCC_KERNEL_EXTRA: dict[str, list[str]] = {}
CXX_COMMON = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra",
              "-I", str(ROOT / "include"), "-I", str(CSRC)]

LIB_CU = sorted(p.name for p in CSRC.glob("*.cu"))
LIB_CPP = ["plan.cpp", "lattice.cpp"]
SIM_CPP = ["simulation.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def _headers() -> list[Path]:
    return list(CSRC.glob("*.h")) + list((ROOT / "include").rglob("*.h"))


def build_library(verbose: bool = False) -> Path:
    """Compile and link libtitan_gb300.so and libtitan_sim.so; returns the first."""
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    objs = []
    hdrs = _headers()
    # a change of compiler flags invalidates every object
    sig = BUILD / "flags.txt"
    flags = " ".join(ARCH + NVCC_COMMON + CXX_COMMON)
    if not sig.exists() or sig.read_text() != flags:
        for o in BUILD.glob("*.o"):
            o.unlink()
        sig.write_text(flags)
    for f in LIB_CU:
        src, obj = CSRC / f, BUILD / (f + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            jobs.append([nvcc, *ARCH, *NVCC_COMMON, *NVCC_KERNEL_EXTRA.get(f, []), "-c", str(src), "-o", str(obj)])
    for f in LIB_CPP + SIM_CPP:
        src, obj = CSRC / f, BUILD / (f + ".o")
        if f in LIB_CPP:
            objs.append(obj)
        if _stale(obj, [src] + hdrs):
            jobs.append(["g++", *CXX_COMMON, "-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    lib = PKG / "libtitan_gb300.so"
    if jobs or not lib.exists():
        _run([nvcc, *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-lcudart"])
    sim = PKG / "libtitan_sim.so"
    sim_objs = [BUILD / (f + ".o") for f in SIM_CPP]
    if jobs or not sim.exists():
        _run(["g++", "-shared", "-o", str(sim), *map(str, sim_objs), "-L", str(PKG), "-ltitan_gb300",
              "-Wl,-rpath,$ORIGIN", "-lpthread"])
    if verbose:
        print("built", lib, sim)
    return lib


def build_oracle(verbose: bool = False) -> Path:
    """Compile the CPU oracle (plain C, OpenMP)."""
    src = ORACLE / "titan_oracle.c"
    out = ORACLE / "libtitan_oracle.so"
    if _stale(out, [src, ORACLE / "titan_oracle.h"]):
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-Wall",
              str(src), "-o", str(out), "-lm"])
    if verbose:
        print("built", out)
    return out


def build_reference_pieces(verbose: bool = False) -> Path | None:
    """Compile the reference's host-callable code into oracle/_ref (only where
    the reference sources exist; the recipe, oracle/build_ref.sh, locates
    them and exits with status 3 when they are absent)."""
    script = ORACLE / "build_ref.sh"
    if not script.exists():
        return None
    out = ORACLE / "_ref" / "libtitan_ref_host.so"
    deps = [script, ORACLE / "ref_host_shim.cu", ORACLE / "ref_gpu_shim.cu", *(ORACLE / "ref_shims").glob("*.h")]
    if not _stale(out, deps) and not _stale(ORACLE / "_ref" / "titan_ref_kernels.cubin", deps):
        return out
    r = subprocess.run(["bash", str(script)], capture_output=True, text=True)
    if r.returncode == 3:  # no reference sources on this machine: the prebuilt pieces (if any) serve
        return out if out.exists() else None
    if r.returncode != 0:
        if verbose:
            print("reference pieces not built:", r.stderr[-2000:])
        return None
    out = ORACLE / "_ref" / "libtitan_ref_host.so"
    return out if out.exists() else None


def build_ref_gpu_harness(verbose: bool = False) -> Path:
    """Compile the driver-API harness that runs the reference's own kernels
    from oracle/_ref/titan_ref_kernels.cubin (test infrastructure only; needs
    no reference file, so it builds wherever the CUDA toolkit is)."""
    src = ORACLE / "ref_gpu_harness.cpp"
    out = ORACLE / "libref_gpu_harness.so"
    cuda = Path(_nvcc()).resolve().parent.parent
    if _stale(out, [src]):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-Wall", "-I", str(cuda / "include"), str(src),
              "-o", str(out), "-L", str(cuda / "lib64"), "-L", str(cuda / "lib64" / "stubs"), "-lcuda"])
    if verbose:
        print("built", out)
    return out


def build_all(verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=4) as ex:
        futs = [ex.submit(build_library, verbose), ex.submit(build_oracle, verbose),
                ex.submit(build_reference_pieces, verbose), ex.submit(build_ref_gpu_harness, verbose)]
        for f in futs:
            f.result()


if __name__ == "__main__":
    build_all(verbose=True)
    sys.exit(0)
