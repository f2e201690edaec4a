"""Python binding of oracle/ref_gpu_harness.cpp: the reference's own CUDA
kernels (src/sim.cu:1046-1169, compiled from the reference sources into
oracle/_ref/titan_ref_kernels.cubin by oracle/build_ref.sh) stepping a scene
exactly as Simulation::execute() does.

TEST INFRASTRUCTURE ONLY: the GPU parity tests compare the engine with it
and bench.py times it beside the engine; nothing in the product imports it.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
CUBIN = HERE / "_ref" / "titan_ref_kernels.cubin"
HARNESS = HERE / "libref_gpu_harness.so"

_P = ctypes.c_void_p
_D = ctypes.POINTER(ctypes.c_double)
_I32 = ctypes.POINTER(ctypes.c_int32)
_U8 = ctypes.POINTER(ctypes.c_uint8)
_LIB = None


def available() -> str | None:
    """None when the reference kernels can run here, else the reason."""
    if not CUBIN.exists():
        return f"{CUBIN.name} not built (needs the reference sources at build time)"
    if not HARNESS.exists():
        return f"{HARNESS.name} not built"
    return None


def _lib():
    global _LIB
    if _LIB is None:
        L = ctypes.CDLL(str(HARNESS))
        L.refgpu_error.restype = ctypes.c_char_p
        L.refgpu_open.argtypes = [ctypes.c_char_p, ctypes.c_int]
        L.refgpu_setup.argtypes = [ctypes.c_int64, _D, _D, _D, _D, _U8, _D, ctypes.c_int64, _I32, _I32, _D, _D, _D,
                                   _I32, _D, ctypes.c_int, _D, ctypes.c_int, _D, _D, ctypes.c_double]
        L.refgpu_step.argtypes = [ctypes.c_int64, ctypes.c_int]
        L.refgpu_time_steps.argtypes = [ctypes.c_int64, ctypes.c_int]
        L.refgpu_time_steps.restype = ctypes.c_double
        L.refgpu_time.restype = ctypes.c_double
        L.refgpu_read.argtypes = [_D, _D, _D, _D]
        L.refgpu_sizes.argtypes = [ctypes.POINTER(ctypes.c_int64)]
        _LIB = L
    return _LIB


def _ptr(a, ct):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ct))


class RefGpuSim:
    """A scene in the reference's device layout (one per process)."""

    def __init__(self, sc: dict, device: int = 0):
        why = available()
        if why:
            raise RuntimeError(why)
        L = _lib()
        if L.refgpu_open(str(CUBIN).encode(), device):
            raise RuntimeError(L.refgpu_error().decode())
        f64 = lambda x: None if x is None else np.ascontiguousarray(x, np.float64)
        i32 = lambda x: None if x is None else np.ascontiguousarray(x, np.int32)
        self.n = int(np.asarray(sc["pos"]).shape[0])
        ns = int(np.asarray(sc["left"]).size)
        keep = dict(pos=f64(sc["pos"]), vel=f64(sc.get("vel")), m=f64(sc["m"]), ext=f64(sc.get("ext")),
                    fixed=None if sc.get("fixed") is None else np.ascontiguousarray(sc["fixed"], np.uint8),
                    drag=f64(sc.get("drag")), left=i32(sc["left"]), right=i32(sc["right"]), k=f64(sc["k"]),
                    rest=f64(sc["rest"]), damping=f64(sc.get("damping")), type=i32(sc.get("type")),
                    omega=f64(sc.get("omega")))
        planes = np.array([[*n, off, fk, fs] for n, off, fk, fs in sc["planes"]], np.float64).reshape(-1, 6)
        balls = np.array([[*c, r] for c, r in sc["balls"]], np.float64).reshape(-1, 4)
        g = np.ascontiguousarray(sc["g"], np.float64)
        rc = L.refgpu_setup(self.n, _ptr(keep["pos"], ctypes.c_double), _ptr(keep["vel"], ctypes.c_double),
                            _ptr(keep["m"], ctypes.c_double), _ptr(keep["ext"], ctypes.c_double),
                            _ptr(keep["fixed"], ctypes.c_uint8), _ptr(keep["drag"], ctypes.c_double), ns,
                            _ptr(keep["left"], ctypes.c_int32), _ptr(keep["right"], ctypes.c_int32),
                            _ptr(keep["k"], ctypes.c_double), _ptr(keep["rest"], ctypes.c_double),
                            _ptr(keep["damping"], ctypes.c_double), _ptr(keep["type"], ctypes.c_int32),
                            _ptr(keep["omega"], ctypes.c_double), len(planes), _ptr(planes, ctypes.c_double),
                            len(balls), _ptr(balls, ctypes.c_double), _ptr(g, ctypes.c_double), float(sc["dt"]))
        if rc:
            raise RuntimeError(L.refgpu_error().decode())

    def step(self, nsteps: int, sync_each: bool = False):
        if _lib().refgpu_step(nsteps, int(sync_each)):
            raise RuntimeError(_lib().refgpu_error().decode())

    def time_steps(self, nsteps: int, sync_each: bool = False) -> float:
        """Milliseconds for nsteps steps (CUDA events, default stream)."""
        ms = _lib().refgpu_time_steps(nsteps, int(sync_each))
        if ms < 0:
            raise RuntimeError(_lib().refgpu_error().decode())
        return ms

    @property
    def time(self) -> float:
        return _lib().refgpu_time()

    def state(self) -> dict:
        pos, vel, acc = (np.zeros((self.n, 3)) for _ in range(3))
        T = np.zeros(self.n)
        if _lib().refgpu_read(_ptr(pos, ctypes.c_double), _ptr(vel, ctypes.c_double), _ptr(acc, ctypes.c_double),
                              _ptr(T, ctypes.c_double)):
            raise RuntimeError(_lib().refgpu_error().decode())
        return {"pos": pos, "vel": vel, "acc": acc, "T": T}

    def close(self):
        _lib().refgpu_close()
