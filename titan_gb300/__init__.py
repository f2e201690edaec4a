"""titan_gb300 -- GB300-native engine for Titan's mass-spring time step.

Python host wrapper over the C ABI declared in include/titan_gb300.h (the
library libtitan_gb300.so built in-tree by titan_gb300.build).  There is no
CPU fallback: when the native library is missing, every entry point raises.

The method names follow titan::Simulation (include/Titan/sim.h:37-220 in the
reference): set_masses/set_springs stand for createMass/createSpring over whole
arrays, add_plane/add_ball for createPlane/createBall, start/step for start()
and the execute() loop body, get_state/set_mass_state for getAll()/setAll().
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

__all__ = ["FP64", "FP32", "FP32C", "TitanError", "Sim", "Server", "lattice", "lattice_springs", "lib",
           "pinned_empty", "library_path"]

FP64, FP32, FP32C = 0, 1, 2
EULER, VERLET, RK2 = 0, 1, 2
PRECISION_NAMES = {FP64: "f64", FP32: "f32", FP32C: "f32c"}

_ERRORS = {1: "EINVAL", 2: "ECUDA", 3: "ENOMEM", 4: "ELIMIT", 5: "ESTATE", 6: "ETIMEOUT", 7: "EBUDGET", 8: "EBUSY"}

_LIB = None


class TitanError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_ERRORS.get(code, code)}: {msg}")
        self.code = code


def library_path() -> Path:
    return Path(__file__).resolve().with_name("libtitan_gb300.so")


_P = ctypes.c_void_p
_D = ctypes.POINTER(ctypes.c_double)
_I32 = ctypes.POINTER(ctypes.c_int32)
_I64 = ctypes.POINTER(ctypes.c_int64)
_U8 = ctypes.POINTER(ctypes.c_uint8)

_SIGS = {
    "titan_gb300_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int, ctypes.c_int]),
    "titan_gb300_destroy": (None, [_P]),
    "titan_gb300_last_error": (ctypes.c_char_p, [_P]),
    "titan_gb300_set_masses": (ctypes.c_int, [_P, ctypes.c_int64, _D, _D, _D, _D, _U8, _D]),
    "titan_gb300_set_springs": (ctypes.c_int, [_P, ctypes.c_int64, _I32, _I32, _D, _D, _D, _I32, _D, _D, _D]),
    "titan_gb300_set_local_constraints": (ctypes.c_int, [_P, _I64, _I32, _D, _D]),
    "titan_gb300_add_plane": (ctypes.c_int, [_P, _D, ctypes.c_double, ctypes.c_double, ctypes.c_double]),
    "titan_gb300_add_ball": (ctypes.c_int, [_P, _D, ctypes.c_double]),
    "titan_gb300_clear_constraints": (ctypes.c_int, [_P]),
    "titan_gb300_set_time_step": (ctypes.c_int, [_P, ctypes.c_double]),
    "titan_gb300_set_integrator": (ctypes.c_int, [_P, ctypes.c_int]),
    "titan_gb300_get_time_step": (ctypes.c_double, [_P]),
    "titan_gb300_set_global_acc": (ctypes.c_int, [_P, _D]),
    "titan_gb300_set_bodies": (ctypes.c_int, [_P, ctypes.c_int64, _I64]),
    "titan_gb300_set_body_plane": (ctypes.c_int, [_P, ctypes.c_int64, _D, ctypes.c_double, ctypes.c_double,
                                                  ctypes.c_double]),
    "titan_gb300_start": (ctypes.c_int, [_P, ctypes.c_int]),
    "titan_gb300_adopt_plan": (ctypes.c_int, [_P, _P]),
    "titan_gb300_plan_host": (ctypes.c_int, [_P, ctypes.c_int]),
    "titan_gb300_set_launch": (ctypes.c_int, [_P, ctypes.c_int]),
    "titan_gb300_set_kernel": (ctypes.c_int, [_P, ctypes.c_int]),
    "titan_gb300_set_occupancy": (ctypes.c_int, [_P, ctypes.c_int]),
    "titan_gb300_kernel_info": (ctypes.c_int, [_P, _I64]),
    "titan_gb300_set_resident": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "titan_gb300_resident_info": (ctypes.c_int, [_P, _I64]),
    "titan_gb300_step": (ctypes.c_int, [_P, ctypes.c_int64]),
    "titan_gb300_prepare_steps": (ctypes.c_int, [_P, ctypes.c_int64]),
    "titan_gb300_synchronize": (ctypes.c_int, [_P]),
    "titan_gb300_poll": (ctypes.c_int, [_P]),
    "titan_gb300_wait": (ctypes.c_int, [_P, ctypes.c_double]),
    "titan_gb300_export_vertices": (ctypes.c_int, [_P, ctypes.c_void_p, ctypes.c_int]),
    "titan_gb300_export_indices": (ctypes.c_int, [_P, ctypes.c_void_p, ctypes.c_int]),
    "titan_gb300_time": (ctypes.c_double, [_P]),
    "titan_gb300_set_time": (ctypes.c_int, [_P, ctypes.c_double]),
    "titan_gb300_device_bytes": (ctypes.c_int64, [_P]),
    "titan_gb300_host_alloc": (ctypes.c_void_p, [ctypes.c_size_t]),
    "titan_gb300_host_free": (None, [ctypes.c_void_p]),
    "titan_gb300_steps": (ctypes.c_int64, [_P]),
    "titan_gb300_get_state": (ctypes.c_int, [_P, _D, _D, _D, _D]),
    "titan_gb300_get_masses": (ctypes.c_int, [_P, ctypes.c_int64, _I64, _D, _D, _D, _D]),
    "titan_gb300_set_mass_state": (ctypes.c_int, [_P, ctypes.c_int64, _I64, _D, _D, _D, _D, _U8, _D, _D]),
    "titan_gb300_set_spring_params": (ctypes.c_int, [_P, ctypes.c_int64, _I64, _D, _D, _D, _I32, _D, _D, _D]),
    "titan_gb300_diagnostics": (ctypes.c_int, [_P, ctypes.c_double, _D, _D]),
    "titan_gb300_stream": (ctypes.c_void_p, [_P]),
    "titan_gb300_plan_info": (ctypes.c_int, [_P, _I64]),
    "titan_gb300_lattice_springs": (ctypes.c_int64, [ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "titan_gb300_lattice": (ctypes.c_int, [_D, _D, ctypes.c_int, ctypes.c_int, ctypes.c_int, _D, _I32, _I32, _D]),
    "titan_gb300_version": (ctypes.c_char_p, []),
    "titan_gb300_server_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                 ctypes.c_int64]),
    "titan_gb300_server_submit": (ctypes.c_int, [_P, _P, ctypes.c_int64, _I64]),
    "titan_gb300_server_poll": (ctypes.c_int, [_P, ctypes.c_int64]),
    "titan_gb300_server_info": (ctypes.c_int, [_P, _I64]),
    "titan_gb300_server_last_error": (ctypes.c_char_p, [_P]),
    "titan_gb300_server_destroy": (None, [_P]),
    "titan_gb300_stl_inside": (ctypes.c_int, [ctypes.c_int, _D, ctypes.c_int64, _D, ctypes.c_int64, ctypes.c_int,
                                              ctypes.c_uint64, _U8]),
}


def lib() -> ctypes.CDLL:
    """Load libtitan_gb300.so (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        path = library_path()
        if not path.exists():
            raise RuntimeError(f"native library {path} is missing: run `python -m titan_gb300.build`")
        L = ctypes.CDLL(str(path))
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def _ptr(a, ctype):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def _f64(a, shape_len=None):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape_len is not None and a.size != shape_len:
        raise ValueError(f"expected {shape_len} values, got {a.size}")
    return a


def _i32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.int32)


def _i64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.int64)


def _u8(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.uint8)


class _PinnedBlock:
    """Page-locked host memory (titan_gb300_host_alloc), freed with the last
    array that views it."""

    def __init__(self, shape, dtype):
        self.dtype = np.dtype(dtype)
        self.shape = tuple(int(x) for x in shape)
        nbytes = int(np.prod(self.shape, dtype=np.int64)) * self.dtype.itemsize
        self.ptr = lib().titan_gb300_host_alloc(max(nbytes, 1))
        if not self.ptr:
            raise MemoryError(f"page-locked host allocation of {nbytes} bytes failed")
        self.__array_interface__ = {"data": (self.ptr, False), "shape": self.shape, "typestr": self.dtype.str,
                                    "version": 3}

    def __del__(self):
        if getattr(self, "ptr", None):
            lib().titan_gb300_host_free(self.ptr)
            self.ptr = None


def pinned_empty(shape, dtype=np.float64) -> np.ndarray:
    """An uninitialised array in page-locked host memory: get_state /
    set_mass_state move it by DMA directly (no staging copy)."""
    return np.asarray(_PinnedBlock(shape, dtype))


def lattice_springs(nx: int, ny: int, nz: int) -> int:
    return int(lib().titan_gb300_lattice_springs(nx, ny, nz))


def lattice(center, dims, nx: int, ny: int, nz: int):
    """createLattice geometry: (pos[n,3], left, right, rest) in the reference's order."""
    n = nx * ny * nz
    ns = lattice_springs(nx, ny, nz)
    pos = np.zeros((n, 3))
    left = np.zeros(ns, np.int32)
    right = np.zeros(ns, np.int32)
    rest = np.zeros(ns)
    c = _f64(center, 3)
    d = _f64(dims, 3)
    rc = lib().titan_gb300_lattice(_ptr(c, ctypes.c_double), _ptr(d, ctypes.c_double), nx, ny, nz,
                                   _ptr(pos, ctypes.c_double), _ptr(left, ctypes.c_int32),
                                   _ptr(right, ctypes.c_int32), _ptr(rest, ctypes.c_double))
    if rc:
        raise TitanError(rc, "lattice")
    return pos, left, right, rest


class Sim:
    """One simulation handle (one CUDA stream, one GPU)."""

    def __init__(self, precision: int = FP64, device: int = 0):
        self._L = lib()
        h = _P()
        rc = self._L.titan_gb300_create(ctypes.byref(h), device, precision)
        if rc:
            raise TitanError(rc, "create (is a CUDA device available?)")
        self._h = h
        self.precision = precision
        self.n = 0
        self.ns = 0
        self._keep = []

    # -- plumbing --
    def _check(self, rc: int, what: str):
        if rc:
            msg = self._L.titan_gb300_last_error(self._h)
            raise TitanError(rc, f"{what}: {msg.decode() if msg else ''}")

    def close(self):
        if getattr(self, "_h", None):
            self._L.titan_gb300_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- scene --
    def set_masses(self, pos, m, vel=None, ext=None, fixed=None, drag=None):
        pos = _f64(pos)
        n = pos.size // 3
        m = _f64(m, n)
        vel, ext, drag = _f64(vel, 3 * n if vel is not None else None), _f64(ext), _f64(drag)
        fixed = _u8(fixed)
        self._check(self._L.titan_gb300_set_masses(self._h, n, _ptr(pos, ctypes.c_double), _ptr(vel, ctypes.c_double),
                                                   _ptr(m, ctypes.c_double), _ptr(ext, ctypes.c_double),
                                                   _ptr(fixed, ctypes.c_uint8), _ptr(drag, ctypes.c_double)),
                    "set_masses")
        self.n = n

    def set_springs(self, left, right, k, rest, damping=None, type=None, omega=None, amp=None, phase=None):
        left, right = _i32(left), _i32(right)
        ns = left.size
        k, rest = _f64(k, ns), _f64(rest, ns)
        damping, omega, amp, phase = (_f64(x, ns) if x is not None else None for x in (damping, omega, amp, phase))
        type = _i32(type)
        self._check(self._L.titan_gb300_set_springs(
            self._h, ns, _ptr(left, ctypes.c_int32), _ptr(right, ctypes.c_int32), _ptr(k, ctypes.c_double),
            _ptr(rest, ctypes.c_double), _ptr(damping, ctypes.c_double), _ptr(type, ctypes.c_int32),
            _ptr(omega, ctypes.c_double), _ptr(amp, ctypes.c_double), _ptr(phase, ctypes.c_double)), "set_springs")
        self.ns = ns

    def set_local_constraints(self, mass_ptr, type, vec, num):
        mass_ptr, type, vec, num = _i64(mass_ptr), _i32(type), _f64(vec), _f64(num)
        self._check(self._L.titan_gb300_set_local_constraints(self._h, _ptr(mass_ptr, ctypes.c_int64),
                                                              _ptr(type, ctypes.c_int32), _ptr(vec, ctypes.c_double),
                                                              _ptr(num, ctypes.c_double)), "set_local_constraints")

    def add_plane(self, normal, offset, friction_k=0.0, friction_s=0.0):
        n = _f64(normal, 3)
        self._check(self._L.titan_gb300_add_plane(self._h, _ptr(n, ctypes.c_double), offset, friction_k, friction_s),
                    "add_plane")

    def add_ball(self, center, radius):
        c = _f64(center, 3)
        self._check(self._L.titan_gb300_add_ball(self._h, _ptr(c, ctypes.c_double), radius), "add_ball")

    def clear_constraints(self):
        self._check(self._L.titan_gb300_clear_constraints(self._h), "clear_constraints")

    def set_time(self, T: float):
        """Set the simulation clock (the time actuation sees)."""
        self._check(self._L.titan_gb300_set_time(self._h, float(T)), "set_time")

    def device_bytes(self) -> int:
        return int(self._L.titan_gb300_device_bytes(self._h))

    def set_integrator(self, kind: int):
        """0 symplectic Euler (default), 1 Verlet, 2 RK2."""
        self._check(self._L.titan_gb300_set_integrator(self._h, int(kind)), "set_integrator")

    def set_time_step(self, dt):
        self._check(self._L.titan_gb300_set_time_step(self._h, dt), "set_time_step")

    def get_time_step(self) -> float:
        return float(self._L.titan_gb300_get_time_step(self._h))

    def set_global_acc(self, g):
        g = _f64(g, 3)
        self._check(self._L.titan_gb300_set_global_acc(self._h, _ptr(g, ctypes.c_double)), "set_global_acc")

    def set_bodies(self, mass_ptr):
        mass_ptr = _i64(mass_ptr)
        self._check(self._L.titan_gb300_set_bodies(self._h, mass_ptr.size - 1, _ptr(mass_ptr, ctypes.c_int64)),
                    "set_bodies")

    def set_body_plane(self, body, normal, offset, friction_k=0.0, friction_s=0.0):
        n = _f64(normal, 3)
        self._check(self._L.titan_gb300_set_body_plane(self._h, body, _ptr(n, ctypes.c_double), offset, friction_k,
                                                       friction_s), "set_body_plane")

    # -- device --
    def set_launch(self, threads_per_cta: int):
        self._check(self._L.titan_gb300_set_launch(self._h, threads_per_cta), "set_launch")

    def set_occupancy(self, min_ctas_per_sm: int):
        """Register cap of the per-tile kernel (FP32 forms): 0 none, 3 or 4
        resident CTAs per SM (at most 256 threads per CTA)."""
        self._check(self._L.titan_gb300_set_occupancy(self._h, min_ctas_per_sm), "set_occupancy")

    def set_kernel(self, variant: int):
        """0 automatic, 1 per-tile kernel, 3 per-tile kernel with asynchronous
        (bulk-copy) staging, 4 warp-specialised persistent kernel (producer
        warp + consumer warps, stage ring of slabs), 6 pull kernel (FP32 and
        FP32C: every mass sums its own springs' forces from streamed spring
        columns against tile states staged by a producer warp)."""
        self._check(self._L.titan_gb300_set_kernel(self._h, variant), "set_kernel")

    def kernel_info(self) -> dict:
        out = np.zeros(4, np.int64)
        self._check(self._L.titan_gb300_kernel_info(self._h, _ptr(out, ctypes.c_int64)), "kernel_info")
        names = {1: "per-tile", 3: "per-tile-async", 4: "warp-specialised", 5: "resident-tiles", 6: "pull"}
        return {"kernel": names.get(int(out[0]), "per-tile"), "ctas": int(out[1]), "threads": int(out[2]),
                "smem_bytes": int(out[3])}

    def set_resident(self, mode: int = 1, bin_masses: int = 0, threads: int = 0):
        """Resident launches (all steps of a call in one kernel): mode -1
        automatic (the default: the halo-free tiles, when the kernel form
        is automatic), 0 off, 1 bins of whole bodies (one
        thread per mass), 2 halo-free tiles (the per-step kernels' two
        phases in shared memory); bin capacity in masses (mode 1) and CTA
        size (0: default)."""
        self._check(self._L.titan_gb300_set_resident(self._h, mode, bin_masses, threads), "set_resident")

    def resident_info(self) -> dict:
        out = np.zeros(8, np.int64)
        self._check(self._L.titan_gb300_resident_info(self._h, _ptr(out, ctypes.c_int64)), "resident_info")
        keys = ("active", "bins", "bodies", "masses", "cap", "threads", "ctas", "smem_bytes")
        return {k: int(v) for k, v in zip(keys, out)}

    def plan_host(self, tile_masses: int = 0):
        """Build the tile plan on the host only (no GPU needed)."""
        self._check(self._L.titan_gb300_plan_host(self._h, tile_masses), "plan_host")

    def adopt_plan(self, src: "Sim"):
        """Use src's plan (same topology) for the next start()."""
        self._check(self._L.titan_gb300_adopt_plan(self._h, src._h), "adopt_plan")

    def start(self, tile_masses: int = 0):
        self._check(self._L.titan_gb300_start(self._h, tile_masses), "start")

    def step(self, nsteps: int = 1):
        self._check(self._L.titan_gb300_step(self._h, nsteps), "step")

    def prepare_steps(self, nsteps: int):
        """Build the CUDA graphs a later step(nsteps) replays, launching nothing."""
        self._check(self._L.titan_gb300_prepare_steps(self._h, nsteps), "prepare_steps")

    def poll(self) -> bool:
        """True when every queued step has finished."""
        rc = self._L.titan_gb300_poll(self._h)
        if rc == 8:  # TITAN_GB300_EBUSY
            return False
        self._check(rc, "poll")
        return True

    def wait(self, timeout_ms: float) -> bool:
        """Block up to timeout_ms; False when the steps are still running."""
        rc = self._L.titan_gb300_wait(self._h, float(timeout_ms))
        if rc == 6:  # TITAN_GB300_ETIMEOUT
            return False
        self._check(rc, "wait")
        return True

    def export_vertices(self, out=None, device_ptr: int = 0):
        """float32 positions (n, 3) in creation order; with device_ptr, written
        to that device address asynchronously instead."""
        if device_ptr:
            self._check(self._L.titan_gb300_export_vertices(self._h, ctypes.c_void_p(device_ptr), 1),
                        "export_vertices")
            return None
        if out is None:
            out = np.empty((self.n, 3), np.float32)
        self._check(self._L.titan_gb300_export_vertices(self._h, out.ctypes.data_as(ctypes.c_void_p), 0),
                    "export_vertices")
        return out

    def export_indices(self, device_ptr: int = 0):
        """uint32 (ns, 2) left/right mass index of each spring ((0, 0) if detached)."""
        if device_ptr:
            self._check(self._L.titan_gb300_export_indices(self._h, ctypes.c_void_p(device_ptr), 1),
                        "export_indices")
            return None
        out = np.empty((self.ns, 2), np.uint32)
        self._check(self._L.titan_gb300_export_indices(self._h, out.ctypes.data_as(ctypes.c_void_p), 0),
                    "export_indices")
        return out

    def synchronize(self):
        self._check(self._L.titan_gb300_synchronize(self._h), "synchronize")

    @property
    def time(self) -> float:
        return float(self._L.titan_gb300_time(self._h))

    @property
    def steps(self) -> int:
        return int(self._L.titan_gb300_steps(self._h))

    @property
    def stream(self) -> int:
        return int(self._L.titan_gb300_stream(self._h) or 0)

    def get_state(self, pos=True, vel=True, acc=False, T=False, out=None):
        n = self.n
        res = out if out is not None else {}
        arrs = {}
        for key, want, shape in (("pos", pos, (n, 3)), ("vel", vel, (n, 3)), ("acc", acc, (n, 3)), ("T", T, (n,))):
            if want:
                a = res.get(key)
                if a is None or a.shape != shape:
                    a = np.empty(shape)
                arrs[key] = a
        self._check(self._L.titan_gb300_get_state(self._h, *(_ptr(arrs.get(k), ctypes.c_double)
                                                             for k in ("pos", "vel", "acc", "T"))), "get_state")
        res.update(arrs)
        return res

    def get_masses(self, idx, pos=True, vel=True, acc=False, T=False):
        idx = _i64(idx)
        c = idx.size
        arrs = {k: np.empty((c, 3)) for k, w in (("pos", pos), ("vel", vel), ("acc", acc)) if w}
        if T:
            arrs["T"] = np.empty(c)
        self._check(self._L.titan_gb300_get_masses(self._h, c, _ptr(idx, ctypes.c_int64),
                                                   *(_ptr(arrs.get(k), ctypes.c_double)
                                                     for k in ("pos", "vel", "acc", "T"))), "get_masses")
        return arrs

    def set_mass_state(self, idx=None, pos=None, vel=None, m=None, ext=None, fixed=None, drag=None, T=None):
        idx = _i64(idx)
        count = idx.size if idx is not None else self.n
        pos, vel, m, ext, drag, T = (_f64(x) for x in (pos, vel, m, ext, drag, T))
        fixed = _u8(fixed)
        self._check(self._L.titan_gb300_set_mass_state(
            self._h, count, _ptr(idx, ctypes.c_int64), _ptr(pos, ctypes.c_double), _ptr(vel, ctypes.c_double),
            _ptr(m, ctypes.c_double), _ptr(ext, ctypes.c_double), _ptr(fixed, ctypes.c_uint8),
            _ptr(drag, ctypes.c_double), _ptr(T, ctypes.c_double)), "set_mass_state")

    def set_spring_params(self, idx=None, k=None, rest=None, damping=None, type=None, omega=None, amp=None,
                          phase=None):
        idx = _i64(idx)
        count = idx.size if idx is not None else self.ns
        k, rest, damping, omega, amp, phase = (_f64(x) for x in (k, rest, damping, omega, amp, phase))
        type = _i32(type)
        self._check(self._L.titan_gb300_set_spring_params(
            self._h, count, _ptr(idx, ctypes.c_int64), _ptr(k, ctypes.c_double), _ptr(rest, ctypes.c_double),
            _ptr(damping, ctypes.c_double), _ptr(type, ctypes.c_int32), _ptr(omega, ctypes.c_double),
            _ptr(amp, ctypes.c_double), _ptr(phase, ctypes.c_double)), "set_spring_params")

    def diagnostics(self, g_mag: float = 9.81):
        e = np.zeros(4)
        p = np.zeros(6)
        self._check(self._L.titan_gb300_diagnostics(self._h, g_mag, _ptr(e, ctypes.c_double),
                                                    _ptr(p, ctypes.c_double)), "diagnostics")
        return {"spring_pe": e[0], "kinetic": e[1], "gravity_pe": e[2], "total": e[3],
                "linear": p[:3].copy(), "angular": p[3:].copy()}

    def plan_info(self) -> dict:
        out = np.zeros(12, np.int64)
        self._check(self._L.titan_gb300_plan_info(self._h, _ptr(out, ctypes.c_int64)), "plan_info")
        keys = ["masses", "springs", "tiles", "entries", "halo", "inc_words", "heavy", "smem_bytes", "threads",
                "algorithmic_bytes_per_step", "implementation_bytes_per_step", "actuated_entries"]
        return {k: int(v) for k, v in zip(keys, out)}


class Server:
    """Device-resident request server (titan_gb300_server_*): one persistent
    kernel steps every submitted Sim (started, symplectic Euler, resident
    tiles and bins off: set_resident(0)) until its steps are done; each
    result is bit-identical to the Sim's own step()."""

    def __init__(self, precision: int = FP32C, device: int = 0, max_slots: int = 4096, tile_smem_bytes: int = 0):
        self._L = lib()
        h = _P()
        rc = self._L.titan_gb300_server_create(ctypes.byref(h), device, precision, max_slots, tile_smem_bytes)
        if rc:
            raise TitanError(rc, "server_create")
        self._h = h
        self.precision = precision
        self.max_slots = max_slots

    def _check(self, rc, what):
        if rc:
            msg = self._L.titan_gb300_server_last_error(self._h)
            raise TitanError(rc, f"{what}: {msg.decode() if msg else ''}")

    def submit(self, sim: "Sim", nsteps: int):
        """Queue nsteps steps of sim; returns a ticket, or None when no slot is free."""
        t = ctypes.c_int64(0)
        rc = self._L.titan_gb300_server_submit(self._h, sim._h, int(nsteps), ctypes.byref(t))
        if rc == 8:  # TITAN_GB300_EBUSY
            return None
        self._check(rc, "server_submit")
        return int(t.value)

    def poll(self, ticket: int) -> bool:
        """True once the request is done (its Sim is usable again)."""
        rc = self._L.titan_gb300_server_poll(self._h, int(ticket))
        if rc == 8:
            return False
        self._check(rc, "server_poll")
        return True

    def wait(self, ticket: int, timeout_s: float = 600.0, sleep_s: float = 50e-6) -> None:
        import time
        t0 = time.perf_counter()
        while not self.poll(ticket):
            if time.perf_counter() - t0 > timeout_s:
                raise TitanError(6, f"request {ticket} not done after {timeout_s} s")
            time.sleep(sleep_s)

    def info(self) -> dict:
        out = np.zeros(6, np.int64)
        self._check(self._L.titan_gb300_server_info(self._h, _ptr(out, ctypes.c_int64)), "server_info")
        keys = ("busy_slots", "free_slots", "launches", "status", "ctas", "smem_bytes")
        return {k: int(v) for k, v in zip(keys, out)}

    def close(self):
        if getattr(self, "_h", None):
            self._L.titan_gb300_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def stl_inside(tri, pts, num_rays: int = 5, seed: int = 1, device: int = 0) -> np.ndarray:
    """Point-in-mesh test of STL import on the GPU (titan_gb300_stl_inside):
    tri (T, 9) or (T, 3, 3) triangle vertices, pts (N, 3); True where more than
    half of num_rays random rays cross the mesh an odd number of times."""
    tri = np.ascontiguousarray(tri, np.float64).reshape(-1, 9)
    pts = np.ascontiguousarray(pts, np.float64).reshape(-1, 3)
    out = np.zeros(pts.shape[0], np.uint8)
    rc = lib().titan_gb300_stl_inside(device, _ptr(tri, ctypes.c_double), tri.shape[0], _ptr(pts, ctypes.c_double),
                                      pts.shape[0], num_rays, seed, _ptr(out, ctypes.c_uint8))
    if rc:
        raise TitanError(rc, "stl_inside")
    return out.astype(bool)

