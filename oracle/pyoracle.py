"""ctypes wrapper of the CPU oracle (oracle/libtitan_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py, never by the product package.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libtitan_oracle.so"

ASCENDING, DESCENDING, ATOMIC_OMP, DEVICE = 0, 1, 2, 3

_D = ctypes.POINTER(ctypes.c_double)
_I32 = ctypes.POINTER(ctypes.c_int32)
_I64 = ctypes.POINTER(ctypes.c_int64)
_U8 = ctypes.POINTER(ctypes.c_uint8)


class ToScene(ctypes.Structure):
    _fields_ = [
        ("n_masses", ctypes.c_int64),
        ("pos", _D), ("vel", _D), ("acc", _D), ("force", _D),
        ("ext", _D), ("m", _D), ("T", _D), ("fixed", _U8), ("drag", _I32),
        ("lc_ptr", _I64), ("lc_type", _I32), ("lc_vec", _D), ("lc_num", _D),
        ("n_springs", ctypes.c_int64),
        ("left", _I32), ("right", _I32),
        ("k", _D), ("rest", _D), ("damping", _D),
        ("type", _I32), ("omega", _D), ("amp", _D), ("phase", _D),
        ("n_planes", ctypes.c_int32),
        ("plane_n", _D), ("plane_off", _D), ("plane_fk", _D), ("plane_fs", _D),
        ("n_balls", ctypes.c_int32),
        ("ball_c", _D), ("ball_r", _D),
        ("mass_bp", _I32), ("bp_n", _D), ("bp_off", _D), ("bp_fk", _D), ("bp_fs", _D),
        ("g", ctypes.c_double * 3), ("dt", ctypes.c_double), ("T_global", ctypes.c_double),
        ("heavy_threshold", ctypes.c_int32),
        ("integrator", ctypes.c_int32),
    ]


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            subprocess.run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                            str(HERE / "titan_oracle.c"), "-o", str(LIB_PATH), "-lm"], check=True)
        L = ctypes.CDLL(str(LIB_PATH))
        L.to_step.restype = ctypes.c_int
        L.to_step.argtypes = [ctypes.POINTER(ToScene), ctypes.c_int64, ctypes.c_int, ctypes.c_int]
        L.to_spring_force.argtypes = [_D, _D, _D, _D, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_double, _D]
        L.to_ball_apply.argtypes = [_D, ctypes.c_double, _D, _D]
        L.to_plane_apply.argtypes = [_D, ctypes.c_double, ctypes.c_double, ctypes.c_double, _D, _D, _D]
        L.to_constraint_plane_apply.argtypes = [_D, ctypes.c_double, _D, _D]
        L.to_direction_apply.argtypes = [_D, ctypes.c_double, _D, _D]
        L.to_normalize.argtypes = [_D, _D]
        L.to_lattice_springs.restype = ctypes.c_int64
        L.to_lattice_springs.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.to_lattice.argtypes = [_D, _D, ctypes.c_int, ctypes.c_int, ctypes.c_int, _D, _I32, _I32, _D]
        L.to_energy.argtypes = [ctypes.POINTER(ToScene), ctypes.c_double, _D]
        L.to_momentum.argtypes = [ctypes.POINTER(ToScene), _D, _D]
        _LIB = L
    return _LIB


def _p(a, t=ctypes.c_double):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(t))


def _f(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def normalize(v):
    v = _f(v).reshape(3).copy()
    out = np.zeros(3)
    lib().to_normalize(_p(v), _p(out))
    return out


def lattice(center, dims, nx, ny, nz):
    L = lib()
    ns = L.to_lattice_springs(nx, ny, nz)
    n = nx * ny * nz
    pos = np.zeros((n, 3))
    left = np.zeros(ns, np.int32)
    right = np.zeros(ns, np.int32)
    rest = np.zeros(ns)
    c, d = _f(center), _f(dims)
    L.to_lattice(_p(c), _p(d), nx, ny, nz, _p(pos), _p(left, ctypes.c_int32), _p(right, ctypes.c_int32), _p(rest))
    return pos, left, right, rest


class OracleSim:
    """Holds a scene (dict, see titan_gb300.workloads) and steps it on the CPU."""

    def __init__(self, sc: dict, heavy_threshold: int = 96):
        n = sc["pos"].shape[0]
        ns = sc["left"].size
        self.n, self.ns = n, ns
        self.pos = _f(sc["pos"]).reshape(n, 3).copy()
        self.vel = (_f(sc["vel"]).reshape(n, 3).copy() if sc.get("vel") is not None else np.zeros((n, 3)))
        self.acc = np.zeros((n, 3))
        self.force = np.zeros((n, 3))
        self.T = np.zeros(n)
        self._keep = {}
        keep = self._keep
        keep["m"] = _f(sc["m"])
        keep["ext"] = _f(sc.get("ext"))
        keep["fixed"] = None if sc.get("fixed") is None else np.ascontiguousarray(sc["fixed"], np.uint8)
        keep["drag"] = None if sc.get("drag") is None else np.ascontiguousarray(
            np.trunc(np.asarray(sc["drag"], float)), np.int32)
        for key in ("left", "right", "type"):
            keep[key] = None if sc.get(key) is None else np.ascontiguousarray(sc[key], np.int32)
        for key in ("k", "rest", "damping", "omega", "amp", "phase"):
            keep[key] = _f(sc.get(key))
        if keep["damping"] is None:
            keep["damping"] = np.zeros(ns)
        planes = sc.get("planes", [])
        keep["plane_n"] = np.array([normalize(p[0]) for p in planes], float).reshape(-1)
        keep["plane_off"] = np.array([p[1] for p in planes], float)
        keep["plane_fk"] = np.array([p[2] for p in planes], float)
        keep["plane_fs"] = np.array([p[3] for p in planes], float)
        balls = sc.get("balls", [])
        keep["ball_c"] = np.array([b[0] for b in balls], float).reshape(-1)
        keep["ball_r"] = np.array([b[1] for b in balls], float)
        if "lc_ptr" in sc:
            self._local(sc)
        if "body_ptr" in sc and sc.get("body_planes"):
            bp = sc["body_planes"]
            mass_bp = np.full(n, -1, np.int32)
            ptr = sc["body_ptr"]
            for b, p in enumerate(bp):
                if p[0] is not None:
                    mass_bp[ptr[b]:ptr[b + 1]] = b
            keep["mass_bp"] = mass_bp
            keep["bp_n"] = np.array([normalize(p[0]) if p[0] is not None else np.zeros(3) for p in bp]).reshape(-1)
            keep["bp_off"] = np.array([p[1] for p in bp], float)
            keep["bp_fk"] = np.array([p[2] for p in bp], float)
            keep["bp_fs"] = np.array([p[3] for p in bp], float)
        s = ToScene()
        s.n_masses = n
        s.pos, s.vel, s.acc, s.force, s.T = _p(self.pos), _p(self.vel), _p(self.acc), _p(self.force), _p(self.T)
        s.ext, s.m = _p(keep["ext"]), _p(keep["m"])
        s.fixed = _p(keep["fixed"], ctypes.c_uint8)
        s.drag = _p(keep["drag"], ctypes.c_int32)
        s.n_springs = ns
        s.left, s.right, s.type = (_p(keep[x], ctypes.c_int32) for x in ("left", "right", "type"))
        s.k, s.rest, s.damping, s.omega, s.amp, s.phase = (_p(keep[x]) for x in
                                                            ("k", "rest", "damping", "omega", "amp", "phase"))
        s.n_planes = len(planes)
        s.plane_n, s.plane_off, s.plane_fk, s.plane_fs = (_p(keep[x]) for x in
                                                          ("plane_n", "plane_off", "plane_fk", "plane_fs"))
        s.n_balls = len(balls)
        s.ball_c, s.ball_r = _p(keep["ball_c"]), _p(keep["ball_r"])
        if "lc_ptr" in keep:
            s.lc_ptr = _p(keep["lc_ptr"], ctypes.c_int64)
            s.lc_type = _p(keep["lc_type"], ctypes.c_int32)
            s.lc_vec, s.lc_num = _p(keep["lc_vec"]), _p(keep["lc_num"])
        if "mass_bp" in keep:
            s.mass_bp = _p(keep["mass_bp"], ctypes.c_int32)
            s.bp_n, s.bp_off, s.bp_fk, s.bp_fs = (_p(keep[x]) for x in ("bp_n", "bp_off", "bp_fk", "bp_fs"))
        for c in range(3):
            s.g[c] = float(sc["g"][c])
        s.dt = float(sc["dt"])
        s.T_global = 0.0
        s.heavy_threshold = heavy_threshold
        s.integrator = int(sc.get("integrator", 0))
        self.s = s

    def _local(self, sc):
        """Sort local constraint records into the reference's application
        order (contact planes, balls, constraint planes, directions) and
        normalise vectors as the reference constructors do."""
        n = self.n
        ptr, typ, vec, num = sc["lc_ptr"], sc["lc_type"], np.asarray(sc["lc_vec"], float).reshape(-1, 3), sc["lc_num"]
        order = {1: 0, 2: 1, 0: 2, 3: 3}
        optr, otyp, ovec, onum = [0], [], [], []
        for i in range(n):
            recs = [r for r in range(ptr[i], ptr[i + 1])]
            for o in (1, 2, 0, 3):
                for r in recs:
                    if typ[r] == o:
                        otyp.append(o)
                        ovec.append(vec[r] if o == 2 else normalize(vec[r]))
                        onum.append(num[r])
            optr.append(len(otyp))
        del order
        self._keep["lc_ptr"] = np.array(optr, np.int64)
        self._keep["lc_type"] = np.array(otyp if otyp else [0], np.int32)
        self._keep["lc_vec"] = np.array(ovec if ovec else [[0, 0, 0]], float).reshape(-1)
        self._keep["lc_num"] = np.array(onum if onum else [0], float)

    @property
    def time(self):
        return self.s.T_global

    def step(self, nsteps=1, order=ASCENDING, nthreads=1):
        rc = lib().to_step(ctypes.byref(self.s), nsteps, order, nthreads)
        if rc != 0:
            raise RuntimeError(f"oracle step failed ({rc})")

    def energy(self, g_mag=9.81):
        out = np.zeros(4)
        lib().to_energy(ctypes.byref(self.s), g_mag, _p(out))
        return out

    def momentum(self):
        lin, ang = np.zeros(3), np.zeros(3)
        lib().to_momentum(ctypes.byref(self.s), _p(lin), _p(ang))
        return lin, ang


def host_threads() -> int:
    return int(os.environ.get("OMP_NUM_THREADS") or os.cpu_count() or 1)


def stl_inside(tri, pts, num_rays=5, seed=1, nthreads=0):
    """Oracle of STL point-in-mesh classification (see titan_oracle.h)."""
    L = lib()
    L.to_stl_inside.argtypes = [_D, ctypes.c_int64, _D, ctypes.c_int64, ctypes.c_int, ctypes.c_uint64,
                                _U8, ctypes.c_int]
    tri = np.ascontiguousarray(tri, np.float64).reshape(-1, 9)
    pts = np.ascontiguousarray(pts, np.float64).reshape(-1, 3)
    out = np.zeros(pts.shape[0], np.uint8)
    rc = L.to_stl_inside(tri.ctypes.data_as(_D), tri.shape[0], pts.ctypes.data_as(_D), pts.shape[0], num_rays,
                         seed, out.ctypes.data_as(_U8), nthreads or host_threads())
    if rc:
        raise ValueError("to_stl_inside failed")
    return out.astype(bool)

