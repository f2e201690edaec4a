"""Generates tests/golden/reference_host.npz from the reference's own code.

Run in a checkout where the reference sources exist (the recipe
oracle/build_ref.sh compiles src/object.cu, src/mass.cu, src/spring.cu and
src/vec.cu into oracle/_ref/libtitan_ref_host.so):

    bash oracle/build_ref.sh && python tests/golden/make_golden.py

Contents (all produced by calling the reference's functions):
  lattice_<nx>_<ny>_<nz>_{pos,left,right,rest}  titan::Lattice (src/object.cu:232-293)
  plane_{in,out}      CudaContactPlane::applyForce (src/object.cu:73-106) via ContactPlane
  ball_{in,out}       CudaBall::applyForce (src/object.cu:53-56)
  cplane_{in,out}     CudaConstraintPlane::applyForce (src/object.cu:115-124)
  dir_{in,out}        CudaDirection::applyForce (src/object.cu:133-141)
  norm_{in,out}       ContactPlane normal normalisation (include/Titan/object.h:103)
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
LIB = ROOT / "oracle" / "_ref" / "libtitan_ref_host.so"
OUT = Path(__file__).resolve().parent / "reference_host.npz"

LATTICES = [((0.0, 0.0, 10.0), (5.0, 5.0, 5.0), (5, 5, 5)),
            ((0.3, -1.0, 2.6), (5.0, 4.0, 3.0), (3, 4, 5)),
            ((1.0, 2.0, 3.0), (0.7, 0.0, 2.0), (1, 3, 2)),
            ((0.0, 0.0, 5.0), (4.0, 4.0, 4.0), (8, 8, 8)),
            ((-2.0, 0.5, 1.25), (1.1, 2.2, 3.3), (7, 2, 9))]


def main():
    R = ctypes.CDLL(str(LIB))
    D = ctypes.POINTER(ctypes.c_double)
    I = ctypes.POINTER(ctypes.c_int32)
    p = lambda a, t=D: a.ctypes.data_as(t)
    R.ref_lattice_springs.restype = ctypes.c_int64
    R.ref_plane_apply.argtypes = [D, ctypes.c_double, ctypes.c_double, ctypes.c_double, D, D, D]
    R.ref_ball_apply.argtypes = [D, ctypes.c_double, D, D]
    R.ref_constraint_plane_apply.argtypes = [D, ctypes.c_double, D, D, D]
    R.ref_direction_apply.argtypes = [D, ctypes.c_double, D, D, D]
    R.ref_normalize.argtypes = [D, D]
    out = {}
    for c, d, dims in LATTICES:
        ns = R.ref_lattice_springs(*dims)
        n = dims[0] * dims[1] * dims[2]
        pos = np.zeros((n, 3))
        left = np.zeros(ns, np.int32)
        right = np.zeros(ns, np.int32)
        rest = np.zeros(ns)
        ca, da = np.array(c), np.array(d)
        R.ref_lattice(p(ca), p(da), *dims, p(pos), p(left, I), p(right, I), p(rest))
        key = "lattice_%d_%d_%d" % dims
        out[key + "_center"], out[key + "_dims"] = ca, da
        out[key + "_pos"], out[key + "_left"], out[key + "_right"], out[key + "_rest"] = pos, left, right, rest

    rng = np.random.default_rng(12345)
    N = 400
    # contact plane: [n(3), off, fk, fs, pos(3), vel(3), force(3)]
    pin = np.zeros((N, 15))
    pout = np.zeros((N, 3))
    for i in range(N):
        n = rng.normal(size=3) if i % 4 else np.array([0.0, 0.0, 1.0])
        off = rng.uniform(-0.5, 0.5)
        fk, fs = (rng.uniform(0, 1.5), rng.uniform(0, 1.5)) if i % 3 else (0.0, 0.0)
        if i % 7 == 0:
            fk = 0.0
        pos = rng.uniform(-1, 1, 3)
        vel = rng.normal(size=3) if i % 5 else np.zeros(3)  # zero velocity -> static branch
        force = rng.normal(scale=5.0, size=3)
        pin[i] = np.concatenate([n, [off, fk, fs], pos, vel, force])
        f = force.copy()
        R.ref_plane_apply(p(n), off, fk, fs, p(pos), p(vel), p(f))
        pout[i] = f
    out["plane_in"], out["plane_out"] = pin, pout
    # ball: [c(3), r, pos(3), force(3)]
    bin_ = np.zeros((N, 10))
    bout = np.zeros((N, 3))
    for i in range(N):
        c = rng.uniform(-1, 1, 3)
        r = rng.uniform(0.1, 2.0)
        pos = rng.uniform(-2, 2, 3)
        force = rng.normal(size=3)
        bin_[i] = np.concatenate([c, [r], pos, force])
        f = force.copy()
        R.ref_ball_apply(p(c), r, p(pos), p(f))
        bout[i] = f
    out["ball_in"], out["ball_out"] = bin_, bout
    # constraint plane and direction: [vec(3), friction, pos(3), vel(3), force(3)] -> [vel, force]
    for name, fn in (("cplane", R.ref_constraint_plane_apply), ("dir", R.ref_direction_apply)):
        cin = np.zeros((N, 13))
        cout = np.zeros((N, 6))
        for i in range(N):
            v = rng.normal(size=3)
            fr = rng.uniform(0, 1)
            pos = rng.normal(size=3)
            vel = rng.normal(size=3) if i % 6 else np.zeros(3)
            force = rng.normal(size=3)
            cin[i] = np.concatenate([v, [fr], pos, vel, force])
            vv, ff = vel.copy(), force.copy()
            fn(p(v), fr, p(pos), p(vv), p(ff))
            cout[i] = np.concatenate([vv, ff])
        out[name + "_in"], out[name + "_out"] = cin, cout
    nin = rng.normal(size=(N, 3)) * rng.uniform(0.01, 100, (N, 1))
    nout = np.zeros((N, 3))
    for i in range(N):
        o = np.zeros(3)
        R.ref_normalize(p(np.ascontiguousarray(nin[i])), p(o))
        nout[i] = o
    out["norm_in"], out["norm_out"] = nin, nout
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, sum(v.nbytes for v in out.values()), "bytes")


if __name__ == "__main__":
    main()
