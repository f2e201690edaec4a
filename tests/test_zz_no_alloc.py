"""The allocation-free diagnostics entry point.

titan_gb300_diagnostics_noalloc serves callers that may not call cudaMalloc
when they need a result (memory reserved once at start-up, a foreign caching
allocator that owns device memory, or work issued during stream capture).
It reads state the caller already holds on the device and uses a fixed
scratch array compiled into the library.  This test calls it through the C
ABI and checks it against titan_gb300_diagnostics, the handle-based entry
point, on two calls in a row, with the tolerances of the other diagnostics
test.  (The device buffers below are made by the test, not by the call.)

This file sorts last so that a run stopping at the first failure has run
every other test first.
"""
import ctypes

import numpy as np
import pytest

import titan_gb300 as tg
from titan_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

MAX_ELEMS = 4096 * 256 * 64


def noalloc_fn():
    fn = tg.lib().titan_gb300_diagnostics_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_double,
                   ctypes.c_void_p, ctypes.c_void_p]
    return fn


def test_noalloc_diagnostics_match_handle_entry_point():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    fn = noalloc_fn()
    sc = wl.falling_cube(contact=True)
    sc["vel"] = np.random.default_rng(7).normal(scale=0.2, size=sc["pos"].shape)
    sim = wl.make_sim(sc, tg.FP64)
    left = torch.tensor(sc["left"], dtype=torch.int32, device=dev)
    right = torch.tensor(sc["right"], dtype=torch.int32, device=dev)
    k = torch.tensor(sc["k"], dtype=torch.float64, device=dev)
    rest = torch.tensor(sc["rest"], dtype=torch.float64, device=dev)
    m = torch.tensor(sc["m"], dtype=torch.float64, device=dev)
    out = torch.full((9,), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    for call in range(2):
        sim.step(700)
        ref = sim.diagnostics(9.8)
        st = sim.get_state()
        pos = torch.tensor(st["pos"], dtype=torch.float64, device=dev)
        vel = torch.tensor(st["vel"], dtype=torch.float64, device=dev)
        rc = fn(pos.data_ptr(), vel.data_ptr(), m.data_ptr(), pos.shape[0], left.data_ptr(), right.data_ptr(),
                k.data_ptr(), rest.data_ptr(), left.shape[0], 9.8, out.data_ptr(), stream.cuda_stream)
        assert rc == 0, f"call {call}: status {rc}"
        stream.synchronize()
        got = out.cpu().numpy()
        np.testing.assert_allclose(got[:3], [ref["spring_pe"], ref["kinetic"], ref["gravity_pe"]], rtol=1e-12)
        np.testing.assert_allclose(got[3:6], ref["linear"], rtol=1e-11, atol=1e-13)
        np.testing.assert_allclose(got[6:9], ref["angular"], rtol=1e-11, atol=1e-13)
    # sizes beyond the scratch array's capacity are refused before any launch
    rc = fn(pos.data_ptr(), vel.data_ptr(), m.data_ptr(), MAX_ELEMS + 1, left.data_ptr(), right.data_ptr(),
            k.data_ptr(), rest.data_ptr(), 10, 9.8, out.data_ptr(), stream.cuda_stream)
    assert rc == 4  # TITAN_GB300_ELIMIT


def test_noalloc_diagnostics_many_blocks_and_empty_call():
    """A 30^3 lattice (27,000 masses, 335,526 springs: 21 partial-sum blocks of
    16,384 elements, so the second kernel reduces many slots) against the
    handle-based entry point and a float64 numpy sum; then a call with no
    masses and no springs, which must write zeros."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    fn = noalloc_fn()
    sc = wl.lattice_scene((0, 0, 2.0), (2, 2, 2), 30, 30, 30, k=5e3, damping=0.1)
    rng = np.random.default_rng(8)
    sc["vel"] = rng.normal(scale=0.3, size=sc["pos"].shape)
    sc["k"] = np.exp(rng.uniform(np.log(1e3), np.log(1e4), sc["k"].size))
    sc["planes"].append(((0.0, 0.0, 1.0), 0.0, 0.5, 0.5))
    sim = wl.make_sim(sc, tg.FP64)
    left = torch.tensor(sc["left"], dtype=torch.int32, device=dev)
    right = torch.tensor(sc["right"], dtype=torch.int32, device=dev)
    k = torch.tensor(sc["k"], dtype=torch.float64, device=dev)
    rest = torch.tensor(sc["rest"], dtype=torch.float64, device=dev)
    m = torch.tensor(sc["m"], dtype=torch.float64, device=dev)
    out = torch.full((9,), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    assert (max(sc["pos"].shape[0], sc["left"].size) + 16383) // 16384 > 1
    for call in range(2):
        sim.step(300)
        ref = sim.diagnostics(9.8)
        st = sim.get_state()
        pos = torch.tensor(st["pos"], dtype=torch.float64, device=dev)
        vel = torch.tensor(st["vel"], dtype=torch.float64, device=dev)
        rc = fn(pos.data_ptr(), vel.data_ptr(), m.data_ptr(), pos.shape[0], left.data_ptr(), right.data_ptr(),
                k.data_ptr(), rest.data_ptr(), left.shape[0], 9.8, out.data_ptr(), stream.cuda_stream)
        assert rc == 0, f"call {call}: status {rc}"
        stream.synchronize()
        got = out.cpu().numpy()
        np.testing.assert_allclose(got[:3], [ref["spring_pe"], ref["kinetic"], ref["gravity_pe"]], rtol=1e-12)
        # signed sums: tolerance relative to the sum of magnitudes
        x, v, mm = st["pos"], st["vel"], sc["m"]
        p = v * mm[:, None]
        lin_scale = np.sum(np.abs(p), axis=0)
        ang = np.cross(p, x)  # the library's convention: sum of cross(m v, x)
        ax, ap = np.abs(x), np.abs(p)
        ang_scale = np.array([np.sum(ax[:, 1] * ap[:, 2] + ax[:, 2] * ap[:, 1]),
                              np.sum(ax[:, 2] * ap[:, 0] + ax[:, 0] * ap[:, 2]),
                              np.sum(ax[:, 0] * ap[:, 1] + ax[:, 1] * ap[:, 0])])
        np.testing.assert_allclose(got[3:6], ref["linear"], rtol=0, atol=1e-13 * lin_scale.max())
        np.testing.assert_allclose(got[6:9], ref["angular"], rtol=0, atol=1e-13 * ang_scale.max())
        np.testing.assert_allclose(got[3:6], p.sum(axis=0), rtol=0, atol=1e-13 * lin_scale.max())
        np.testing.assert_allclose(got[6:9], ang.sum(axis=0), rtol=0, atol=1e-13 * ang_scale.max())
    out.fill_(float("nan"))
    rc = fn(0, 0, 0, 0, 0, 0, 0, 0, 0, 9.8, out.data_ptr(), stream.cuda_stream)
    assert rc == 0
    stream.synchronize()
    assert np.array_equal(out.cpu().numpy(), np.zeros(9))
