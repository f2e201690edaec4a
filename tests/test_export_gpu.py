"""Asynchronous rollout completion (poll / bounded wait) and the headless
vertex / index export that replaces the reference's OpenGL buffers."""
import numpy as np
import pytest

import titan_gb300 as tg
from titan_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [tg.FP64, tg.FP32, tg.FP32C])
def test_export_vertices_host_and_device(precision):
    import torch
    sc = wl.falling_cube(contact=True)
    s = wl.make_sim(sc, precision)
    s.step(123)
    pos = s.get_state(pos=True, vel=False)["pos"]
    v = s.export_vertices()
    assert v.dtype == np.float32 and v.shape == pos.shape
    assert np.array_equal(v, pos.astype(np.float32))
    d = torch.empty((s.n, 3), dtype=torch.float32, device="cuda")
    s.export_vertices(device_ptr=d.data_ptr())
    s.synchronize()
    assert np.array_equal(d.cpu().numpy(), v)
    di = torch.empty((s.ns, 2), dtype=torch.int32, device="cuda")
    s.export_indices(device_ptr=di.data_ptr())
    assert np.array_equal(di.cpu().numpy().view(np.uint32), s.export_indices())


def test_poll_and_bounded_wait():
    sc = wl.actuated_lattice(40)
    s = wl.make_sim(sc, tg.FP32C)
    s.synchronize()
    assert s.poll()
    s.step(3000)  # tens of milliseconds of queued work
    assert not s.wait(0.0)
    assert s.wait(60000.0)
    assert s.poll()
    assert s.steps == 3000
