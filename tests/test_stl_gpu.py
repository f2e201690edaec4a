"""STL import's point-in-mesh test on the GPU (titan_gb300_stl_inside)
against the oracle's restatement: the same classification bit for bit
(same counter-based rays, the reference's ray-triangle arithmetic)."""
import numpy as np
import pytest

import titan_gb300 as tg
from oracle import pyoracle as po
from tests import meshes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mesh", ["cube", "sphere", "l_shape"])
@pytest.mark.parametrize("num_rays", [1, 5, 64])
def test_stl_inside_matches_oracle(mesh, num_rays):
    tri = {"cube": meshes.cube(), "sphere": meshes.icosphere(1.3, (0.2, -0.1, 0.3), levels=2),
           "l_shape": meshes.l_shape()}[mesh]
    rng = np.random.default_rng(num_rays)
    lo, hi = tri.reshape(-1, 3).min(0) - 0.3, tri.reshape(-1, 3).max(0) + 0.3
    pts = rng.uniform(lo, hi, size=(20000, 3))
    pts[:1000] = np.round(pts[:1000], 1)  # lattice-like points, some on faces and edges
    got = tg.stl_inside(tri, pts, num_rays=num_rays, seed=77)
    want = po.stl_inside(tri, pts, num_rays=num_rays, seed=77)
    assert np.array_equal(got, want), int(np.sum(got != want))
    assert 0 < got.sum() < got.size


def test_stl_inside_many_triangles():
    tri = meshes.icosphere(1.0, levels=4)  # 5120 triangles: several shared-memory chunks
    pts = np.random.default_rng(5).uniform(-1.2, 1.2, size=(4096, 3))
    assert np.array_equal(tg.stl_inside(tri, pts, num_rays=5, seed=3), po.stl_inside(tri, pts, num_rays=5, seed=3))
