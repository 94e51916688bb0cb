"""rc_trace_rays on the GPU against the oracle: the reference's Moller-Trumbore traversal and
the watertight mode (RC_FLAG_WATERTIGHT) on caller-given rays."""
import numpy as np
import pytest

from oracle import pyoracle as po
from render_engine_gb300 import native as N
from render_engine_gb300 import scene as S

from trace_scenes import edge_rays, lattice_mesh, lattice_scene_bytes, random_rays

pytestmark = pytest.mark.gpu


def _gpu(data, flags):
    ctx = N.Context(flags=flags)
    ctx.load_bytes(data)
    return ctx


def test_watertight_edge_rays_bitexact_vs_oracle():
    _, h = lattice_mesh()
    data = lattice_scene_bytes()
    rays = edge_rays(h)
    pc, tc = po.Scene(data=data).trace_rays(0, rays, watertight=True)
    ctx = _gpu(data, N.FLAG_WATERTIGHT)
    pg, tg = ctx.trace_rays(0, rays)
    assert ctx.device_flags() == 0
    ctx.close()
    assert (pg <= -2).all(), int((pg == -1).sum())       # no ray through a shared edge or vertex leaks
    np.testing.assert_array_equal(pg, pc)
    np.testing.assert_array_equal(tg.view(np.uint32), tc.view(np.uint32))


@pytest.mark.parametrize("watertight", [False, True])
def test_street_rays_vs_oracle(watertight):
    """Hit primitive IDs and distances on a format-3 street: the watertight mode bit for bit
    (every product rounded on its own on both sides); the reference's test equal except at
    ulp-level ties (distances to 1e-5 relative)."""
    data = S.write(S.street_scene(points=12000, buildings=6, size=60.0))
    rays = random_rays(data, 40000, seed=5)
    pc, tc = po.Scene(data=data).trace_rays(0, rays, watertight=watertight)
    ctx = _gpu(data, N.FLAG_WATERTIGHT if watertight else 0)
    pg, tg = ctx.trace_rays(0, rays)
    pg2, tg2 = ctx.trace_rays(2, rays)          # another state: the cube moved
    assert ctx.device_flags() == 0
    ctx.close()
    pc2, _ = po.Scene(data=data).trace_rays(2, rays, watertight=watertight)
    if watertight:
        np.testing.assert_array_equal(pg, pc)
        np.testing.assert_array_equal(tg.view(np.uint32), tc.view(np.uint32))
        np.testing.assert_array_equal(pg2, pc2)
    else:
        same = pg == pc
        assert same.mean() > 0.999, same.mean()
        hit = same & (pg != -1)
        rel = np.abs(tg[hit] - tc[hit]) / np.abs(tc[hit])
        assert (rel <= 1e-5).all(), rel.max()
        assert (pg2 == pc2).mean() > 0.999
    assert (pg <= -2).mean() > 0.2


def test_trace_rays_arguments():
    data = lattice_scene_bytes()
    ctx = _gpu(data, 0)
    p, t = ctx.trace_rays(0, np.zeros((0, 6), np.float32))
    assert len(p) == 0 and len(t) == 0
    with pytest.raises(N.RCError):
        ctx.trace_rays(9, np.zeros((1, 6), np.float32))
    # a ray pointing away from everything: no hit, +inf
    p, t = ctx.trace_rays(0, np.array([[5.0, 5.0, 50.0, 0.0, 0.0, 1.0]], np.float32))
    assert p[0] == -1 and np.isinf(t[0])
    ctx.close()
