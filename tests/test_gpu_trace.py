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
    ulp-level ties, each one logged (distances to 1e-5 relative)."""
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
        # every disagreement is logged as a tie: two triangles hit at the same distance (1e-5
        # relative: a shared edge or vertex, where the rounded barycentrics of both accept the
        # ray), or a ray through an edge that one side's rounding lets through
        diff = ~same
        both = diff & (pg != -1) & (pc != -1)
        with np.errstate(invalid="ignore"):   # misses carry an infinite distance
            ties = both & (np.abs(tg - tc) <= 1e-5 * np.abs(tc))
        leaks = diff & ((pg == -1) != (pc == -1))
        assert (ties | leaks).sum() == diff.sum(), (int(diff.sum()), int(ties.sum()), int(leaks.sum()))
        assert leaks.mean() <= 1e-4, leaks.mean()
        print("street rays: %d of %d differ from the oracle, all logged ties (%d same-distance, %d edge leaks)"
              % (int(diff.sum()), len(pg), int(ties.sum()), int(leaks.sum())))
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


def _dag_tree(lo, hi, depth: int = 14) -> np.ndarray:
    """A node array in the format-3 layout whose inner nodes share their children: nodes
    2j+1 and 2j+2 both link to 2j+3 and 2j+4, so a ray that enters the root box visits 2^depth
    leaves, far beyond the traversal guard of 4 x nodes + 64 visits.  Every link and leaf range
    is in bounds (the loader accepts it); the guard ends the walk and raises FLAG_BVH_VISITS."""
    n = 2 * depth + 1
    out = np.zeros((n, 8), np.float32)
    for k in range(n):
        out[k, 0:3] = lo
        out[k, 4:7] = hi
        leaf = k >= n - 2
        link = 0 if leaf else (1 if k == 0 else 2 * ((k - 1) // 2) + 3)
        out[k, 3] = np.array([link], np.int32).view(np.float32)[0]
        out[k, 7] = np.array([4 if leaf else 0], np.int32).view(np.float32)[0]
    return out


def test_trace_rays_keeps_frame_guard_flags():
    """rc_trace_rays between frames leaves the guard word of the run's kernels alone: a flag that
    the state build raised (traversal guard on a shared-child tree) is still reported by
    rc_device_flags after a trace_rays call that raised nothing itself."""
    sc = S.read(lattice_scene_bytes())
    V = np.asarray(sc.mesh["ST"], np.float32).reshape(-1, 9)
    v0 = V[:, 0:3]
    pts = np.concatenate([v0, v0 + V[:, 3:6], v0 + V[:, 6:9]])
    sc.mesh["BN"] = _dag_tree(pts.min(0) - 0.01, pts.max(0) + 0.01)
    ctx = _gpu(S.write(sc), 0)       # the state builds' shadow rays trip the guard (word of the run)
    ctx.sync()                       # the builds run behind the load
    p, t = ctx.trace_rays(0, np.array([[5.0, 5.0, 50.0, 0.0, 0.0, 1.0]], np.float32))   # misses the root box
    assert p[0] == -1 and np.isinf(t[0])
    assert ctx.device_flags() & 1      # FLAG_BVH_VISITS, raised before the call, survives it
    assert ctx.device_flags() == 0     # read once, then cleared
    ctx.close()
