"""The oracle's ray trace for caller-given rays, and its watertight triangle test (no GPU)."""
import numpy as np

from oracle import pyoracle as po
from render_engine_gb300 import scene as S

from trace_scenes import edge_rays, lattice_mesh, lattice_scene_bytes, random_rays


def test_watertight_known_answer():
    """One lattice cell seen straight down: both tests return the exact distance and the same
    triangle away from the edges."""
    data = lattice_scene_bytes()
    sc = po.Scene(data=data)
    _, h = lattice_mesh()
    rays = []
    for (i, j) in ((3, 5), (10, 10), (17, 2)):
        if h[i, j] == h[i + 1, j] == h[i, j + 1] == h[i + 1, j + 1]:
            rays.append([i + 0.25, j + 0.6, 10.0, 0.0, 0.0, -1.0])
            rays.append([i + 0.75, j + 0.1, 10.0, 0.0, 0.0, -2.0])
    if not rays:   # no flat cell among those: take the first flat cell of the lattice
        for i in range(20):
            if h[i, 1] == h[i + 1, 1] == h[i, 2] == h[i + 1, 2]:
                rays = [[i + 0.25, 1.6, 10.0, 0.0, 0.0, -1.0], [i + 0.75, 1.1, 10.0, 0.0, 0.0, -2.0]]
                break
    rays = np.array(rays, np.float32)
    pm, tm = sc.trace_rays(0, rays, watertight=False)
    pw, tw = sc.trace_rays(0, rays, watertight=True)
    assert (pm <= -2).all() and np.array_equal(pm, pw)
    z = np.array([h[int(r[0]), int(r[1])] for r in rays], np.float32)
    np.testing.assert_array_equal(tw, (10.0 - z) / -rays[:, 5])
    np.testing.assert_array_equal(tm, tw)


def test_watertight_rays_through_shared_edges_never_leak():
    """Rays aimed exactly at lattice vertices and shared edges of a closed height field: every
    one hits with the watertight test and its conservative box test.  (Moller-Trumbore's barycentric tests can reject the point on both sides
    of an edge; its count is reported, not asserted.)"""
    _, h = lattice_mesh()
    sc = po.Scene(data=lattice_scene_bytes())
    rays = edge_rays(h)
    pw, tw = sc.trace_rays(0, rays, watertight=True)
    pm, _ = sc.trace_rays(0, rays, watertight=False)
    assert (pw <= -2).all(), int((pw == -1).sum())
    # most rays cross the surface at their target point (t = 1); others meet a nearer hill
    # first, or only touch the target vertex (a valley seen from below, a peak from above) and
    # go on to their next crossing
    assert np.isfinite(tw).all() and (tw > 0).all()
    assert (np.abs(tw - 1.0) <= 1e-5).mean() > 0.95
    print("Moller-Trumbore misses on %d edge rays: %d" % (len(rays), int((pm == -1).sum())))


def test_watertight_agrees_with_moller_trumbore_off_edges():
    """On the street mesh, the two tests pick the same triangle and distance except at ties."""
    data = S.write(S.street_scene(points=5000, buildings=4, size=40.0))
    sc = po.Scene(data=data)
    rays = random_rays(data, 20000)
    pm, tm = sc.trace_rays(0, rays, watertight=False)
    pw, tw = sc.trace_rays(0, rays, watertight=True)
    same = pm == pw
    assert same.mean() > 0.998, same.mean()
    hit = same & (pm != -1)
    rel = np.abs(tm[hit] - tw[hit]) / np.maximum(np.abs(tm[hit]), 1e-30)
    assert (rel <= 1e-5).mean() > 0.999, np.quantile(rel, 0.999)
    assert (pm <= -2).mean() > 0.2   # most rays end on the static mesh


def test_trace_rays_state_and_dynamic_triangles():
    """The movable cube (dynamic quads) is found before the static mesh, per state."""
    data = lattice_scene_bytes()
    sc = po.Scene(data=data)
    st = S.read(data).states
    rays = []
    for s in range(len(st)):
        c = st[s].T.reshape(-1, 9)[:, :3].mean(0)   # near the cube of state s
        rays.append([c[0] + 0.01, c[1] + 0.02, 20.0, 0.0, 0.0, -1.0])
    rays = np.array(rays, np.float32)
    for s in range(len(st)):
        p, t = sc.trace_rays(s, rays)
        assert p[s] >= 0, (s, p)       # a quad of the cube, not a static triangle
        assert np.isfinite(t[s])
