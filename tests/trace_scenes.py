"""Seeded ray sets for the trace tests: a height-field mesh on an integer lattice (every
vertex, edge midpoint and shared-edge point exactly representable, so shared vertices are the
same floats in both triangles) and rays aimed exactly at its vertices and edges."""
import numpy as np

from render_engine_gb300 import scene as S

GRID = 24


def lattice_mesh(seed: int = 0):
    """GRID x GRID unit cells over [0, GRID]^2, integer heights 0..2, each cell split into two
    triangles along an alternating diagonal (n, 3, 3)."""
    rng = np.random.default_rng(seed)
    h = rng.integers(0, 3, size=(GRID + 1, GRID + 1)).astype(np.float32)
    tris = []
    for j in range(GRID):
        for i in range(GRID):
            a = (i, j, h[i, j]); b = (i + 1, j, h[i + 1, j]); c = (i, j + 1, h[i, j + 1]); d = (i + 1, j + 1, h[i + 1, j + 1])
            if (i + j) % 2:
                tris += [[a, b, d], [a, d, c]]
            else:
                tris += [[a, b, c], [b, d, c]]
    return np.array(tris, np.float32), h


def lattice_scene_bytes(seed: int = 0) -> bytes:
    V, _ = lattice_mesh(seed)
    n = len(V)
    L = np.array([[4.0, 4.0, 8.0], [12.0, 12.0, 8.0], [20.0, 4.0, 8.0]], np.float32)
    I = [[20, 20, 0], [0, 20, 0], [20, 20, 0], [20, 20, 20], [0, 20, 0]]
    box = [(-8.0, -8.0, 1.0)] * 2 + [(-8.0, 30.0, 1.0)] * 3    # the movable cube stays off the lattice
    sc = S.mesh_scene(V, np.full(n, 0.5, np.float32), np.ones(n, np.uint8), L, I, box, 1.0, 3000, seed)
    return S.write(sc)


def edge_rays(h: np.ndarray, n: int = 6000, seed: int = 1) -> np.ndarray:
    """Rays (origin, direction) from above and below the lattice whose exact line passes through
    an interior lattice vertex or the midpoint of an interior edge or cell diagonal: origin +
    1 * direction is that point, all values dyadic."""
    rng = np.random.default_rng(seed)
    i = rng.integers(1, GRID - 1, n)
    j = rng.integers(1, GRID - 1, n)
    kind = rng.integers(0, 4, n)    # vertex, x edge, y edge, diagonal midpoint
    tx = i + np.where((kind == 1) | (kind == 3), 0.5, 0.0)
    ty = j + np.where((kind == 2) | (kind == 3), 0.5, 0.0)
    hz = h[i, j].astype(np.float64)
    hx = h[i + 1, j].astype(np.float64)
    hy = h[i, j + 1].astype(np.float64)
    hd = h[i + 1, j + 1].astype(np.float64)
    diag_a = np.where((i + j) % 2 == 1, 0.5 * (hz + hd), 0.5 * (hx + hy))   # the cell's split diagonal
    tz = np.select([kind == 0, kind == 1, kind == 2], [hz, 0.5 * (hz + hx), 0.5 * (hz + hy)], diag_a)
    below = rng.random(n) < 0.25
    ox = tx + rng.integers(-64, 65, n) / 16.0
    oy = ty + rng.integers(-64, 65, n) / 16.0
    oz = np.where(below, -6.0, 24.0) + rng.integers(0, 16, n) / 8.0
    o = np.stack([ox, oy, oz], 1)
    d = np.stack([tx, ty, tz], 1) - o
    return np.concatenate([o, d], 1).astype(np.float32)


def random_rays(data: bytes, n: int = 20000, seed: int = 2) -> np.ndarray:
    """Rays from the scene's cache points (offset 1e-3 along the normal) in random directions of
    the normal's hemisphere."""
    sc = S.read(data)
    st = sc.states[0]
    rng = np.random.default_rng(seed)
    k = rng.integers(0, sc.Np, n)
    P = np.asarray(st.P, np.float64).reshape(-1, 3)[k]
    N = np.asarray(st.N, np.float64).reshape(-1, 3)[k]
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d *= np.sign((d * N).sum(1, keepdims=True) + 1e-12)
    return np.concatenate([P + N * 1e-3, d], 1).astype(np.float32)
