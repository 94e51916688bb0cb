"""Scene files: reader, writer and seeded procedural generators.

File layout (little endian), the reference's formats 2 and 3 (cuda/poc_gpu.cu:751-801 reads
them, cuda/prep_mesh.cuh:242-297 writes format 3):

    int32 header[8] = Np, Nq, Nt, NS, NL, NR, has_ref, format
    format 3 only: float lo[3], ext[3], hcell; int32 nst, nnodes, hsize, npst;
                   float ST[9 nst], STN[4 nst], BN[8 nnodes]; uint64 HK[hsize]; int32 HV[hsize]
    float L[3 NL]; float A[Np]; int32 region[Np]
    per state: float inten[NL], P[3 Np], N[3 Np], Q[12 Nq]; int32 dims[2 Nq], off[Nq];
               float T[9 Nt]; int32 TQ[Nt]; has_ref: float ref[Np]; uint8 valid[Np]; float Pw[NL Np]
    per ordered state pair (NS*NS): int32 n, occluder voxels[n]; per light: int32 n, voxels[n]

Format-2 event voxels are cells of a 16 x 8 x 6 grid over the 8 x 4 x 3 m box; format 3 stores
them on the transit grid directly.
"""
from __future__ import annotations

import io
from dataclasses import dataclass, field

import numpy as np

FX, FY, FZ = 16, 8, 6
X1, Y1, Z1 = 8.0, 4.0, 3.0


@dataclass
class State:
    inten: np.ndarray            # (NL,) float32
    P: np.ndarray                # (Np, 3) float32
    N: np.ndarray                # (Np, 3) float32
    Q: np.ndarray                # (Nq, 12) float32: o, u, v, n
    dims: np.ndarray             # (Nq, 2) int32
    off: np.ndarray              # (Nq,) int32
    T: np.ndarray                # (Nt, 9) float32: v0, e1, e2
    TQ: np.ndarray               # (Nt,) int32
    ref: np.ndarray | None = None
    valid: np.ndarray | None = None
    Pw: np.ndarray | None = None  # (Np, NL)


@dataclass
class Scene:
    NR: int
    L: np.ndarray                # (NL, 3)
    A: np.ndarray                # (Np,)
    region: np.ndarray           # (Np,)
    states: list[State]
    occ: dict = field(default_factory=dict)   # (a, b) -> voxel list
    em: dict = field(default_factory=dict)    # (a, b, l) -> voxel list
    fmt: int = 2
    mesh: dict | None = None     # format-3 block

    @property
    def Np(self) -> int:
        return int(self.A.shape[0])

    @property
    def NL(self) -> int:
        return int(self.L.shape[0])

    @property
    def NS(self) -> int:
        return len(self.states)


def write(scene: Scene) -> bytes:
    s0 = scene.states[0]
    has_ref = int(s0.ref is not None)
    b = io.BytesIO()
    b.write(np.array([scene.Np, s0.Q.shape[0], s0.T.shape[0], scene.NS, scene.NL, scene.NR, has_ref, scene.fmt], np.int32).tobytes())
    if scene.fmt == 3:
        m = scene.mesh
        b.write(np.asarray(m["lo"], np.float32).tobytes() + np.asarray(m["ext"], np.float32).tobytes())
        b.write(np.float32(m["hcell"]).tobytes())
        b.write(np.array([len(m["ST"]), len(m["BN"]), len(m["HK"]), m["npst"]], np.int32).tobytes())
        for k, dt in (("ST", np.float32), ("STN", np.float32), ("BN", np.float32), ("HK", np.uint64), ("HV", np.int32)):
            b.write(np.ascontiguousarray(m[k], dt).tobytes())
    b.write(np.ascontiguousarray(scene.L, np.float32).tobytes())
    b.write(np.ascontiguousarray(scene.A, np.float32).tobytes())
    b.write(np.ascontiguousarray(scene.region, np.int32).tobytes())
    for s in scene.states:
        for arr, dt in ((s.inten, np.float32), (s.P, np.float32), (s.N, np.float32), (s.Q, np.float32), (s.dims, np.int32),
                        (s.off, np.int32), (s.T, np.float32), (s.TQ, np.int32)):
            b.write(np.ascontiguousarray(arr, dt).tobytes())
        if has_ref:
            b.write(np.ascontiguousarray(s.ref, np.float32).tobytes())
            b.write(np.ascontiguousarray(s.valid, np.uint8).tobytes())
            b.write(np.ascontiguousarray(s.Pw, np.float32).tobytes())
    for a in range(scene.NS):
        for c in range(scene.NS):
            o = np.asarray(scene.occ.get((a, c), []), np.int32)
            b.write(np.int32(len(o)).tobytes() + o.tobytes())
            for l in range(scene.NL):
                e = np.asarray(scene.em.get((a, c, l), []), np.int32)
                b.write(np.int32(len(e)).tobytes() + e.tobytes())
    return b.getvalue()


def header(data: bytes) -> dict:
    """The eight header integers of a scene file."""
    h = np.frombuffer(data, dtype=np.int32, count=8)
    return dict(zip(("np", "nq", "nt", "ns", "nl", "nr", "has_ref", "fmt"), (int(x) for x in h)))


def read(data: bytes) -> Scene:
    off = 0

    def rd(dt, n):
        nonlocal off
        a = np.frombuffer(data, dtype=dt, count=n, offset=off)
        off += a.nbytes
        return a.copy()

    h = rd(np.int32, 8)
    Np, Nq, Nt, NS, NL, NR, has_ref, fmt = (int(x) for x in h)
    mesh = None
    if fmt == 3:
        lo, ext, hcell = rd(np.float32, 3), rd(np.float32, 3), float(rd(np.float32, 1)[0])
        m = rd(np.int32, 4)
        mesh = dict(lo=lo, ext=ext, hcell=hcell, npst=int(m[3]), ST=rd(np.float32, 9 * m[0]).reshape(-1, 9),
                    STN=rd(np.float32, 4 * m[0]).reshape(-1, 4), BN=rd(np.float32, 8 * m[1]).reshape(-1, 8),
                    HK=rd(np.uint64, m[2]), HV=rd(np.int32, m[2]))
    L = rd(np.float32, 3 * NL).reshape(NL, 3)
    A = rd(np.float32, Np)
    region = rd(np.int32, Np)
    states = []
    for _ in range(NS):
        st = State(inten=rd(np.float32, NL), P=rd(np.float32, 3 * Np).reshape(Np, 3), N=rd(np.float32, 3 * Np).reshape(Np, 3),
                   Q=rd(np.float32, 12 * Nq).reshape(Nq, 12), dims=rd(np.int32, 2 * Nq).reshape(Nq, 2), off=rd(np.int32, Nq),
                   T=rd(np.float32, 9 * Nt).reshape(Nt, 9), TQ=rd(np.int32, Nt))
        if has_ref:
            st.ref, st.valid, st.Pw = rd(np.float32, Np), rd(np.uint8, Np), rd(np.float32, NL * Np).reshape(Np, NL)
        states.append(st)
    occ, em = {}, {}
    for a in range(NS):
        for c in range(NS):
            n = int(rd(np.int32, 1)[0])
            occ[(a, c)] = rd(np.int32, n)
            for l in range(NL):
                n = int(rd(np.int32, 1)[0])
                em[(a, c, l)] = rd(np.int32, n)
    if off != len(data):
        raise ValueError("trailing bytes in scene")
    return Scene(NR=NR, L=L, A=A, region=region, states=states, occ=occ, em=em, fmt=fmt, mesh=mesh)


# ------------------------------------------------------------------------------ generator
def _box_quads(lo, hi, with_bottom=False):
    """Outward quads (o, u, v, n) of an axis-aligned box; u x v points along n."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    dx, dy, dz = x1 - x0, y1 - y0, z1 - z0
    q = [
        ((x1, y0, z0), (0, dy, 0), (0, 0, dz), (1, 0, 0)),
        ((x0, y0, z0), (0, 0, dz), (0, dy, 0), (-1, 0, 0)),
        ((x0, y1, z0), (0, 0, dz), (dx, 0, 0), (0, 1, 0)),
        ((x0, y0, z0), (dx, 0, 0), (0, 0, dz), (0, -1, 0)),
        ((x0, y0, z1), (dx, 0, 0), (0, dy, 0), (0, 0, 1)),
    ]
    if with_bottom:
        q.append(((x0, y0, z0), (0, dy, 0), (dx, 0, 0), (0, 0, -1)))
    return q


def _room_quads():
    """Inward-facing walls of the 8 x 4 x 3 m room (floor, ceiling, four walls)."""
    return [
        ((0, 0, 0), (8, 0, 0), (0, 4, 0), (0, 0, 1)),
        ((0, 4, 3), (8, 0, 0), (0, -4, 0), (0, 0, -1)),
        ((0, 0, 0), (0, 0, 3), (8, 0, 0), (0, 1, 0)),
        ((8, 4, 0), (0, 0, 3), (-8, 0, 0), (0, -1, 0)),
        ((0, 4, 0), (0, 0, 3), (0, -4, 0), (1, 0, 0)),
        ((8, 0, 0), (0, 0, 3), (0, 4, 0), (-1, 0, 0)),
    ]


def _fine_voxels_of_box(lo, hi):
    out = set()
    for i in range(FX):
        for j in range(FY):
            for k in range(FZ):
                a0, a1 = i * X1 / FX, (i + 1) * X1 / FX
                b0, b1 = j * Y1 / FY, (j + 1) * Y1 / FY
                c0, c1 = k * Z1 / FZ, (k + 1) * Z1 / FZ
                if a1 > lo[0] and a0 < hi[0] and b1 > lo[1] and b0 < hi[1] and c1 > lo[2] and c0 < hi[2]:
                    out.add((k * FY + j) * FX + i)
    return sorted(out)


def _fine_voxel(p):
    i = min(max(int(p[0] / X1 * FX), 0), FX - 1)
    j = min(max(int(p[1] / Y1 * FY), 0), FY - 1)
    k = min(max(int(p[2] / Z1 * FZ), 0), FZ - 1)
    return (k * FY + j) * FX + i


def box_room(points: int = 1_082_802, boxes: int = 4, seed: int = 0, lights: int = 3, region_m: float = 0.55) -> Scene:
    """Seeded box room in the reference's format 2: an 8 x 4 x 3 m room, `boxes` static boxes and
    one movable box (5 faces each; 6 + 5 (boxes + 1) quads, two triangles per quad), point
    lights, albedo U[0.5, 0.8] per quad, cache points on a regular grid of every quad sized so
    the total is close to `points`.  Five states, the event kinds of the reference's box scenes:

        0 base lights          1 light 0 off          2 light 0 off, box moved
        3 light 0 on, box moved 4 base lights, box back, light 1 brighter
    """
    rng = np.random.default_rng(seed)
    static = []
    for _ in range(boxes):
        for _ in range(100):
            sx, sy, sz = rng.uniform(0.4, 1.4), rng.uniform(0.4, 1.2), rng.uniform(0.5, 2.2)
            x0, y0 = rng.uniform(0.3, 8 - 0.3 - sx), rng.uniform(0.3, 4 - 0.3 - sy)
            cand = (np.array([x0, y0, 0.0]), np.array([x0 + sx, y0 + sy, sz]))
            if all(cand[1][0] < b[0][0] - 0.2 or cand[0][0] > b[1][0] + 0.2 or cand[1][1] < b[0][1] - 0.2 or cand[0][1] > b[1][1] + 0.2
                   for b in static):
                static.append(cand)
                break
    # movable box: two positions clear of the static boxes
    mv_size = np.array([0.8, 0.8, 0.8])
    pos = []
    for _ in range(400):
        x0, y0 = rng.uniform(0.3, 8 - 0.3 - mv_size[0]), rng.uniform(0.3, 4 - 0.3 - mv_size[1])
        lo = np.array([x0, y0, 0.0])
        hi = lo + mv_size
        if all(hi[0] < b[0][0] - 0.1 or lo[0] > b[1][0] + 0.1 or hi[1] < b[0][1] - 0.1 or lo[1] > b[1][1] + 0.1 for b in static) and \
                all(np.abs(lo - p[0]).max() > 1.5 for p in pos):
            pos.append((lo, hi))
        if len(pos) == 2:
            break
    if len(pos) < 2:
        raise RuntimeError("no room for the movable box")
    L = np.array([[6.6, 3.0, 2.6], [1.0, 1.0, 2.6], [6.2, 0.7, 1.2]] + [[rng.uniform(0.5, 7.5), rng.uniform(0.5, 3.5), rng.uniform(1.5, 2.8)]
                                                                        for _ in range(max(0, lights - 3))], np.float32)[:lights]
    base = np.array([12.0, 3.0, 5.0] + [4.0] * max(0, lights - 3), np.float32)[:lights]
    inten = [base.copy() for _ in range(5)]
    inten[1][0] = 0
    inten[2][0] = 0
    if lights > 1:
        inten[4][1] = base[1] * 1.5
    box_at = [0, 0, 1, 1, 0]

    def quads_for(state):
        q = _room_quads()
        for lo, hi in static:
            q += _box_quads(lo, hi)
        q += _box_quads(*pos[box_at[state]])
        return q

    q0 = quads_for(0)
    Nq = len(q0)
    area = sum(np.linalg.norm(np.cross(np.array(u, float), np.array(v, float))) for _, u, v, _ in q0)
    h = np.sqrt(area / points)
    dims = []
    for o, u, v, n in q0:
        nu = max(1, int(round(np.linalg.norm(u) / h)))
        nv = max(1, int(round(np.linalg.norm(v) / h)))
        dims.append((nu, nv))
    dims = np.array(dims, np.int32)
    counts = dims[:, 0] * dims[:, 1]
    off = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int32)
    Np = int(counts.sum())
    alb_q = rng.uniform(0.5, 0.8, size=Nq).astype(np.float32)
    A = np.repeat(alb_q, counts).astype(np.float32)
    # regions: tiles of about region_m x region_m on every quad
    region = np.empty(Np, np.int32)
    nr = 0
    for qi, (o, u, v, n) in enumerate(q0):
        nu, nv = dims[qi]
        tu = max(1, int(round(np.linalg.norm(u) / region_m)))
        tv = max(1, int(round(np.linalg.norm(v) / region_m)))
        iu = np.arange(nu) * tu // nu
        iv = np.arange(nv) * tv // nv
        region[off[qi]: off[qi] + nu * nv] = (nr + iv[:, None] * tu + iu[None, :]).reshape(-1)
        nr += tu * tv
    states = []
    for s in range(5):
        qs = quads_for(s)
        Q = np.array([[*o, *u, *v, *n] for o, u, v, n in qs], np.float32)
        P = np.empty((Np, 3), np.float32)
        N = np.empty((Np, 3), np.float32)
        T = np.empty((2 * Nq, 9), np.float32)
        for qi in range(Nq):
            o, u, v, n = Q[qi, 0:3], Q[qi, 3:6], Q[qi, 6:9], Q[qi, 9:12]
            nu, nv = dims[qi]
            fu = ((np.arange(nu, dtype=np.float32) + np.float32(0.5)) / np.float32(nu)).astype(np.float32)
            fv = ((np.arange(nv, dtype=np.float32) + np.float32(0.5)) / np.float32(nv)).astype(np.float32)
            pts = o[None, None, :] + u[None, None, :] * fu[None, :, None] + v[None, None, :] * fv[:, None, None]
            P[off[qi]: off[qi] + nu * nv] = pts.reshape(-1, 3)
            N[off[qi]: off[qi] + nu * nv] = n
            T[2 * qi] = np.concatenate([o, u, v])
            T[2 * qi + 1] = np.concatenate([o + u + v, -u, -v])
        TQ = np.repeat(np.arange(Nq, dtype=np.int32), 2)
        states.append(State(inten=inten[s], P=P, N=N, Q=Q, dims=dims, off=off, T=T, TQ=TQ))
    occ, em = {}, {}
    for a in range(5):
        for b in range(5):
            if a != b and box_at[a] != box_at[b]:
                occ[(a, b)] = sorted(set(_fine_voxels_of_box(*pos[0])) | set(_fine_voxels_of_box(*pos[1])))
            for l in range(lights):
                if a != b and inten[a][l] == 0 and inten[b][l] > 0:
                    em[(a, b, l)] = [_fine_voxel(L[l])]
    return Scene(NR=nr, L=L, A=A, region=region, states=states, occ=occ, em=em, fmt=2)


# ------------------------------------------------------------------ format 3 (mesh scenes)
def _mix64(x: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser on uint64 arrays (the hash of the cache-point table)."""
    x = x.astype(np.uint64)
    with np.errstate(over="ignore"):
        x ^= x >> np.uint64(30)
        x *= np.uint64(0xBF58476D1CE4E5B9)
        x ^= x >> np.uint64(27)
        x *= np.uint64(0x94D049BB133111EB)
        x ^= x >> np.uint64(31)
    return x


def _cell_key(cx, cy, cz, b) -> np.ndarray:
    m = np.uint64(0xFFFFF)
    k = (cx.astype(np.int64).astype(np.uint64) & m)
    k = (k << np.uint64(20)) | (cy.astype(np.int64).astype(np.uint64) & m)
    k = (k << np.uint64(20)) | (cz.astype(np.int64).astype(np.uint64) & m)
    return ((k << np.uint64(3)) | b.astype(np.uint64)) + np.uint64(1)


def _normal_bucket(n: np.ndarray) -> np.ndarray:
    a = np.abs(n)
    out = np.where(n[:, 2] > 0, 4, 5)
    out = np.where((a[:, 1] >= a[:, 2]), np.where(n[:, 1] > 0, 2, 3), out)
    out = np.where((a[:, 0] >= a[:, 1]) & (a[:, 0] >= a[:, 2]), np.where(n[:, 0] > 0, 0, 1), out)
    return out.astype(np.int64)


def build_bvh(V: np.ndarray, leaf: int = 4):
    """Median-split BVH over triangles V (n, 3, 3).  Returns (nodes (K, 8) float32 in the
    reference's layout -- bmin, left child or first triangle as int bits, bmax, triangle count
    as int bits (0 for inner nodes, children at left and left + 1) -- and the triangle order)."""
    n = V.shape[0]
    tlo, thi = V.min(axis=1), V.max(axis=1)
    cen = 0.5 * (tlo + thi)
    order = np.arange(n)
    nodes = [None]
    stack = [(0, 0, n)]
    while stack:
        node, s, e = stack.pop()
        idx = order[s:e]
        lo, hi = tlo[idx].min(axis=0), thi[idx].max(axis=0)
        cnt = e - s
        c = cen[idx]
        ext = c.max(axis=0) - c.min(axis=0)
        ax = int(np.argmax(ext))
        if cnt <= leaf or (ext[ax] < 1e-7 and cnt <= 64):
            nodes[node] = (lo, s, hi, cnt)
            continue
        mid = cnt // 2
        part = np.argpartition(c[:, ax], mid)
        order[s:e] = idx[part]
        left = len(nodes)
        nodes += [None, None]
        nodes[node] = (lo, left, hi, 0)
        stack.append((left + 1, s + mid, e))
        stack.append((left, s, s + mid))
    out = np.zeros((len(nodes), 8), np.float32)
    for k, (lo, a, hi, cnt) in enumerate(nodes):
        out[k, 0:3] = lo
        out[k, 3] = np.array([a], np.int32).view(np.float32)[0]
        out[k, 4:7] = hi
        out[k, 7] = np.array([cnt], np.int32).view(np.float32)[0]
    return out, order


def mesh_scene(V: np.ndarray, alb: np.ndarray, double_sided: np.ndarray, lights: np.ndarray, intensities: list,
               box_pos: list, box_half: float, points: int, seed: int = 0, grid=(8, 4, 4)) -> Scene:
    """Format-3 scene from a static triangle mesh (the layout the reference's `prep` writes,
    cuda/prep_mesh.cuh:242-297): static triangles in BVH order with normals and double-sided
    flags, a BVH, cache points sampled on the surfaces into hash cells (cell side h, dominant
    normal bucket), the cell table with linear probing on mix64 of the cell key, 4x4x4-cell
    verification zones, a movable cube (6 quads, 12 dynamic triangles) whose two positions
    the states choose, and event voxel lists on the `grid` transit grid."""
    rng = np.random.default_rng(seed)
    V = np.asarray(V, np.float32)
    nt = V.shape[0]
    lo = V.reshape(-1, 3).min(axis=0)
    hi = V.reshape(-1, 3).max(axis=0)
    diag = float(np.linalg.norm(hi - lo))
    pad = 0.01 * diag + 0.05
    lo = (lo - pad).astype(np.float32)
    hi = (hi + pad).astype(np.float32)
    ext = (hi - lo).astype(np.float32)
    BN, order = build_bvh(V)
    Vo = V[order]
    ST = np.concatenate([Vo[:, 0], Vo[:, 1] - Vo[:, 0], Vo[:, 2] - Vo[:, 0]], axis=1).astype(np.float32)
    cr = np.cross(ST[:, 3:6].astype(np.float64), ST[:, 6:9].astype(np.float64))
    ln = np.linalg.norm(cr, axis=1)
    nrm = (cr / np.where(ln > 0, ln, 1.0)[:, None]).astype(np.float32)
    flags = np.asarray(double_sided, np.int32)[order]
    STN = np.concatenate([nrm, flags.view(np.float32)[:, None]], axis=1).astype(np.float32)
    # cache cells: area-proportional samples, cell keyed by position and normal bucket
    area = 0.5 * np.linalg.norm(np.cross((V[:, 1] - V[:, 0]).astype(np.float64), (V[:, 2] - V[:, 0]).astype(np.float64)), axis=1)
    sides = np.where(np.asarray(double_sided) > 0, 2, 1)
    h = float(np.sqrt((area * sides).sum() / points))
    ns = np.maximum(1, np.ceil(area / (h * h) * 4.0)).astype(np.int64)
    tri = np.repeat(np.arange(nt), ns)
    a = rng.random(tri.size)
    b = rng.random(tri.size)
    flip = a + b > 1
    a[flip], b[flip] = 1 - a[flip], 1 - b[flip]
    P = V[tri, 0] + (V[tri, 1] - V[tri, 0]) * a[:, None] + (V[tri, 2] - V[tri, 0]) * b[:, None]
    tn = np.cross((V[:, 1] - V[:, 0]).astype(np.float64), (V[:, 2] - V[:, 0]).astype(np.float64))
    tn = (tn / np.maximum(np.linalg.norm(tn, axis=1), 1e-30)[:, None])
    Ps, Ns, As = [P], [tn[tri]], [np.asarray(alb, np.float64)[tri]]
    ds = np.asarray(double_sided)[tri] > 0
    Ps.append(P[ds]); Ns.append(-tn[tri][ds]); As.append(np.asarray(alb, np.float64)[tri][ds])
    P = np.concatenate(Ps).astype(np.float32)
    Nn = np.concatenate(Ns).astype(np.float32)
    Al = np.concatenate(As)
    c = np.floor((P - lo) / np.float32(h)).astype(np.int64)
    ctr = lo + (c + 0.5) * np.float32(h)
    d2 = ((P - ctr) ** 2).sum(axis=1)
    keys = _cell_key(c[:, 0], c[:, 1], c[:, 2], _normal_bucket(Nn))
    srt = np.lexsort((d2, keys))
    ks = keys[srt]
    first = np.ones(ks.size, bool)
    first[1:] = ks[1:] != ks[:-1]
    rep = srt[first]
    ukeys = keys[rep]
    # albedo of a cell: mean over its samples
    inv = np.searchsorted(ukeys, keys[srt]) if False else None
    grp = np.cumsum(first) - 1
    asum = np.bincount(grp, weights=Al[srt])
    acnt = np.bincount(grp)
    Ast = (asum / acnt).astype(np.float32)
    Pst, Nst = P[rep], Nn[rep]
    npst = ukeys.size
    HS = 1024
    while HS < 2 * npst:
        HS <<= 1
    mask = HS - 1
    HK = np.zeros(HS, np.uint64)
    HV = np.full(HS, -1, np.int32)
    h0 = (_mix64(ukeys) & np.uint64(0xFFFFFFFF)).astype(np.int64) & mask
    for i in range(npst):
        j = int(h0[i])
        while HK[j] != 0:
            j = (j + 1) & mask
        HK[j] = ukeys[i]
        HV[j] = i
    cx = ((ukeys - np.uint64(1)) >> np.uint64(43)).astype(np.int64) & 0xFFFFF
    cy = ((ukeys - np.uint64(1)) >> np.uint64(23)).astype(np.int64) & 0xFFFFF
    cz = ((ukeys - np.uint64(1)) >> np.uint64(3)).astype(np.int64) & 0xFFFFF
    bk = ((ukeys - np.uint64(1)) & np.uint64(7)).astype(np.int64)
    zkey = _cell_key(cx >> 2, cy >> 2, cz >> 2, bk)
    _, zone = np.unique(zkey, return_inverse=True)
    NR = int(zone.max()) + 1
    # movable cube: 6 quads, bnu x bnu points per face, 4 x 4 points per zone
    bnu = max(2, int(round(2 * box_half / h)))
    nbox = 6 * bnu * bnu
    tu = (bnu + 3) // 4
    cube_region = []
    for q in range(6):
        for iv in range(bnu):
            for iu in range(bnu):
                cube_region.append(NR + q * tu * tu + (iv // 4) * tu + iu // 4)
    NR += 6 * tu * tu
    A = np.concatenate([Ast, np.full(nbox, 0.7, np.float32)])
    region = np.concatenate([zone.astype(np.int32), np.array(cube_region, np.int32)])
    Np = npst + nbox
    L = np.asarray(lights, np.float32).reshape(-1, 3)
    states = []
    for si, inten in enumerate(intensities):
        cpos = np.asarray(box_pos[si], np.float32)
        quads = _box_quads(cpos - box_half, cpos + box_half, with_bottom=True)
        Q = np.array([[*o, *u, *v, *n] for o, u, v, n in quads], np.float32)
        Pc, Nc, T = [], [], []
        for qi in range(6):
            o, u, v, n = Q[qi, 0:3], Q[qi, 3:6], Q[qi, 6:9], Q[qi, 9:12]
            f = ((np.arange(bnu, dtype=np.float32) + np.float32(0.5)) / np.float32(bnu)).astype(np.float32)
            pts = o[None, None, :] + u[None, None, :] * f[None, :, None] + v[None, None, :] * f[:, None, None]
            Pc.append(pts.reshape(-1, 3))
            Nc.append(np.repeat(n[None, :], bnu * bnu, axis=0))
            T.append(np.concatenate([o, u, v]))
            T.append(np.concatenate([o + u + v, -u, -v]))
        dims = np.full((6, 2), bnu, np.int32)
        off = (npst + np.arange(6) * bnu * bnu).astype(np.int32)
        states.append(State(inten=np.asarray(inten, np.float32), P=np.concatenate([Pst] + Pc).astype(np.float32),
                            N=np.concatenate([Nst] + Nc).astype(np.float32), Q=Q, dims=dims, off=off,
                            T=np.array(T, np.float32), TQ=np.repeat(np.arange(6, dtype=np.int32), 2)))
    VX, VY, VZ = grid

    def vox(p):
        i = min(max(int((p[0] - lo[0]) / ext[0] * VX), 0), VX - 1)
        j = min(max(int((p[1] - lo[1]) / ext[1] * VY), 0), VY - 1)
        k = min(max(int((p[2] - lo[2]) / ext[2] * VZ), 0), VZ - 1)
        return (k * VY + j) * VX + i

    occ, em = {}, {}
    NS = len(intensities)
    for a_ in range(NS):
        for b_ in range(NS):
            if a_ != b_ and tuple(box_pos[a_]) != tuple(box_pos[b_]):
                vs = set()
                for p in (box_pos[a_], box_pos[b_]):
                    for x in np.linspace(-box_half, box_half, 12):
                        for y in np.linspace(-box_half, box_half, 12):
                            for z in np.linspace(-box_half, box_half, 12):
                                vs.add(vox(np.array(p, np.float32) + np.array([x, y, z], np.float32)))
                occ[(a_, b_)] = sorted(vs)
            for l in range(L.shape[0]):
                if a_ != b_ and intensities[a_][l] == 0 and intensities[b_][l] > 0:
                    em[(a_, b_, l)] = [vox(L[l])]
    mesh = dict(lo=lo, ext=ext, hcell=np.float32(h), npst=npst, ST=ST, STN=STN, BN=BN, HK=HK, HV=HV)
    return Scene(NR=NR, L=L, A=A, region=region, states=states, occ=occ, em=em, fmt=3, mesh=mesh)


def street_mesh(buildings: int = 40, seed: int = 0, facade_cell: float = 2.0, size: float = 120.0):
    """Seeded street: a ground plane (split into a grid of quads) and `buildings` boxes 5-30 m
    tall along two rows, their facades subdivided into cells of about `facade_cell` metres.
    Returns (V (n, 3, 3) float32, albedo per triangle, double-sided flags)."""
    rng = np.random.default_rng(seed)
    tris, albs = [], []

    def quad(o, u, v, alb, nu, nv):
        o, u, v = (np.asarray(x, np.float64) for x in (o, u, v))
        for j in range(nv):
            for i in range(nu):
                a = o + u * (i / nu) + v * (j / nv)
                du, dv = u / nu, v / nv
                tris.append([a, a + du, a + dv])
                tris.append([a + du + dv, a + dv, a + du])
                albs.extend([alb, alb])

    g = max(1, int(size / 8))
    quad((-size / 2, -size / 2, 0), (size, 0, 0), (0, size, 0), 0.35, g, g)
    for b in range(buildings):
        side = 1 if b % 2 else -1
        x0 = -size / 2 + 4 + (b // 2) * (size - 8) / max(1, buildings // 2)
        w = rng.uniform(6, (size - 8) / max(1, buildings // 2) - 1)
        d = rng.uniform(8, 16)
        hgt = rng.uniform(5, 30)
        y0 = side * 8 if side > 0 else -8 - d
        alb = rng.uniform(0.2, 0.8)
        lo = np.array([x0, y0, 0.0])
        hi = np.array([x0 + w, y0 + d, hgt])
        for o, u, v, n in _box_quads(lo, hi):
            nu = max(1, int(np.linalg.norm(u) / facade_cell))
            nv = max(1, int(np.linalg.norm(v) / facade_cell))
            quad(o, u, v, alb, nu, nv)
    V = np.array(tris, np.float32)
    return V, np.array(albs, np.float32), np.zeros(len(tris), np.uint8)


def city_mesh(buildings: int = 400, seed: int = 0, facade_cell: float = 1.6, block: float = 32.0, street: float = 10.0):
    """Seeded city: a square grid of sqrt(buildings)^2 blocks separated by streets, one box
    building per block (footprint 50-90 % of the block, 5-60 m tall), facades subdivided into
    cells of about `facade_cell` metres, on a ground plane split into 8 m quads.  About 1 M
    triangles with the defaults.  Returns (V (n, 3, 3) float32, albedo per triangle,
    double-sided flags)."""
    rng = np.random.default_rng(seed)
    g = int(round(np.sqrt(buildings)))
    pitch = block + street
    size = g * pitch + street
    tris, albs = [], []

    def quad(o, u, v, alb, nu, nv):
        o, u, v = (np.asarray(x, np.float64) for x in (o, u, v))
        i, j = np.meshgrid(np.arange(nu), np.arange(nv), indexing="xy")
        a = o + u * (i.reshape(-1, 1) / nu) + v * (j.reshape(-1, 1) / nv)
        du, dv = u / nu, v / nv
        t1 = np.stack([a, a + du, a + dv], 1)
        t2 = np.stack([a + du + dv, a + dv, a + du], 1)
        tris.append(np.stack([t1, t2], 1).reshape(-1, 3, 3))
        albs.append(np.full(2 * nu * nv, alb))

    cells = max(1, int(size / 8))
    quad((-size / 2, -size / 2, 0), (size, 0, 0), (0, size, 0), 0.3, cells, cells)
    for by in range(g):
        for bx in range(g):
            w = rng.uniform(0.5, 0.9) * block
            d = rng.uniform(0.5, 0.9) * block
            hgt = rng.uniform(5, 60)
            x0 = -size / 2 + street + bx * pitch + rng.uniform(0, block - w)
            y0 = -size / 2 + street + by * pitch + rng.uniform(0, block - d)
            alb = rng.uniform(0.2, 0.8)
            for o, u, v, n in _box_quads(np.array([x0, y0, 0.0]), np.array([x0 + w, y0 + d, hgt])):
                nu = max(1, int(np.linalg.norm(u) / facade_cell))
                nv = max(1, int(np.linalg.norm(v) / facade_cell))
                quad(o, u, v, alb, nu, nv)
    V = np.concatenate(tris).astype(np.float32)
    return V, np.concatenate(albs).astype(np.float32), np.zeros(len(V), np.uint8)


def street_scene(points: int = 20000, buildings: int = 8, seed: int = 0, facade_cell: float = 2.0, size: float = 60.0,
                 lights: int = 3) -> Scene:
    """Format-3 street scene: street_mesh + three lamp-post lights and the movable cube; five
    states as the reference's prep (lights {0,1} on, 1 off, cube moved, light 2 on first time,
    light 0 off with the cube moved).  With lights > 3 the extra lamps stand along the street
    (4-6 m high, seeded), emission U[1, 50], on in every state."""
    V, alb, ds = street_mesh(buildings, seed, facade_cell, size)
    L = [[-size / 4, 0.0, 4.0], [0.0, 2.0, 4.0], [size / 4, -2.0, 4.0]][:lights]
    I = [[20, 20, 0], [0, 20, 0], [20, 20, 0], [20, 20, 20], [0, 20, 0]]
    I = [row[:lights] for row in I]
    if lights > 3:
        rng = np.random.default_rng(seed + 1000)
        for _ in range(lights - 3):
            L.append([rng.uniform(-size / 2 + 2, size / 2 - 2), rng.uniform(-5.0, 5.0), rng.uniform(4.0, 6.0)])
        extra = rng.uniform(1.0, 50.0, lights - 3).round(3).tolist()
        I = [row + extra for row in I]
    L = np.array(L, np.float32)
    box = [(-2.0, 0.0, 1.0), (-2.0, 0.0, 1.0), (4.0, -1.0, 1.0), (-2.0, 0.0, 1.0), (4.0, -1.0, 1.0)]
    return mesh_scene(V, alb, ds, L, I, box, 1.0, points, seed)


def with_references(scene: Scene, ctx) -> Scene:
    """The scene with the converged references a context computed for it
    (``native.Context.build_reference`` on this scene): ref, valid and the per-light warm
    start of every state, so that the written file carries them (has_ref = 1)."""
    from . import native as N
    nl = scene.NL
    for k, st in enumerate(scene.states):
        st.ref = ctx.state_array(k, N.SA_REF).astype(np.float32)
        st.valid = ctx.state_array(k, N.SA_VALID).astype(np.uint8)
        st.Pw = ctx.state_array(k, N.SA_PW).reshape(-1, nl).astype(np.float32)
    return scene


def write_msh1(V: np.ndarray, albedo: np.ndarray, double_sided: np.ndarray) -> bytes:
    """A mesh in the MSH1 layout the `prep` mode reads (prep_mesh.cuh:22-29): "MSH1", the
    triangle count, 9 floats per triangle (metres, z up), one albedo per triangle, one
    double-sided byte per triangle."""
    V = np.ascontiguousarray(V, np.float32).reshape(-1, 9)
    n = len(V)
    return (b"MSH1" + np.int32(n).tobytes() + V.tobytes() + np.ascontiguousarray(albedo, np.float32).reshape(n).tobytes()
            + np.ascontiguousarray(double_sided, np.uint8).reshape(n).tobytes())
