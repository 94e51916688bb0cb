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
import struct
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
