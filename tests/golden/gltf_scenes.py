"""Small synthetic glTF 2.0 scenes for the glTF -> MSH1 converter's tests (render_engine_gb300/gltf.py).

Each scene exercises rules of the converter: node hierarchies with matrices and TRS, instancing,
a mirrored instance, every material kind (metallic-roughness with and without texture,
specular-glossiness, BLEND, transmission, MASK, no material), double-sided materials, non-triangle
primitives, non-indexed primitives, 8/16/32-bit indices, interleaved vertex buffers, data-URI and
external buffers (with a percent-encoded file name), centimetre units, degenerate triangles, a file
without a scene list, normalized integer positions, index counts that are not a multiple of 3 and
accessors without a buffer view.

`write_all(directory)` writes them (.gltf, plus the external .bin); `to_glb(path, out)` packs a
single-buffer scene as a binary .glb.  Used by tests/golden/make_gltf_golden.py (which runs the
reference's converter on them) and by the tests.
"""
import base64
import json
import math
import os
import struct

import numpy as np

FLOAT, U8, U16, U32 = 5126, 5121, 5123, 5125


class Builder:
    """Accumulates binary data into numbered buffers and describes it as views and accessors."""

    def __init__(self):
        self.meta = {"asset": {"version": "2.0", "generator": "render_engine_gb300 tests"}, "buffers": [], "bufferViews": [],
                     "accessors": [], "meshes": [], "nodes": [], "materials": []}
        self.data = []

    def buffer(self):
        self.data.append(bytearray())
        self.meta["buffers"].append({})
        return len(self.data) - 1

    def view(self, buf, raw, stride=None):
        b = self.data[buf]
        while len(b) % 4:
            b.append(0)
        v = {"buffer": buf, "byteOffset": len(b), "byteLength": len(raw)}
        if stride:
            v["byteStride"] = stride
        b.extend(raw)
        self.meta["bufferViews"].append(v)
        return len(self.meta["bufferViews"]) - 1

    def accessor(self, view, ctype, kind, count, offset=0, normalized=False, minmax=None):
        a = {"componentType": ctype, "type": kind, "count": count}
        if view is not None:
            a["bufferView"] = view
        if offset:
            a["byteOffset"] = offset
        if normalized:
            a["normalized"] = True
        if minmax is not None:
            a["min"], a["max"] = [float(x) for x in minmax[0]], [float(x) for x in minmax[1]]
        self.meta["accessors"].append(a)
        return len(self.meta["accessors"]) - 1

    def positions(self, buf, P):
        P = np.ascontiguousarray(P, np.float32)
        return self.accessor(self.view(buf, P.tobytes()), FLOAT, "VEC3", len(P), minmax=(P.min(0), P.max(0)))

    def indices(self, buf, I, ctype):
        dt = {U8: np.uint8, U16: np.uint16, U32: np.uint32}[ctype]
        I = np.ascontiguousarray(I, dt).reshape(-1)
        return self.accessor(self.view(buf, I.tobytes()), ctype, "SCALAR", len(I))

    def material(self, **m):
        self.meta["materials"].append(m)
        return len(self.meta["materials"]) - 1

    def mesh(self, *prims):
        self.meta["meshes"].append({"primitives": list(prims)})
        return len(self.meta["meshes"]) - 1

    def node(self, **n):
        self.meta["nodes"].append(n)
        return len(self.meta["nodes"]) - 1

    def write(self, path, external=None):
        """Write the .gltf; buffer `k` in `external` (name -> index) goes to a file of that name
        (its URI percent-encoded), the others are embedded as data URIs."""
        base = os.path.dirname(os.path.abspath(path))
        external = external or {}
        for k, raw in enumerate(self.data):
            self.meta["buffers"][k]["byteLength"] = len(raw)
            names = [n for n, i in external.items() if i == k]
            if names:
                with open(os.path.join(base, names[0]), "wb") as f:
                    f.write(bytes(raw))
                self.meta["buffers"][k]["uri"] = names[0].replace(" ", "%20")
            else:
                self.meta["buffers"][k]["uri"] = "data:application/octet-stream;base64," + base64.b64encode(bytes(raw)).decode()
        with open(path, "w") as f:
            json.dump(self.meta, f, indent=1)


def box(lo, hi, inward=False):
    """12 triangles of an axis-aligned box (shared corners, 8 vertices)."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    P = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], np.float32)
    faces = [(0, 3, 2, 1), (4, 5, 6, 7), (0, 1, 5, 4), (3, 7, 6, 2), (0, 4, 7, 3), (1, 2, 6, 5)]
    I = []
    for a, b, c, d in faces:
        t = [(a, b, c), (a, c, d)]
        I += [(x, z, y) for x, y, z in t] if inward else t
    return P, np.array(I, np.int64)


def quat_y(deg):
    h = math.radians(deg) / 2
    return [0.0, math.sin(h), 0.0, math.cos(h)]


def hierarchy(directory):
    """Rooms, crates, panels; every material kind; instancing and a mirrored instance."""
    g = Builder()
    ext, emb = g.buffer(), g.buffer()
    m_wall = g.material(pbrMetallicRoughness={"baseColorFactor": [0.8, 0.7, 0.6, 1.0]})
    m_tex = g.material(pbrMetallicRoughness={"baseColorFactor": [0.9, 0.9, 0.9, 1.0], "baseColorTexture": {"index": 0}})
    m_blend = g.material(alphaMode="BLEND", pbrMetallicRoughness={"baseColorFactor": [1, 1, 1, 0.3]})
    m_gloss = g.material(doubleSided=True, extensions={"KHR_materials_pbrSpecularGlossiness": {"diffuseFactor": [0.2, 0.5, 0.3, 1]}})
    m_glass = g.material(extensions={"KHR_materials_transmission": {"transmissionFactor": 0.9}})
    m_mask = g.material(alphaMode="MASK", doubleSided=True, pbrMetallicRoughness={"baseColorFactor": [0.1, 0.6, 0.1, 1],
                                                                                  "baseColorTexture": {"index": 1}})
    m_dark = g.material(pbrMetallicRoughness={"baseColorFactor": [0.01, 0.01, 0.01, 1]})
    # room: 8 x 3 x 4 m (y up), faces inward, 16-bit indices, external buffer
    P, I = box((0, 0, 0), (8, 3, 4), inward=True)
    room = g.mesh({"attributes": {"POSITION": g.positions(ext, P)}, "indices": g.indices(ext, I, U16), "material": m_wall})
    # crate: 24 vertices interleaved with normals (stride 24), 8-bit indices; a BLEND primitive
    # and a line primitive beside it
    Pc, Ic = box((-0.5, 0, -0.5), (0.5, 1, 0.5))
    Pv = Pc[Ic.reshape(-1)]                                      # 36 unshared vertices
    Nv = np.repeat(np.eye(3, dtype=np.float32), 12, axis=0)
    inter = np.concatenate([Pv, Nv], axis=1).astype(np.float32)
    vw = g.view(ext, inter.tobytes(), stride=24)
    apos = g.accessor(vw, FLOAT, "VEC3", 36, minmax=(Pv.min(0), Pv.max(0)))
    anrm = g.accessor(vw, FLOAT, "VEC3", 36, offset=12)
    ilocal = np.arange(36)
    crate = g.mesh({"attributes": {"POSITION": apos, "NORMAL": anrm}, "indices": g.indices(ext, ilocal, U8), "material": m_tex},
                   {"attributes": {"POSITION": apos}, "indices": g.indices(ext, ilocal[:6], U8), "material": m_blend},
                   {"attributes": {"POSITION": apos}, "indices": g.indices(ext, ilocal[:8], U8), "material": m_wall, "mode": 1})
    # panel: a non-indexed double-sided quad, data-URI buffer
    Pq = np.array([[0, 0, 0], [1.5, 0, 0], [1.5, 1, 0], [0, 0, 0], [1.5, 1, 0], [0, 1, 0]], np.float32)
    panel = g.mesh({"attributes": {"POSITION": g.positions(emb, Pq)}, "material": m_gloss})
    glass = g.mesh({"attributes": {"POSITION": g.positions(emb, Pq)}, "material": m_glass})
    # leaves: 32-bit indices, MASK material; a primitive without material beside a dark one
    Pl, Il = box((0, 0, 0), (0.6, 0.2, 0.6))
    leaves = g.mesh({"attributes": {"POSITION": g.positions(emb, Pl)}, "indices": g.indices(emb, Il, U32), "material": m_mask},
                    {"attributes": {"POSITION": g.positions(emb, Pl * 0.5)}, "indices": g.indices(emb, Il, U16)},
                    {"attributes": {"POSITION": g.positions(emb, Pl + 1.0)}, "indices": g.indices(emb, Il, U16), "material": m_dark})
    n_room = g.node(mesh=room, name="room")
    n_mirror = g.node(mesh=crate, scale=[-1.0, 1.0, 1.0], translation=[1.0, 0.0, 0.5], name="mirrored crate")
    M = np.eye(4)
    M[:3, 3] = (2.0, 0.0, 1.0)
    c, s = math.cos(0.4), math.sin(0.4)
    M[:3, :3] = [[c, 0, s], [0, 1, 0], [-s, 0, c]]
    n_crate = g.node(mesh=crate, matrix=[float(x) for x in M.T.reshape(-1)], children=[n_mirror], name="crate")
    n_panel = g.node(mesh=panel, translation=[4.0, 0.5, 3.9], rotation=quat_y(180.0), scale=[1.0, 1.2, 1.0], name="panel")
    n_root = g.node(children=[n_room, n_crate, n_panel], translation=[0.25, 0.0, -0.5], rotation=quat_y(30.0), name="root")
    n_glass = g.node(mesh=glass, translation=[3, 1, 2])
    n_nomat = g.node(mesh=leaves, translation=[5, 0, 1], scale=[1, 2, 1])
    n_leaves = g.node(mesh=leaves, translation=[6, 2, 3], children=[n_nomat])
    g.node(mesh=room, name="unused, only in the second scene")
    g.meta["scenes"] = [{"nodes": [n_root, n_glass, n_leaves]}, {"nodes": [len(g.meta["nodes"]) - 1]}]
    g.meta["scene"] = 0
    g.write(os.path.join(directory, "hierarchy.gltf"), external={"geometry data.bin": ext})


def centimetres(directory):
    """A 12 x 3 x 8 m hall modelled in centimetres, one degenerate triangle, one data-URI buffer."""
    g = Builder()
    b = g.buffer()
    m = g.material(pbrMetallicRoughness={"baseColorFactor": [0.5, 0.5, 0.5, 1]})
    P, I = box((0, 0, 0), (1200, 300, 800), inward=True)
    P2, I2 = box((100, 0, 100), (180, 120, 160))
    Pd = np.array([[10, 0, 10], [20, 0, 20], [30, 0, 30]], np.float32)   # collinear: zero area
    PA = np.concatenate([P, P2 + 0.0, Pd])
    IA = np.concatenate([I, I2 + 8, np.array([[16, 17, 18]])])
    mesh = g.mesh({"attributes": {"POSITION": g.positions(b, PA)}, "indices": g.indices(b, IA, U16), "material": m})
    g.node(mesh=mesh)
    g.meta["scenes"] = [{"nodes": [0]}]
    g.write(os.path.join(directory, "centimetres.gltf"))


def noscene(directory):
    """No scene list (every node is a root, so a child is placed once more on its own), normalized
    16-bit positions, an index count that is not a multiple of 3, an accessor without a buffer view."""
    g = Builder()
    b = g.buffer()
    P, I = box((0.1, 0.0, 0.1), (0.9, 0.5, 0.7))
    Q = np.round(P * 65535).astype(np.uint16)
    apos = g.accessor(g.view(b, Q.tobytes()), U16, "VEC3", len(Q), normalized=True, minmax=(Q.min(0), Q.max(0)))
    ragged = np.concatenate([I.reshape(-1), [0, 1]])             # 38 indices: the last two are dropped
    zeros = g.accessor(None, FLOAT, "VEC3", 6)
    mesh = g.mesh({"attributes": {"POSITION": apos}, "indices": g.indices(b, ragged, U16)},
                  {"attributes": {"POSITION": zeros}})
    child = 1
    g.node(mesh=mesh, scale=[4.0, 4.0, 4.0], children=[child])
    g.node(mesh=mesh, translation=[0.0, 0.0, 5.0])
    g.write(os.path.join(directory, "noscene.gltf"))


SCENES = {"hierarchy.gltf": hierarchy, "centimetres.gltf": centimetres, "noscene.gltf": noscene}


def write_all(directory):
    os.makedirs(directory, exist_ok=True)
    for fn in SCENES.values():
        fn(directory)
    return sorted(SCENES)


def to_glb(path, out):
    """Pack a scene whose only buffer is a data URI as a binary .glb (JSON chunk, BIN chunk)."""
    with open(path) as f:
        meta = json.load(f)
    assert len(meta["buffers"]) == 1
    raw = base64.b64decode(meta["buffers"][0]["uri"].split(",", 1)[1])
    del meta["buffers"][0]["uri"]
    js = json.dumps(meta).encode()
    js += b" " * (-len(js) % 4)
    raw += b"\0" * (-len(raw) % 4)
    body = struct.pack("<II", len(js), 0x4E4F534A) + js + struct.pack("<II", len(raw), 0x004E4942) + raw
    with open(out, "wb") as f:
        f.write(struct.pack("<III", 0x46546C67, 2, 12 + len(body)) + body)
