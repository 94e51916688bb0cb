"""glTF 2.0 scene -> MSH1 triangle mesh, the input of the `prep` mode.

The counterpart of the reference's scenes_publiques/convertir.py (the step run_cuda.sh runs before
`poc_gpu_l3 prep` on a public scene, run_cuda.sh:99-103): same command line, same output bytes,
same summary line.

    python -m render_engine_gb300.gltf <scene.gltf|scene.glb> <out.mesh> [--echelle S]

What a scene becomes (each rule is the reference converter's, so that the same scene prepares into
the same bench scene):

* every node of the default scene (every node of the file as a root when it has no scene list) is
  walked depth first, a node's own primitives before its children, with its matrix or its
  translation / rotation / scale composed onto its parent's; a mesh used by several nodes is
  placed once per node;
* only triangle lists are kept (primitive mode 4); an instance whose matrix mirrors (negative
  determinant) has its second and third vertices swapped, so that the faces keep their side;
* each triangle's albedo is the luminance (0.2126, 0.7152, 0.0722) of its material's base colour
  factor (baseColorFactor, or diffuseFactor of a specular-glossiness material), halved when the
  material has a colour texture (textures are not read), then clamped to [0.05, 0.85]; a primitive
  without material gets 0.6; materials that let light through (alphaMode BLEND, or a transmission
  factor above 0) are left out, MASK materials are kept opaque; doubleSided is kept;
* glTF's y-up frame becomes the bench's z-up one, (x, y, z) -> (x, -z, y) (a proper rotation);
  units are metres: a scene whose bounding-box diagonal exceeds 400 is taken to be in centimetres
  and scaled by 0.01 unless --echelle gives the factor;
* triangles whose doubled area (|e1 x e2| in float32) is not above 1e-10 are dropped.

Accessor reading follows the reference converter too: strided buffer views, integer components
marked `normalized` divided by their type's maximum, accessors without a buffer view read as
zeros, sparse substitutions not applied.  Beyond the reference, a binary .glb container is read as
well (its JSON chunk and its BIN chunk as buffer 0), and percent-encoded buffer file names are
decoded in full.

MSH1 (little endian): "MSH1", int32 n, float32[n][9] vertices, float32[n] albedo, uint8[n]
double-sided (scene.write_msh1).
"""
from __future__ import annotations

import base64
import json
import os
import struct
import sys
import urllib.parse

import numpy as np

from .scene import write_msh1

_COMPONENT = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5125: np.uint32, 5126: np.float32}
_WIDTH = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT2": 4, "MAT3": 9, "MAT4": 16}
_LUMA = (0.2126, 0.7152, 0.0722)
_GLB_MAGIC, _GLB_JSON, _GLB_BIN = 0x46546C67, 0x4E4F534A, 0x004E4942
CENTIMETRE_DIAGONAL = 400.0


class GltfError(ValueError):
    """The file is not a glTF 2.0 scene this converter can read."""


class Document:
    """A parsed glTF: its JSON and its buffers (bytes)."""

    def __init__(self, meta: dict, buffers: list[bytes]):
        self.meta = meta
        self.buffers = buffers

    @classmethod
    def open(cls, path: str) -> "Document":
        with open(path, "rb") as f:
            raw = f.read()
        base = os.path.dirname(os.path.abspath(path))
        glb_bin = None
        if len(raw) >= 12 and struct.unpack_from("<I", raw, 0)[0] == _GLB_MAGIC:
            meta, glb_bin = _parse_glb(raw)
        else:
            meta = json.loads(raw.decode("utf-8"))
        buffers = []
        for k, b in enumerate(meta.get("buffers", [])):
            uri = b.get("uri")
            if uri is None:
                if k != 0 or glb_bin is None:
                    raise GltfError("buffer %d has no uri and no binary chunk" % k)
                buffers.append(glb_bin)
            elif uri.startswith("data:"):
                buffers.append(base64.b64decode(uri.split(",", 1)[1]))
            else:
                with open(os.path.join(base, urllib.parse.unquote(uri)), "rb") as f:
                    buffers.append(f.read())
        return cls(meta, buffers)

    def accessor(self, index: int) -> np.ndarray:
        """Accessor `index` as a (count, width) array of its component type (float32 when normalized)."""
        a = self.meta["accessors"][index]
        count, width, dtype = a["count"], _WIDTH[a["type"]], np.dtype(_COMPONENT[a["componentType"]])
        if "bufferView" not in a:
            return np.zeros((count, width), dtype)
        view = self.meta["bufferViews"][a["bufferView"]]
        buf = self.buffers[view["buffer"]]
        start = view.get("byteOffset", 0) + a.get("byteOffset", 0)
        row = dtype.itemsize * width
        stride = view.get("byteStride", row)
        if count == 0:
            out = np.zeros((0, width), dtype)
        elif stride == row:
            out = np.frombuffer(buf, dtype, count * width, start).reshape(count, width)
        else:
            rows = np.frombuffer(buf, np.uint8, (count - 1) * stride + row, start)
            out = np.lib.stride_tricks.as_strided(rows, (count, row), (stride, 1)).copy().view(dtype).reshape(count, width)
        if a.get("normalized") and dtype != np.float32:
            out = out.astype(np.float32) / np.iinfo(dtype).max
        return out


def _parse_glb(raw: bytes) -> tuple[dict, bytes | None]:
    magic, version, length = struct.unpack_from("<III", raw, 0)
    if version != 2:
        raise GltfError("binary glTF version %d (2 expected)" % version)
    pos, meta, binary = 12, None, None
    end = min(length, len(raw))
    while pos + 8 <= end:
        size, kind = struct.unpack_from("<II", raw, pos)
        chunk = raw[pos + 8:pos + 8 + size]
        if kind == _GLB_JSON and meta is None:
            meta = json.loads(chunk.decode("utf-8"))
        elif kind == _GLB_BIN and binary is None:
            binary = bytes(chunk)
        pos += 8 + size
    if meta is None:
        raise GltfError("binary glTF without a JSON chunk")
    return meta, binary


def _rotation(q) -> np.ndarray:
    """3x3 rotation of the unit quaternion (x, y, z, w)."""
    x, y, z, w = (float(c) for c in q)
    xx, yy, zz = x * x, y * y, z * z
    return np.array([[1 - 2 * (yy + zz), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (xx + zz), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (xx + yy)]])


def local_matrix(node: dict) -> np.ndarray:
    """The node's 4x4 transform (column-major `matrix`, else T * R * S)."""
    if "matrix" in node:
        return np.asarray(node["matrix"], np.float64).reshape(4, 4).T
    m = np.eye(4)
    m[:3, :3] = _rotation(node.get("rotation", (0.0, 0.0, 0.0, 1.0))) * np.asarray(node.get("scale", (1.0, 1.0, 1.0)), np.float64)[None, :]
    m[:3, 3] = node.get("translation", (0.0, 0.0, 0.0))
    return m


def material(meta: dict, index) -> tuple[float, bool, bool]:
    """(albedo, double-sided, lets light through) of material `index` (None: no material)."""
    if index is None:
        return 0.6, False, False
    m = meta["materials"][index]
    ext = m.get("extensions", {})
    gloss = ext.get("KHR_materials_pbrSpecularGlossiness")
    if gloss is not None:
        colour, textured = gloss.get("diffuseFactor", (1, 1, 1, 1)), "diffuseTexture" in gloss
    else:
        pbr = m.get("pbrMetallicRoughness", {})
        colour, textured = pbr.get("baseColorFactor", (1, 1, 1, 1)), "baseColorTexture" in pbr
    luma = _LUMA[0] * colour[0] + _LUMA[1] * colour[1] + _LUMA[2] * colour[2]
    albedo = min(0.85, max(0.05, luma * (0.5 if textured else 1.0)))
    through = ext.get("KHR_materials_transmission", {}).get("transmissionFactor", 0) > 0 or m.get("alphaMode") == "BLEND"
    return albedo, bool(m.get("doubleSided", False)), through


def walk(meta: dict):
    """(node index, world matrix) of every node instance, depth first, parents before children."""
    if "scenes" in meta:
        roots = meta["scenes"][meta.get("scene", 0)]["nodes"]
    else:
        roots = list(range(len(meta.get("nodes", []))))
    nodes = meta.get("nodes", [])
    stack = [(r, np.eye(4)) for r in reversed(roots)]
    while stack:
        k, parent = stack.pop()
        world = parent @ local_matrix(nodes[k])
        yield k, world
        for c in reversed(nodes[k].get("children", [])):
            stack.append((c, world))


def triangles(doc: Document) -> tuple[np.ndarray, np.ndarray, np.ndarray, int]:
    """World-space triangles (n, 3, 3) float32 in glTF axes, albedo, double-sided flags, and the
    number of primitives left out as transparent."""
    meta = doc.meta
    mats = [material(meta, k) for k in range(len(meta.get("materials", [])))]
    geometry = {}
    parts, albedo, sided = [], [], []
    through = 0
    for k, world in walk(meta):
        node = meta["nodes"][k]
        if "mesh" not in node:
            continue
        for prim in meta["meshes"][node["mesh"]]["primitives"]:
            if prim.get("mode", 4) != 4:
                continue
            mi = prim.get("material")
            alb, ds, tr = mats[mi] if mi is not None else material(meta, None)
            if tr:
                through += 1
                continue
            key = (prim["attributes"]["POSITION"], prim.get("indices"))
            if key not in geometry:
                pos = doc.accessor(key[0]).astype(np.float64)
                if key[1] is None:
                    idx = np.arange(len(pos))
                else:
                    idx = doc.accessor(key[1]).reshape(-1).astype(np.int64)
                ntri = len(idx) // 3
                geometry[key] = (pos, idx[:3 * ntri].reshape(ntri, 3))
            pos, idx = geometry[key]
            placed = pos @ world[:3, :3].T + world[:3, 3]
            tri = placed[idx]
            if np.linalg.det(world[:3, :3]) < 0:
                tri = tri[:, [0, 2, 1]]
            parts.append(tri.astype(np.float32))
            albedo.append(np.full(len(tri), alb, np.float32))
            sided.append(np.full(len(tri), 1 if ds else 0, np.uint8))
    if not parts:
        raise GltfError("the scene has no opaque triangles")
    return np.concatenate(parts), np.concatenate(albedo), np.concatenate(sided), through


def convert(src: str, dst: str | None = None, scale: float | None = None) -> tuple[np.ndarray, np.ndarray, np.ndarray, dict]:
    """Convert `src`; write the MSH1 mesh to `dst` when given.  Returns (vertices (n, 9) float32,
    albedo, double-sided, summary)."""
    doc = Document.open(src)
    tri, alb, ds, through = triangles(doc)
    # y up -> z up: (x, y, z) -> (x, -z, y)
    tri = tri[:, :, [0, 2, 1]]
    tri[:, :, 1] *= -1
    flat = tri.reshape(-1, 3)
    diag = float(np.linalg.norm(flat.max(0) - flat.min(0)))
    if scale is None:
        scale = 0.01 if diag > CENTIMETRE_DIAGONAL else 1.0
    V = tri.reshape(-1, 9)
    V *= scale
    e1, e2 = V[:, 3:6] - V[:, 0:3], V[:, 6:9] - V[:, 0:3]
    keep = np.linalg.norm(np.cross(e1, e2), axis=1) > 1e-10
    V, alb, ds = V[keep], alb[keep], ds[keep]
    if dst is not None:
        with open(dst, "wb") as f:
            f.write(write_msh1(V, alb, ds))
    pts = V.reshape(-1, 3)
    lo, hi = pts.min(0), pts.max(0)
    summary = {"type": "maillage", "source": os.path.basename(src), "triangles": int(len(V)),
               "transparents_ignores": through, "echelle": scale, "taille_m": [round(float(x), 2) for x in hi - lo],
               "double_face": round(float(ds.mean()), 3), "albedo_moyen": round(float(alb.mean()), 3)}
    return V, alb, ds, summary


def main(argv=None) -> int:
    args = list(sys.argv[1:] if argv is None else argv)
    scale = None
    if "--echelle" in args:
        k = args.index("--echelle")
        scale = float(args[k + 1])
        del args[k:k + 2]
    if len(args) != 2:
        sys.stderr.write(__doc__)
        return 2
    _, _, _, summary = convert(args[0], args[1], scale)
    print(json.dumps(summary))
    return 0


if __name__ == "__main__":
    sys.exit(main())
