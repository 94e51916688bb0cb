"""The glTF -> MSH1 converter (render_engine_gb300/gltf.py) against the reference's own converter.

tests/golden/gltf/ holds synthetic glTF scenes (tests/golden/gltf_scenes.py) and, for each, the mesh
and summary line that the reference's unmodified scenes_publiques/convertir.py wrote for it
(tests/golden/make_gltf_golden.py).  Ours must write the same bytes and the same summary.  The
scenes cover hierarchies with matrices and TRS, instancing, a mirrored instance, every material
kind, non-triangle and non-indexed primitives, 8/16/32-bit indices, interleaved buffers, external
and data-URI buffers, centimetre units, degenerate triangles, a file without a scene list,
normalized positions, ragged index counts and accessors without a buffer view."""
import json
import os
import shutil
import struct
import sys

import numpy as np
import pytest

from render_engine_gb300 import gltf

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "gltf")
sys.path.insert(0, os.path.join(HERE, "golden"))
import gltf_scenes  # noqa: E402

SCENES = ["hierarchy", "centimetres", "noscene"]


def _msh1(raw):
    assert raw[:4] == b"MSH1"
    n = struct.unpack_from("<i", raw, 4)[0]
    V = np.frombuffer(raw, np.float32, 9 * n, 8).reshape(n, 9)
    A = np.frombuffer(raw, np.float32, n, 8 + 36 * n)
    D = np.frombuffer(raw, np.uint8, n, 8 + 40 * n)
    assert len(raw) == 8 + 41 * n
    return V, A, D


@pytest.mark.parametrize("name", SCENES)
def test_same_mesh_as_the_reference_converter(tmp_path, name):
    out = tmp_path / (name + ".mesh")
    V, A, D, summary = gltf.convert(os.path.join(GOLD, name + ".gltf"), str(out))
    with open(os.path.join(GOLD, name + ".mesh"), "rb") as f:
        ref = f.read()
    mine = out.read_bytes()
    Vr, Ar, Dr = _msh1(ref)
    Vm, Am, Dm = _msh1(mine)
    assert len(Vm) == len(Vr)
    assert np.array_equal(Am, Ar) and np.array_equal(Dm, Dr)
    assert np.array_equal(Vm, Vr), np.abs(Vm - Vr).max()
    assert mine == ref
    with open(os.path.join(GOLD, name + ".json")) as f:
        assert summary == json.loads(f.read())


def test_generated_scenes_are_the_committed_ones(tmp_path):
    """The fixtures are what gltf_scenes.py writes (the generator and the fixtures stay in step)."""
    gltf_scenes.write_all(str(tmp_path))
    for name in os.listdir(tmp_path):
        with open(tmp_path / name, "rb") as f, open(os.path.join(GOLD, name), "rb") as g:
            assert f.read() == g.read(), name


def test_rules_on_the_hierarchy_scene():
    V, A, D, s = gltf.convert(os.path.join(GOLD, "hierarchy.gltf"))
    # room 12 + crate 12 x 2 instances + panel 2 + leaves (12 + 12 + 12) x 2 placements
    assert len(V) == 12 + 24 + 2 + 72 and s["transparents_ignores"] == 3
    want = sorted([0.2126 * 0.8 + 0.7152 * 0.7 + 0.0722 * 0.6, 0.9 * 0.5, 0.2126 * 0.2 + 0.7152 * 0.5 + 0.0722 * 0.3,
                   0.5 * (0.2126 * 0.1 + 0.7152 * 0.6 + 0.0722 * 0.1), 0.6, 0.05])   # wall, textured, gloss, mask, none, dark
    assert np.allclose(np.unique(A), want, rtol=1e-6)
    assert D.sum() == 2 + 24                                     # the double-sided panel and the MASK leaves
    # z up: the room's floor (y = 0 in glTF) is at z = 0 and its ceiling at z = 3
    z = V.reshape(-1, 3, 3)[:12, :, 2]
    assert np.isclose(z.min(), 0.0, atol=1e-6) and np.isclose(z.max(), 3.0, atol=1e-6)


def test_mirrored_instance_keeps_its_faces_outward():
    V, _, _, _ = gltf.convert(os.path.join(GOLD, "hierarchy.gltf"))
    T = V.reshape(-1, 3, 3)
    crates = [T[12:24], T[24:36]]                                # matrix instance, then its mirrored child
    for c in crates:
        n = np.cross(c[:, 1] - c[:, 0], c[:, 2] - c[:, 0])
        centre = c.reshape(-1, 3).mean(0)
        out = ((c.mean(1) - centre) * n).sum(1)
        assert (out > 0).all()


def test_centimetre_scene_is_scaled_and_degenerate_dropped():
    V, _, _, s = gltf.convert(os.path.join(GOLD, "centimetres.gltf"))
    assert s["echelle"] == 0.01 and s["triangles"] == 24 and s["taille_m"] == [12.0, 8.0, 3.0]
    V2, _, _, s2 = gltf.convert(os.path.join(GOLD, "centimetres.gltf"), scale=0.02)
    assert s2["echelle"] == 0.02 and np.allclose(V2, 2 * V, rtol=1e-6)


def test_glb_gives_the_same_mesh(tmp_path):
    glb = tmp_path / "centimetres.glb"
    gltf_scenes.to_glb(os.path.join(GOLD, "centimetres.gltf"), str(glb))
    a = tmp_path / "a.mesh"
    b = tmp_path / "b.mesh"
    gltf.convert(os.path.join(GOLD, "centimetres.gltf"), str(a))
    gltf.convert(str(glb), str(b))
    assert a.read_bytes() == b.read_bytes()


def test_cli_and_errors(tmp_path, capsys):
    shutil.copy(os.path.join(GOLD, "noscene.gltf"), tmp_path / "n.gltf")
    assert gltf.main([str(tmp_path / "n.gltf"), str(tmp_path / "n.mesh"), "--echelle", "2"]) == 0
    line = json.loads(capsys.readouterr().out)
    assert line["echelle"] == 2.0 and line["triangles"] == 36
    assert gltf.main([str(tmp_path / "n.gltf")]) == 2
    empty = {"asset": {"version": "2.0"}, "nodes": [{}], "scenes": [{"nodes": [0]}]}
    (tmp_path / "e.gltf").write_text(json.dumps(empty))
    with pytest.raises(gltf.GltfError):
        gltf.convert(str(tmp_path / "e.gltf"))
    (tmp_path / "v1.glb").write_bytes(struct.pack("<III", 0x46546C67, 1, 12))
    with pytest.raises(gltf.GltfError):
        gltf.convert(str(tmp_path / "v1.glb"))
