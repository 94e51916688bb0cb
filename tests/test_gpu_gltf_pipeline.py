"""The public-scene pipeline of the reference's run_cuda.sh (run_cuda.sh:88-116) through this
repository: glTF -> MSH1 (render_engine_gb300/gltf.py, the converter's command line) -> `poc_gpu_l3
prep` -> `poc_gpu_l3 timing` and frames, on the synthetic scene tests/golden/gltf/centimetres.gltf (a
closed 12 x 8 x 3 m hall with a box inside, modelled in centimetres; its converted mesh equals the
reference converter's, tests/test_gltf.py).  The prepared scene runs
the reference's own kernels bit for bit like the product."""
import json
import os
import subprocess
import sys

import pytest

from oracle import pyref
from render_engine_gb300 import build
from render_engine_gb300 import methods as M

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def public_scene(tmp_path_factory):
    d = tmp_path_factory.mktemp("pub")
    mesh, scene = d / "hall.mesh", d / "hall.bin"
    r = subprocess.run([sys.executable, "-m", "render_engine_gb300.gltf", os.path.join(HERE, "golden", "gltf", "centimetres.gltf"),
                        str(mesh)], capture_output=True, text=True, timeout=120, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    conv = json.loads(r.stdout)
    exe = os.path.join(os.path.dirname(build.build()), "poc_gpu_l3")
    r = subprocess.run([exe, "prep", str(mesh), str(scene), "20000"], capture_output=True, text=True, timeout=900,
                       env=dict(os.environ, PREP_ITER_MAX="128"))
    assert r.returncode == 0, r.stderr
    prep = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    return exe, conv, prep, scene


def test_prep_line_reads_like_the_reference(public_scene):
    _, conv, prep, _ = public_scene
    line = [x for x in prep if x.get("type") == "prep"][-1]
    # the keys analyse_cuda.py reads for a public scene (analyse_cuda.py:90-94)
    assert line["triangles"] == conv["triangles"] == 24 and conv["echelle"] == 0.01
    assert 15000 <= line["np"] <= 25000 and line["cellule_m"] > 0 and len(line["bruit_ref"]) == 5
    assert max(line["bruit_ref"]) < 0.06, line


def test_timing_mode_on_the_prepared_scene(public_scene):
    exe, _, _, scene = public_scene
    r = subprocess.run([exe, "timing", str(scene)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    rows = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    tim = {x["name"]: x for x in rows if x.get("type") == "timing"}
    assert "Classique 1.0x" in tim and "v4-A2C suivi 1/4" in tim
    assert all(v["trace"] > 0 for v in tim.values())


def test_prepared_public_scene_runs_the_reference_kernels_bitexact(public_scene):
    if not pyref.available(3):
        pytest.skip("reference kernels not built")
    sys.path.insert(0, HERE)
    from test_gpu_parity import _frames_vs_reference
    _, _, _, scene = public_scene
    m = M.by_name(M.timing_methods(), "v4-A2C suivi 1/4")
    _frames_vs_reference(scene.read_bytes(), 3, m, [0] * 10 + [1] * 8 + [2] * 8 + [3] * 6, 23)
