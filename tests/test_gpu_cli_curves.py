"""Every published error curve, printed live by the drop-in binaries on the GPU.

poc_gpu_l3 / poc_gpu_l8 run the commands of the reference's published RTX 4060 files:
reference/cuda_rtx4060/scen_main.jsonl (`poc_gpu_l3 scen scene_main.bin 10`), scen_holdout.jsonl
(`poc_gpu_l3 scen scene_holdout.bin 10`, the validation scene) and scen_stress.jsonl
(`poc_gpu_l8 scenf scene_stress.bin 10 scenarios_stress.txt`).  Every one of the
126 + 126 + 112 (scenario, method) curves they print must match the published one
(tests/golden/golden_scen_*.json) frame for frame within 1e-3 relative, with the same `last` frame
and pre/post means.  tests/test_cli_golden_curves.py checks the fixtures one such run left in
tests/golden/cli/; this test prints them again."""
import json
import os
import subprocess
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from test_cli_golden_curves import GOLDEN, assert_curves_match, scen_rows  # noqa: E402

from render_engine_gb300 import build  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bindir():
    return os.path.dirname(build.build())


@pytest.mark.parametrize("exe,mode,scene,published,count", [
    ("poc_gpu_l3", "scen", "scene_main.bin", "golden_scen_main.json", 126),
    ("poc_gpu_l3", "scen", "scene_holdout.bin", "golden_scen_holdout.json", 126),
    ("poc_gpu_l8", "scenf", "scene_stress.bin", "golden_scen_stress.json", 112),
])
def test_binary_prints_every_published_curve(bindir, tmp_path, exe, mode, scene, published, count):
    from conftest import golden_bytes
    p = tmp_path / scene
    p.write_bytes(golden_bytes(scene))
    cmd = [os.path.join(bindir, exe), mode, str(p), "10"]
    if mode == "scenf":
        cmd.append(os.path.join(GOLDEN, "scenarios_stress.txt"))
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    assert json.loads(lines[0])["type"] == "scene"
    assert_curves_match(scen_rows(lines), published, count, "%s %s %s" % (exe, mode, scene))
