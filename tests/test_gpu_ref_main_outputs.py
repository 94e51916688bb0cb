"""The drop-in binaries, live on the GPU, against the reference's own binaries for the modes the
reference publishes no output of: `quality`, `recon`, `taa` (poc_gpu_l3 on scene_main,
poc_gpu_l8 on the 8-light scene_stress) and run_cuda.sh's `scenf` lines, compared row by row with
what the reference's binaries printed for the same commands on a GB300 (tests/golden/ref_main/,
made by tests/golden/make_ref_main_fixtures.sh; the comparison rules are those of
tests/test_ref_main_outputs.py, which checks the fixtures one such run of this repository's
binaries left)."""
import os
import subprocess
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from test_ref_main_outputs import GOLDEN, REF_MAIN, compare  # noqa: E402

from render_engine_gb300 import build  # noqa: E402

pytestmark = pytest.mark.gpu

COMMANDS = [
    ("poc_gpu_l3", "quality", "quality_main.jsonl", "scene_main.bin", ["4", "1,1.5"]),
    ("poc_gpu_l3", "recon", "recon_main.jsonl", "scene_main.bin", ["4"]),
    ("poc_gpu_l3", "taa", "taa_main.jsonl", "scene_main.bin", ["10", os.path.join(GOLDEN, "scenarios_main.txt")]),
    ("poc_gpu_l3", "scenf", "scenf_main.jsonl", "scene_main.bin", ["10", os.path.join(GOLDEN, "scenarios_main.txt")]),
    ("poc_gpu_l3", "scenf", "scenf_holdout.jsonl", "scene_holdout.bin", ["10", os.path.join(GOLDEN, "scenarios_main.txt")]),
    ("poc_gpu_l8", "quality", "quality_stress.jsonl", "scene_stress.bin", ["4", "1,1.5"]),
    ("poc_gpu_l8", "recon", "recon_stress.jsonl", "scene_stress.bin", ["4"]),
    ("poc_gpu_l8", "taa", "taa_stress.jsonl", "scene_stress.bin", ["10", os.path.join(GOLDEN, "scenarios_stress.txt")]),
]


@pytest.fixture(scope="module")
def bindir():
    return os.path.dirname(build.build())


@pytest.mark.parametrize("exe,mode,name,scene,args", COMMANDS)
def test_live_output_matches_the_reference_binary(bindir, tmp_path, exe, mode, name, scene, args):
    from conftest import golden_bytes
    p = tmp_path / scene
    p.write_bytes(golden_bytes(scene))
    r = subprocess.run([os.path.join(bindir, exe), mode, str(p), *args], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    with open(os.path.join(REF_MAIN, name)) as f:
        ref = f.read().splitlines()
    n, worst = compare(mode, r.stdout.splitlines(), ref)
    print("%s %s: %d rows, worst relative difference %.2e" % (mode, scene, n, worst))
