"""The drop-in binary, live on the GPU, against the reference's own binary for the modes the
reference publishes no output of: `quality`, `recon`, `taa` and run_cuda.sh's `scenf` lines,
compared row by row with what the reference's `poc_gpu_l3` printed for the same commands on a
GB300 (tests/golden/ref_main/, made by tests/golden/make_ref_main_fixtures.sh; the comparison rules
are those of tests/test_ref_main_outputs.py, which checks the fixtures one such run of this
repository's binary left)."""
import os
import subprocess
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from test_ref_main_outputs import GOLDEN, REF_MAIN, compare  # noqa: E402

from render_engine_gb300 import build  # noqa: E402

pytestmark = pytest.mark.gpu

COMMANDS = [
    ("quality", "quality_main.jsonl", "scene_main.bin", ["4", "1,1.5"]),
    ("recon", "recon_main.jsonl", "scene_main.bin", ["4"]),
    ("taa", "taa_main.jsonl", "scene_main.bin", ["10", os.path.join(GOLDEN, "scenarios_main.txt")]),
    ("scenf", "scenf_main.jsonl", "scene_main.bin", ["10", os.path.join(GOLDEN, "scenarios_main.txt")]),
    ("scenf", "scenf_holdout.jsonl", "scene_holdout.bin", ["10", os.path.join(GOLDEN, "scenarios_main.txt")]),
]


@pytest.fixture(scope="module")
def exe():
    return os.path.join(os.path.dirname(build.build()), "poc_gpu_l3")


@pytest.mark.parametrize("mode,name,scene,args", COMMANDS)
def test_live_output_matches_the_reference_binary(exe, tmp_path, mode, name, scene, args):
    from conftest import golden_bytes
    p = tmp_path / scene
    p.write_bytes(golden_bytes(scene))
    r = subprocess.run([exe, mode, str(p), *args], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    with open(os.path.join(REF_MAIN, name)) as f:
        ref = f.read().splitlines()
    n, worst = compare(mode, r.stdout.splitlines(), ref)
    print("%s %s: %d rows, worst relative difference %.2e" % (mode, scene, n, worst))
