"""The drop-in boundary with the reference's own consumers: the JSONL the drop-in binaries print
(tests/golden/cli/, made on a GB300 by tests/golden/make_cli_fixtures.sh with run_cuda.sh's
commands and file names) goes through the unmodified cuda/analyse_cuda.py and cuda/budget.py of
a reference checkout ($RC_REFERENCE_DIR, else a directory named "reference" beside this
repository; the test is skipped without one).  The scripts must exit 0 and read every table, and
the gains G that analyse_cuda.py computes from our scen_main.jsonl / scen_stress.jsonl /
scen_holdout.jsonl must match
those it computes from the reference's published RTX 4060 files (same commands, same seeds) within
the curves' tolerance."""
import os
import re
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "tests", "golden", "cli")
REF = os.environ.get("RC_REFERENCE_DIR") or os.path.join(os.path.dirname(ROOT), "reference")
SCRIPTS = os.path.join(REF, "cuda")
PUBLISHED = os.path.join(REF, "reference", "cuda_rtx4060")
HOLDOUT = "Scene de validation (jamais vue pendant la mise au point)"

pytestmark = pytest.mark.skipif(not os.path.exists(os.path.join(SCRIPTS, "analyse_cuda.py")),
                                reason="no reference checkout (its analysis scripts are read from there)")


def _analyse(d):
    r = subprocess.run([sys.executable, os.path.join(SCRIPTS, "analyse_cuda.py"), str(d)], capture_output=True, text=True,
                       timeout=120, env=dict(os.environ, PYTHONIOENCODING="utf-8"))
    assert r.returncode == 0, r.stderr
    return r.stdout


def _gains(md, title):
    """{method: [4 G values]} of the gain table under the section `title`."""
    sec = md.split("## " + title, 1)[1].split("\n## ", 1)[0]
    out = {}
    for line in sec.splitlines():
        m = re.match(r"\| (.+?) \| ([\d.]+) \(\w[^)]*\) \| ([\d.]+) \(.*?\) \| ([\d.]+) \(.*?\) \| ([\d.]+) \(.*?\) \|", line)
        if m:
            out[m.group(1)] = [float(m.group(k)) for k in range(2, 6)]
    return out


def test_analyse_and_budget_accept_our_jsonl(tmp_path):
    for f in ("scen_main.jsonl", "scen_holdout.jsonl", "scen_stress.jsonl", "timing_43k.jsonl", "timing_1M.jsonl", "res_1M.jsonl"):
        shutil.copy(os.path.join(CLI, f), tmp_path / f)
    md = _analyse(tmp_path)
    assert "## Scene principale" in md and "## Scene stress" in md and "## " + HOLDOUT in md
    assert "Temps GPU par image (timing_43k.jsonl, 43526 points, NVIDIA GB300)" in md
    assert "Temps GPU par image (timing_1M.jsonl, 1082802 points, NVIDIA GB300)" in md
    assert "VRAM : contexte" in md
    for t in ("timing_43k.jsonl", "timing_1M.jsonl"):
        r = subprocess.run([sys.executable, os.path.join(SCRIPTS, "budget.py"), str(tmp_path / t)], capture_output=True,
                           text=True, timeout=60)
        assert r.returncode == 0, r.stderr
        assert 1.0 <= float(r.stdout.strip()) <= 4.0, t


@pytest.mark.parametrize("ours,theirs,title", [("scenf_main.jsonl", "scen_main.jsonl", "Scene principale"),
                                               ("scenf_holdout.jsonl", "scen_holdout.jsonl", HOLDOUT)])
def test_run_cuda_scenf_output_reads(tmp_path, ours, theirs, title):
    """run_cuda.sh's own scenf commands on scene_main and scene_holdout (scenarios_main.txt, 10
    seeds), under the file names run_cuda.sh gives them."""
    shutil.copy(os.path.join(CLI, ours), tmp_path / theirs)
    md = _analyse(tmp_path)
    g = _gains(md, title)
    assert "v4-A2C memoire verifiee+rampe" in g and all(x > 0 for v in g.values() for x in v)


@pytest.mark.parametrize("name,title", [("scen_main.jsonl", "Scene principale"),
                                        ("scen_stress.jsonl", "Scene stress (8 lampes, mur mobile, boites)"),
                                        ("scen_holdout.jsonl", HOLDOUT)])
def test_gains_match_the_published_ones(tmp_path, name, title):
    if not os.path.exists(os.path.join(PUBLISHED, name)):
        pytest.skip("published results absent")
    ours, theirs = tmp_path / "ours", tmp_path / "theirs"
    ours.mkdir()
    theirs.mkdir()
    shutil.copy(os.path.join(CLI, name), ours / name)
    shutil.copy(os.path.join(PUBLISHED, name), theirs / name)
    a, b = _gains(_analyse(ours), title), _gains(_analyse(theirs), title)
    assert set(a) == set(b) and len(a) >= 3
    for m in a:
        for x, y in zip(a[m], b[m]):
            assert abs(x - y) <= 0.03 * y, (m, a[m], b[m])
