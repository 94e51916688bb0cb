"""Every error curve the drop-in binaries printed on a GB300 against the reference's published ones.

tests/golden/cli/scen_main.jsonl, scen_stress.jsonl and scen_holdout.jsonl are the JSONL that
poc_gpu_l3 / poc_gpu_l8 printed on a GB300 (tests/golden/make_cli_fixtures.sh: the published files'
own commands, 10 seeds); tests/golden/golden_scen_main.json, golden_scen_stress.json and
golden_scen_holdout.json hold the curves the reference's binary printed on an RTX 4060
(reference/cuda_rtx4060/scen_main.jsonl, scen_stress.jsonl, scen_holdout.jsonl, 10-seed means,
5 decimals; the holdout scene is the validation box scene the reference never tuned on).  Each of
the 126 + 112 + 126 (scenario, method) curves must be there, frame for frame
within 1e-3 relative: the GPU path's frames equal the reference kernels' bit for bit except where the
reference itself sums with float atomics, so what is left is that run-to-run spread and the
published files' rounding.  The GPU run itself is in the -m gpu tests (test_gpu_parity.py, three
curves); this test reads the fixtures only."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
TOL = 1e-3


def _published(name):
    with open(os.path.join(GOLDEN, name)) as f:
        g = json.load(f)
    return {(r["scen"], r["name"]): r for r in g["rows"]}


def scen_rows(lines):
    """{(scenario, method): row} of the `scen` lines of a JSONL text."""
    rows = {}
    for line in lines:
        if line.startswith("{"):
            r = json.loads(line)
            if r.get("type") == "scen":
                rows[(r["scen"], r["name"])] = r
    return rows


def _printed(name):
    with open(os.path.join(GOLDEN, "cli", name)) as f:
        return scen_rows(f)


CASES = [("scen_main.jsonl", "golden_scen_main.json", 126), ("scen_stress.jsonl", "golden_scen_stress.json", 112),
         ("scen_holdout.jsonl", "golden_scen_holdout.json", 126)]


@pytest.mark.parametrize("printed,published,count", CASES)
def test_every_printed_curve_matches_the_published_one(printed, published, count):
    assert_curves_match(_printed(printed), published, count, printed)


def assert_curves_match(ours, published, count, label):
    """Every published (scenario, method) curve of `published` is in `ours`, frame for frame
    within TOL relative, with the same `last` frame and pre/post means."""
    theirs = _published(published)
    assert len(theirs) == count
    assert set(ours) == set(theirs)
    worst = 0.0
    for k, g in theirs.items():
        r = ours[k]
        a, b = np.asarray(r["curve"]), np.asarray(g["curve"])
        assert a.shape == b.shape, k
        rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-6)
        worst = max(worst, float(rel.max()))
        assert rel.max() < TOL, (k, float(rel.max()))
        assert r["last"] == g["last"], k
        for key in ("pre", "post"):
            assert abs(r[key] - g[key]) <= TOL * max(abs(g[key]), 1e-3) + 1e-5, (k, key, r[key], g[key])
    print("%s: %d curves, worst relative difference %.2e" % (label, len(theirs), worst))


def test_scene_line_names_the_gpu():
    with open(os.path.join(GOLDEN, "cli", "scen_main.jsonl")) as f:
        head = json.loads(f.readline())
    assert head["type"] == "scene" and head["np"] == 10728 and "GB300" in head["gpu"]
