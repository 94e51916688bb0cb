"""The CPU oracle against the reference's published golden error curves.

The reference ships, for its box scenes, the per-frame error curves that its own binary
printed on an RTX 4060 (reference/cuda_rtx4060/scen_main.jsonl, scen_stress.jsonl and, for the
validation scene scene_holdout the reference never tuned on, scen_holdout.jsonl; means over 10
seeds, 5 decimals).  The oracle restates the reference in C; it must reproduce those
curves.  The only differences allowed are those of the C library's cosf/sinf/rsqrt against
CUDA's (a few ulp on ray directions), which move the 10-seed means by less than 2e-3
relative.

The quality mode's outputs are not published; the reference's own binary printed them on a
GB300 (tests/golden/ref_main/quality_main.jsonl: `poc_gpu_l3 quality scene_main.bin 4 1,1.5`, made
by tests/golden/make_ref_main_fixtures.sh), and the oracle's 4-seed pre/post means must match
them to 2e-3 on a sample of its rows across the method families.  Over all 300 rows 282 agree to
1e-3.  The rest are DDGI rows, up to 5.8e-3 with the 0.25 threshold.  With one ray per point,
a region's frame-to-frame relative change is about 1/sqrt(15) for its ~15 points, which is the
threshold itself.  So the per-region test flips on the last-ulp differences of the C library's
cosf/sinf against CUDA's, and the runs drift apart.  The GPU path uses CUDA's functions and
stays within 8.7e-4 of the reference binary on those rows (one row; the others within 2.2e-4).
"""
import json
import os

import numpy as np
import pytest

from oracle import pyoracle as po
from render_engine_gb300 import methods as M

TOL = 2e-3


def _scenario(golden, name):
    for r in golden["rows"]:
        if r["scen"] == name:
            return r
    raise KeyError(name)


def _curve(run, method, seq, seed0, nseeds):
    acc = np.zeros(len(seq))
    for sd in range(nseeds):
        acc += np.asarray(run.run(method, seq, seed0 + sd)) / nseeds
    return acc


@pytest.fixture(scope="module")
def main_run(scene_main_bytes):
    sc = po.Scene(data=scene_main_bytes)
    sc.build()
    return po.Run(sc)


CASES_MAIN = [
    ("R1 allumee-eteinte-rallumee", "Accumulation+parlampe N=32, 1.53x"),
    ("R1 allumee-eteinte-rallumee", "SHaRC N=64 resp=8, 1.57x"),
    ("R1 allumee-eteinte-rallumee", "v4-A2C memoire verifiee+rampe"),
    ("R2 allumee-eteinte-porte-rallumee", "v5-A instantanes verifies"),
    ("R3 porte ouverte-fermee-rouverte", "v5-AB instantanes+projection"),
    ("I3 lampe allumee 1re fois", "Oracle"),
]


@pytest.mark.parametrize("scen,method", CASES_MAIN)
def test_oracle_matches_rtx4060_curves_main(main_run, golden_main, scen, method):
    parts = dict(M.SCEN_SCENARIOS)[scen]
    seq = M.sequence(parts)
    m = M.by_name(M.scen_methods(), method)
    gold = [r for r in golden_main["rows"] if r["scen"] == scen and r["name"] == method][0]
    ours = _curve(main_run, m, seq, golden_main["seed0"], golden_main["nseeds"])
    g = np.asarray(gold["curve"])
    rel = np.abs(ours - g) / np.maximum(g, 1e-6)
    assert rel.max() < TOL, (scen, method, rel.max())
    last = gold["last"]
    post = ours[last:last + 30].mean()
    assert abs(post - gold["post"]) / gold["post"] < TOL


@pytest.mark.parametrize("scen,method", [("R1 allumee-eteinte-rallumee", "v4-A2C memoire verifiee+rampe"),
                                         ("I4 boite", "v5-AB instantanes+projection")])
def test_oracle_matches_rtx4060_curves_holdout(scene_holdout_bytes, golden_holdout, scen, method):
    sc = po.Scene(data=scene_holdout_bytes)
    sc.build()
    run = po.Run(sc)
    seq = M.sequence(dict(M.SCEN_SCENARIOS)[scen])
    m = M.by_name(M.scen_methods(), method)
    gold = [r for r in golden_holdout["rows"] if r["scen"] == scen and r["name"] == method][0]
    ours = _curve(run, m, seq, golden_holdout["seed0"], golden_holdout["nseeds"])
    g = np.asarray(gold["curve"])
    rel = np.abs(ours - g) / np.maximum(g, 1e-6)
    assert rel.max() < TOL, (scen, method, rel.max())
    last = gold["last"]
    assert abs(ours[last:last + 30].mean() - gold["post"]) / gold["post"] < TOL


def _stress_scenarios():
    import os
    out = {}
    for line in open(os.path.join(os.path.dirname(__file__), "golden", "scenarios_stress.txt")):
        line = line.strip()
        if not line or line.startswith("#"):
            continue
        name, rest = line.split(";", 1)
        out[name] = [tuple(int(x) for x in t.split(":")) for t in rest.split(",")]
    return out


@pytest.mark.parametrize("scen,method", [("G3 quatre objets deplaces", "v3"),
                                         ("L2 quatre lampes eteintes puis rallumees", "SHaRC N=64 resp=8, 1.57x")])
def test_oracle_matches_rtx4060_curves_stress(scene_stress_bytes, golden_stress, scen, method):
    sc = po.Scene(data=scene_stress_bytes)
    sc.build()
    run = po.Run(sc)
    inten = [sc_state for sc_state in range(sc.NS)]
    from render_engine_gb300 import scene as S
    parsed = S.read(scene_stress_bytes)
    dyn = 0
    for s in range(1, sc.NS):
        for l in range(sc.NL):
            if parsed.states[s].inten[l] != parsed.states[0].inten[l]:
                dyn |= 1 << l
    m = M.by_name(M.scenf_methods(dyn), method)
    seq = M.sequence(_stress_scenarios()[scen])
    gold = [r for r in golden_stress["rows"] if r["scen"] == scen and r["name"] == method][0]
    ours = _curve(run, m, seq, golden_stress["seed0"], golden_stress["nseeds"])
    g = np.asarray(gold["curve"])
    rel = np.abs(ours - g) / np.maximum(g, 1e-6)
    assert rel.max() < TOL, (scen, method, rel.max())


QUALITY_ROWS = [("SHaRC N=16 resp=4, 1.00x rayons", 1.0, 0), ("Accumulation+parlampe N=32, 1.50x rayons", 1.5, 1),
                ("Accumulation N=8, 1.00x rayons", 1.0, 3), ("DDGI+parlampe h=0.97 seuil=1.00 borne=1, 1.50x rayons", 1.5, 3),
                ("DDGI h=0.90 seuil=0.50 borne=0, 1.00x rayons", 1.0, 2), ("Cache a dependances v3, suivi 1/4", 1.0, 1),
                ("Oracle", 1.0, 0)]


@pytest.mark.parametrize("name,budget,event", QUALITY_ROWS)
def test_oracle_matches_the_reference_binary_quality(main_run, name, budget, event):
    gold = None
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_main", "quality_main.jsonl")
    with open(path) as f:
        for line in f:
            r = json.loads(line)
            if r.get("type") == "quality" and r["name"] == name and round(r["budget"], 3) == budget and r["event"] == event:
                gold = r
    m = [x for x in M.quality_methods([1.0, 1.5]) if x.name == name and round(x.budget, 3) == budget][0]
    seq = [event] * 50 + [event + 1] * 50     # poc_gpu.cu:1555: the event at frame 50
    pre = post = 0.0
    for sd in range(4):
        er = np.asarray(main_run.run(m, seq, 1000 + sd))
        pre += er[30:50].mean() / 4
        post += er[50:80].mean() / 4
    assert abs(pre - gold["pre"]) <= TOL * gold["pre"] + 1e-5, (pre, gold["pre"])
    assert abs(post - gold["post"]) <= TOL * gold["post"] + 1e-5, (post, gold["post"])


def test_oracle_matches_the_reference_binary_recon_curves(main_run):
    """`recon scene_main.bin 4` (poc_gpu.cu:1489-1512): every per-seed error curve of its four
    methods over the four events, seeds 1000 + sd, single runs rather than means (worst 5.2e-4)."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_main", "recon_main.jsonl")
    gold = {}
    with open(path) as f:
        for line in f:
            r = json.loads(line)
            if r.get("type") == "recon_seeds":
                gold[(r["name"], r["event"])] = np.asarray(r["curves"])
    checked = 0
    for m in M.recon_methods():
        for e in range(4):
            seq = [e] * 50 + [e + 1] * 50
            g = gold[(m.name, e)]
            for sd in range(len(g)):
                er = np.asarray(main_run.run(m, seq, 1000 + sd))
                rel = np.abs(er - g[sd]) / np.maximum(g[sd], 1e-6)
                assert rel.max() < TOL, (m.name, e, sd, rel.max())
                checked += 1
    assert checked == 4 * 4 * 4
