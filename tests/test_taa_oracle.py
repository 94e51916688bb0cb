"""The taa mode's CPU restatement (oracle/rc_oracle.c, run_taa_mode of poc_gpu.cu:1175-1282).

The reference publishes no taa outputs.  Its own binary's, printed on a GB300
(tests/golden/ref_main/taa_main.jsonl: `poc_gpu_l3 taa scene_main.bin 10 scenarios_main.txt`,
made by tests/golden/make_ref_main_fixtures.sh), pin the restatement: its 10-seed error curves
must match to 2e-4 relative (the printed 5 decimals and the C library's cosf/sinf against
CUDA's).  On the GPU the library's taa kernels are pinned against the reference's own k_taa_*
kernels (tests/test_gpu_taa.py).  Here also the restatement's own invariants: reproducible runs,
history bounds, the reactive mask sources, and that every mask helps after an event on the
golden scene.
"""
import json
import os

import numpy as np
import pytest

from oracle import pyoracle as po

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def taa(scene_main_bytes):
    return po.Taa(po.Scene(data=scene_main_bytes))


SEQ = [0] * 40 + [1] * 40   # light 0 switches off at frame 40


def _run(t, mask, alpha=0.1, gamma=1.0, seed=5000):
    t.begin(alpha, gamma, mask, SEQ[0], seed)
    return np.array([t.frame(s)[0] for s in SEQ])


def test_reproducible_and_seeded(taa):
    a = _run(taa, 0)
    b = _run(taa, 0)
    c = _run(taa, 0, seed=5001)
    assert (a == b).all() and (a != c).any()
    assert np.isfinite(a).all() and (a > 0).all() and (a < 1).all()


def test_masks(taa):
    post = {}
    for mask in range(5):
        e = _run(taa, mask)
        post[mask] = e[40:70].mean()
        if mask in (0, 2, 3, 4):   # identical until the event: those masks act only on events
            assert np.allclose(e[:40], _run(taa, 0)[:40], rtol=0, atol=0)
    for mask in (1, 2, 3, 4):
        assert post[mask] < post[0], (mask, post)
    assert post[4] <= min(post[2], post[3]) * 1.05   # the oracle mask is the upper bound


def test_dependency_mask_flags_the_event(taa):
    taa.begin(0.1, 1.0, 2, 0, 5000)
    for f, s in enumerate(SEQ[:41]):
        taa.frame(s)
        if f == 39:
            cur = taa.array(6)
            assert cur.any()
    react = taa.array(4)
    flagged = react > 0
    assert 0 < flagged.mean() < 1   # some points, not all
    taa.begin(0.1, 1.0, 4, 0, 5000)
    for s in SEQ[:41]:
        taa.frame(s)
    assert ((taa.array(4) > 0) & ~flagged).mean() < 0.1   # the oracle's points are mostly among them


def test_history_within_clamp(taa):
    taa.begin(0.2, 1.0, 0, 0, 5000)
    for s in SEQ[:10]:
        taa.frame(s)
    H, mu, sg = taa.array(1), taa.array(2), taa.array(3)
    x = taa.array(0)
    assert (H >= np.minimum(mu - sg, x) - 1e-4).all() and (H <= np.maximum(mu + sg, x) + 1e-4).all()


# run_taa_mode's methods (poc_gpu.cu:1219-1228): name -> (alpha, gamma, mask)
TAA_METHODS = {"TAA borne alpha=0.05": (0.05, 1.0, 0), "TAA borne alpha=0.20": (0.2, 1.0, 0),
               "TAA simple alpha=0.10 (sans bornage)": (0.1, 0.0, 0), "TAA + detection aveugle": (0.1, 1.0, 1),
               "TAA + masque dependances": (0.1, 1.0, 2), "TAA + masque dependances verifie": (0.1, 1.0, 3),
               "TAA + masque oracle": (0.1, 1.0, 4)}


@pytest.fixture(scope="module")
def taa_stress(scene_stress_bytes):
    return po.Taa(po.Scene(data=scene_stress_bytes))


def _reference_curve(fixture, scenarios, scen, method):
    gold = None
    with open(os.path.join(GOLDEN, "ref_main", fixture)) as f:
        for line in f:
            r = json.loads(line)
            if r.get("type") == "taa" and r["scen"] == scen and r["name"] == method:
                gold = r
    parts = None
    with open(os.path.join(GOLDEN, scenarios)) as f:
        for line in f:
            line = line.strip()
            if not line or line.startswith("#"):
                continue
            name, rest = line.split(";", 1)
            if name == scen:
                parts = [tuple(int(x) for x in t.split(":")) for t in rest.split(",")]
    return gold, parts


@pytest.mark.parametrize("scen,method", [("L2 quatre lampes eteintes puis rallumees", "TAA + masque dependances verifie"),
                                         ("G3 quatre objets deplaces", "TAA + masque dependances"),
                                         ("M1 extinction, mur effondre dans le noir, rallumage", "TAA borne alpha=0.20")])
def test_matches_the_reference_binary_8_lights(taa_stress, scen, method):
    """The same against the reference's poc_gpu_l8 on the 8-light scene_stress
    (tests/golden/ref_main/taa_stress.jsonl, scenarios_stress.txt)."""
    gold, parts = _reference_curve("taa_stress.jsonl", "scenarios_stress.txt", scen, method)
    _check(taa_stress, gold, parts, method)


@pytest.mark.parametrize("scen,method", [("R1 allumee-eteinte-rallumee", "TAA + masque dependances verifie"),
                                         ("I4 boite", "TAA borne alpha=0.05"),
                                         ("R2 allumee-eteinte-porte-rallumee", "TAA + detection aveugle"),
                                         ("I2 porte", "TAA simple alpha=0.10 (sans bornage)"),
                                         ("I1 lampe eteinte", "TAA + masque oracle")])
def test_matches_the_reference_binary(taa, scen, method):
    gold, parts = _reference_curve("taa_main.jsonl", "scenarios_main.txt", scen, method)
    _check(taa, gold, parts, method)


def _check(taa, gold, parts, method):
    seq = [s for s, n in parts for _ in range(n)]
    alpha, gamma, mask = TAA_METHODS[method]
    curve = np.zeros(len(seq))
    for sd in range(10):                     # the reference's seeds 5000 + sd, 10 seeds
        taa.begin(alpha, gamma, mask, seq[0], 5000 + sd)
        for f, s in enumerate(seq):
            curve[f] += taa.frame(s)[0] / 10
    g = np.asarray(gold["curve"])
    rel = np.abs(curve - g) / g
    assert rel.max() < 2e-4, (method, rel.max())
    last = gold["last"]
    assert abs(curve[last:last + 30].mean() - gold["post"]) <= 2e-4 * gold["post"] + 1e-5
