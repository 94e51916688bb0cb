"""The taa mode's CPU restatement (oracle/rc_oracle.c, run_taa_mode of poc_gpu.cu:1175-1282).

The reference ships no taa outputs, so the mode's parity is pinned on the GPU against the
reference's own k_taa_* kernels (tests/test_gpu_taa.py); here the restatement's own invariants:
reproducible runs, history bounds, the reactive mask sources, and that every mask helps after
an event on the golden scene.
"""
import numpy as np
import pytest

from oracle import pyoracle as po


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
