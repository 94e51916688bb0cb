"""The drop-in command line (poc_gpu_l3 / poc_gpu_l8) on the GPU: the JSONL lines the
reference's scripts read (run_cuda.sh, analyse_cuda.py), and the recon mode's statistics
recomputed from the library frame by frame."""
import json
import os
import subprocess

import numpy as np
import pytest

from render_engine_gb300 import build
from render_engine_gb300 import methods as M
from render_engine_gb300 import native as N

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def exe():
    return os.path.join(os.path.dirname(build.build()), "poc_gpu_l3")


@pytest.fixture(scope="module")
def scene_file(tmp_path_factory, scene_main_bytes):
    p = tmp_path_factory.mktemp("scene") / "scene_main.bin"
    p.write_bytes(scene_main_bytes)
    return str(p)


def _lines(exe, *args, timeout=600):
    r = subprocess.run([exe, *args], capture_output=True, text=True, timeout=timeout)
    assert r.returncode == 0, r.stderr
    return [json.loads(x) for x in r.stdout.splitlines() if x.strip()]


def test_res_and_timing_lines(exe, scene_file):
    res = _lines(exe, "res", scene_file)
    assert res[0]["type"] == "scene" and res[0]["np"] == 10728 and res[0]["mask_bits"] == 128
    assert any(x["type"] == "vram" and x["scene_mb"] > 0 for x in res)
    tim = _lines(exe, "timing", scene_file)
    rows = [x for x in tim if x["type"] == "timing"]
    assert len(rows) >= 5 and all(x["trace"] > 0 for x in rows)
    assert {"v4-A2C suivi 1/4", "v3 complet"} <= {x["name"] for x in rows}


def test_light_count_mismatch_is_an_error(exe, scene_stress_bytes, tmp_path):
    p = tmp_path / "stress.bin"
    p.write_bytes(scene_stress_bytes)   # 8 lights, the l3 binary expects 3
    r = subprocess.run([exe, "res", str(p)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 1 and "light" in r.stderr


def test_recon_matches_the_library(exe, scene_file, scene_main_bytes):
    out = _lines(exe, "recon", scene_file, "2")
    seeds = [x for x in out if x["type"] == "recon_seeds"]
    bv = [x for x in out if x["type"] == "recon_bv"]
    assert len(seeds) == len(bv) == 4 * 4            # 4 methods x 4 events
    name = "SHaRC N=64 resp=8, 1.52x"
    s0 = next(x for x in seeds if x["name"] == name and x["event"] == 0)
    b0 = next(x for x in bv if x["name"] == name and x["event"] == 0)
    # the same runs through the library, frame by frame
    m = M.Method(name=name, mode=0, nmax=64.0, budget=1.52, resp_mask=1, nmax_resp=8.0, rescale=True)
    ctx = N.Context()
    ctx.load_bytes(scene_main_bytes)
    nl = ctx.info()["nl"]
    seq = [0] * 50 + [1] * 50
    F0, NF = 45, 55
    sums = np.zeros((NF, 10728), np.float64)
    sqs = np.zeros((NF, 10728), np.float64)
    for sd in range(2):
        ctx.begin(m, seq[0], 1000 + sd)
        for f, st in enumerate(seq):
            ctx.frame(st, want_err=True)
            if F0 <= f < F0 + NF:
                lc = ctx.array(N.A_LC).reshape(-1, nl).astype(np.float64)
                dormant = ctx.scalar(N.S_DORMANT)
                live = [l for l in range(nl) if not (dormant >> l) & 1]
                e = lc[:, live].sum(axis=1)
                sums[f - F0] += e
                sqs[f - F0] += e * e
        assert np.allclose(ctx.errors(), s0["curves"][sd], rtol=0, atol=6e-6)
    rold = ctx.state_array(0, N.SA_REF).astype(np.float64)
    rnew = ctx.state_array(1, N.SA_REF).astype(np.float64)
    valid = ctx.state_array(1, N.SA_VALID).astype(bool)
    rel = np.abs(rnew - rold) / (rold + 1e-2)
    cat = np.where(rel > 0.2, 0, np.where(rel > 0.05, 1, 2))
    assert b0["mref"] == pytest.approx(rnew[valid].mean(), rel=1e-5)
    for k in range(3):
        sel = valid & (cat == k)
        assert b0["cats"][k]["n"] == int(sel.sum())
        if not sel.any():
            continue
        mu = sums[:, sel] / 2
        bias2 = ((mu - rnew[sel]) ** 2).mean(axis=1)
        var = np.clip(sqs[:, sel] / 2 - mu * mu, 0, None).mean(axis=1)
        assert np.allclose(b0["cats"][k]["bias2"], bias2, rtol=2e-3, atol=1e-9)
        assert np.allclose(b0["cats"][k]["var"], var, rtol=2e-2, atol=1e-7)
