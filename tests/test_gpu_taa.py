"""The taa mode (rc_taa_*, poc_gpu_l3 taa) on the GPU.

* Bit-exact against the reference's own k_taa_* kernels (oracle/_ref cubin driven by
  oracle/refrun.cpp with run_taa_mode's host logic): from identical state every frame, the
  samples, the 3x3 statistics, the new history, the reactive and pending flags and the
  dependency masks agree bit for bit.  The blind and verified masks decide per zone from float
  sums the reference adds with atomics in an undefined order; there a zone whose test sits on
  its threshold may decide differently (bounded below).
* Against the CPU restatement (oracle/rc_oracle.c): per-frame errors.
* The command line's taa lines match the library run.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from oracle import pyoracle as po
from oracle import pyref
from render_engine_gb300 import build
from render_engine_gb300 import native as N

pytestmark = pytest.mark.gpu

SEQ = [0] * 35 + [1] * 12 + [2] * 12 + [3] * 12 + [0] * 10
STATE = (N.T_H, N.T_REACT, N.T_PEND, N.T_CUR, N.T_PREV)


@pytest.mark.parametrize("alpha,gamma,mask", [(0.1, 1.0, 0), (0.05, 1.0, 0), (0.1, 0.0, 0), (0.1, 1.0, 1), (0.1, 1.0, 2),
                                              (0.1, 1.0, 3), (0.1, 1.0, 4)])
def test_taa_vs_reference_kernels(scene_main_bytes, alpha, gamma, mask):
    if not pyref.available(3):
        pytest.skip("reference kernels not built")
    ctx = N.Context()
    ctx.load_bytes(scene_main_bytes)
    ref = pyref.RefRunner(3, scene_main_bytes)
    ctx.taa_begin(alpha, gamma, mask, SEQ[0], 5000)
    ref.taa_begin(alpha, gamma, mask, SEQ[0], 5000)
    np_ = ctx.info()["np"]
    zone_frames = 0
    for f, s in enumerate(SEQ):
        for w in STATE:   # identical state before every frame
            ref.taa_array(w, ctx.taa_array(w))
        e = ctx.taa_frame(s, want_err=True)
        er = ref.taa_frame(s)
        x, xr = ctx.taa_array(N.T_X), ref.taa_array(N.T_X)
        assert np.array_equal(x.view(np.uint32), xr.view(np.uint32)), (f, int((x != xr).sum()))
        for w in (N.T_MU, N.T_SG):
            assert np.array_equal(ctx.taa_array(w).view(np.uint32), ref.taa_array(w).view(np.uint32)), (f, w)
        cur, curr = ctx.taa_array(N.T_CUR), ref.taa_array(N.T_CUR)
        assert (cur != curr).sum() <= max(1, int(2e-5 * np_)), f   # dependency-walk ties
        react, reactr = ctx.taa_array(N.T_REACT), ref.taa_array(N.T_REACT)
        pend, pendr = ctx.taa_array(N.T_PEND), ref.taa_array(N.T_PEND)
        H, Hr = ctx.taa_array(N.T_H), ref.taa_array(N.T_H)
        if np.array_equal(react, reactr) and np.array_equal(pend, pendr):
            assert np.array_equal(H.view(np.uint32), Hr.view(np.uint32)), f
            assert e == pytest.approx(er, rel=1e-6)
        else:
            assert mask in (1, 3), f
            zone_frames += 1
            assert (react != reactr).mean() < 0.01, f
            same = react == reactr
            assert np.array_equal(H[same].view(np.uint32), Hr[same].view(np.uint32)), f
    assert zone_frames <= 2
    ref.close()
    ctx.close()


def test_taa_vs_cpu_oracle(scene_main_bytes):
    ctx = N.Context()
    ctx.load_bytes(scene_main_bytes)
    t = po.Taa(po.Scene(data=scene_main_bytes))
    for mask in (0, 2, 4):
        ctx.taa_begin(0.1, 1.0, mask, SEQ[0], 5000)
        t.begin(0.1, 1.0, mask, SEQ[0], 5000)
        for f, s in enumerate(SEQ):
            e = ctx.taa_frame(s, want_err=True)
            eo, _ = t.frame(s)
            x, xo = ctx.taa_array(N.T_X), t.array(0)
            assert np.isclose(x, xo, rtol=1e-5, atol=1e-6).mean() > 0.999, (mask, f)
            assert e == pytest.approx(eo, rel=2e-3), (mask, f)
    ctx.close()


def test_taa_command_line(tmp_path, scene_main_bytes):
    exe = os.path.join(os.path.dirname(build.build()), "poc_gpu_l3")
    scene = tmp_path / "scene_main.bin"
    scene.write_bytes(scene_main_bytes)
    scen = tmp_path / "scen.txt"
    scen.write_text("# name;state:frames,...\nlampe;0:30,1:40\n")
    r = subprocess.run([exe, "taa", str(scene), "1", str(scen)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.strip()]
    lines = [x for x in lines if x.get("type") == "taa"]
    assert [x["name"] for x in lines] == ["TAA borne alpha=0.05", "TAA borne alpha=0.10", "TAA borne alpha=0.20",
                                          "TAA simple alpha=0.10 (sans bornage)", "TAA + detection aveugle",
                                          "TAA + masque dependances", "TAA + masque dependances verifie", "TAA + masque oracle"]
    assert all(x["type"] == "taa" and x["scen"] == "lampe" and x["last"] == 30 and len(x["curve"]) == 70 for x in lines)
    # the same run through the library
    ctx = N.Context()
    ctx.load_bytes(scene_main_bytes)
    ctx.taa_begin(0.1, 1.0, 2, 0, 5000)
    errs = [ctx.taa_frame(s, want_err=True) for s in [0] * 30 + [1] * 40]
    ctx.close()
    dep = lines[5]
    assert np.allclose(dep["curve"], errs, rtol=0, atol=6e-6)
    assert dep["pre"] == pytest.approx(np.mean(errs[10:30]), abs=1e-5)
    assert dep["post"] == pytest.approx(np.mean(errs[30:60]), abs=1e-5)
    oracle, plain = lines[7], lines[1]
    assert oracle["post"] < plain["post"]
