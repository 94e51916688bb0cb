"""The metric's error part against the reference's own kernels: the per-frame luminance error over
all valid points and over the event region, from this library's frames and from the reference's
(oracle/_ref, driven by oracle/refrun.cpp), each run on its own from the same start (no state copied
between them), must agree to 1e-3 relative on every frame.

The error is the reference's per-frame metric (poc_gpu.cu:683-696): sqrt(sum (est - ref)^2 / n) /
(sum ref / n) over the valid points, est the cache summed over the lights that are not dormant.
The event region of a state change a -> b is the valid points whose reference changes by more than
5 %, |ref_b - ref_a| / (ref_a + 0.01) > 0.05 (the upper recon categories, poc_gpu.cu:1520-1526).
Scenes: the reference's scene_main (its converged references stored in the file; a light switched
off, the occluder moved, a light switched back on) and its 1,082,802-point timing scene
scene_scale_1M (references from the GPU stochastic Jacobi, two state changes)."""
import math

import numpy as np
import pytest

from oracle import pyref
from render_engine_gb300 import methods as M
from render_engine_gb300 import native as N

pytestmark = pytest.mark.gpu

SEQ = [0] * 40 + [1] * 40 + [2] * 40 + [3] * 30


def _err(lc, dormant, ref, mask):
    nl = lc.shape[1]
    keep = np.array([(dormant >> l) & 1 == 0 for l in range(nl)])
    est = lc[:, keep].astype(np.float64).sum(axis=1)[mask]
    r = ref.astype(np.float64)[mask]
    return math.sqrt(((est - r) ** 2).mean()) / r.mean()


@pytest.mark.parametrize("name", ["v4-A2C suivi 1/4", "v3 complet", "SHaRC responsive 1.0x"])
def test_event_region_error_matches_reference(scene_main_bytes, name):
    if not pyref.available(3):
        pytest.skip("reference kernels not built")
    ctx = N.Context()
    info = ctx.load_bytes(scene_main_bytes)
    nl = info["nl"]
    ref_run = pyref.RefRunner(nl, scene_main_bytes)
    refs = [ctx.state_array(k, N.SA_REF) for k in range(info["ns"])]
    valid = [ctx.state_array(k, N.SA_VALID) != 0 for k in range(info["ns"])]
    m = M.by_name(M.timing_methods(), name)
    ctx.begin(m, SEQ[0], 13)
    ref_run.begin(m, SEQ[0], 13)
    region = None
    worst = 0.0
    checked = 0
    for f, s in enumerate(SEQ):
        if f > 0 and SEQ[f - 1] != s:
            a = refs[SEQ[f - 1]].astype(np.float64)
            region = valid[s] & (np.abs(refs[s] - a) / (a + 1e-2) > 0.05)
            assert region.sum() > 0, f
        ctx.frame(s)
        ref_run.frame(s)
        la, lb = ctx.array(N.A_LC).reshape(-1, nl), ref_run.array(N.A_LC).reshape(-1, nl)
        da, db = ctx.scalar(N.S_DORMANT), ref_run.scalar(N.S_DORMANT)
        assert da == db, f
        masks = [valid[s]] + ([region] if region is not None else [])
        for mk in masks:
            ea, eb = _err(la, da, refs[s], mk), _err(lb, db, refs[s], mk)
            rel = abs(ea - eb) / max(eb, 1e-9)
            worst = max(worst, rel)
            checked += 1
            assert rel <= 1e-3, (name, f, ea, eb)
    assert checked >= len(SEQ) + 100
    print("%s: %d per-frame errors, worst relative difference %.2e" % (name, checked, worst))
    ref_run.close()
    ctx.close()


@pytest.fixture(scope="module")
def scale_1m_with_refs():
    """The reference's 1,082,802-point timing scene with converged references and their warm start
    written in (the GPU stochastic Jacobi of the scene preparation, rc_reference_build), so that
    both implementations start from the same cache."""
    import sys
    sys.path.insert(0, __import__("os").path.dirname(__file__))
    from conftest import golden_bytes
    from render_engine_gb300 import scene as S
    data = golden_bytes("scene_scale_1M.bin")
    q = N.Context()
    info = q.load_bytes(data)
    q.build_reference()
    np_, nl = info["np"], info["nl"]
    sc = S.read(data)
    for k, st in enumerate(sc.states):
        st.ref = q.state_array(k, N.SA_REF)
        st.valid = q.state_array(k, N.SA_VALID).astype(np.uint8)
        st.Pw = q.state_array(k, N.SA_PW).reshape(np_, nl)
    q.close()
    return S.write(sc)


def test_event_region_error_matches_reference_at_1m_points(scale_1m_with_refs):
    """The headline workload: scene_scale_1M, `v4-A2C suivi 1/4`, two state changes (frames 60 and
    120 of the reference's timing sequence)."""
    if not pyref.available(3):
        pytest.skip("reference kernels not built")
    data = scale_1m_with_refs
    seq = [0] * 60 + [1] * 60 + [2] * 20
    ctx = N.Context()
    info = ctx.load_bytes(data)
    nl = info["nl"]
    ref_run = pyref.RefRunner(nl, data)
    refs = [ctx.state_array(k, N.SA_REF) for k in range(3)]
    valid = [ctx.state_array(k, N.SA_VALID) != 0 for k in range(3)]
    m = M.by_name(M.timing_methods(), "v4-A2C suivi 1/4")
    ctx.begin(m, seq[0], 11)
    ref_run.begin(m, seq[0], 11)
    region, worst, checked = None, 0.0, 0
    for f, s in enumerate(seq):
        if f > 0 and seq[f - 1] != s:
            a = refs[seq[f - 1]].astype(np.float64)
            region = valid[s] & (np.abs(refs[s] - a) / (a + 1e-2) > 0.05)
            assert region.sum() > 0, f
        ctx.frame(s)
        ref_run.frame(s)
        if f % 4 and region is None:
            continue   # every fourth frame before the first change, every frame after it
        la, lb = ctx.array(N.A_LC).reshape(-1, nl), ref_run.array(N.A_LC).reshape(-1, nl)
        da, db = ctx.scalar(N.S_DORMANT), ref_run.scalar(N.S_DORMANT)
        assert da == db, f
        for mk in [valid[s]] + ([region] if region is not None else []):
            ea, eb = _err(la, da, refs[s], mk), _err(lb, db, refs[s], mk)
            rel = abs(ea - eb) / max(eb, 1e-9)
            worst = max(worst, rel)
            checked += 1
            assert rel <= 1e-3, (f, ea, eb)
    print("scene_scale_1M: %d per-frame errors, worst relative difference %.2e" % (checked, worst))
    ref_run.close()
    ctx.close()
