"""Converged references computed on the GPU (rc_reference_build: the stochastic Jacobi of
the reference's scene preparation, prep_mesh.cuh:182-213, 459-518)."""
import numpy as np
import pytest

from render_engine_gb300 import methods as M
from render_engine_gb300 import native as N
from render_engine_gb300 import scene as S

pytestmark = pytest.mark.gpu


def test_references_of_the_golden_scene_agree_with_its_own(scene_main_bytes):
    ctx = N.Context()
    ctx.load_bytes(scene_main_bytes)
    ns = ctx.info()["ns"]
    theirs = [ctx.state_array(k, N.SA_REF).copy() for k in range(ns)]
    valid = [ctx.state_array(k, N.SA_VALID).astype(bool) for k in range(ns)]
    noise, iters = ctx.build_reference(noise_target=0.02)
    assert all(n <= 0.02 or it >= 2048 for n, it in zip(noise, iters)), (noise, iters)
    for k in range(ns):
        ours = ctx.state_array(k, N.SA_REF)
        v = valid[k] & ctx.state_array(k, N.SA_VALID).astype(bool)
        assert v.mean() > 0.8
        rel = np.sqrt(np.mean((ours[v] - theirs[k][v]) ** 2)) / np.mean(theirs[k][v])
        assert rel < 0.08, (k, rel)           # both converged estimates of the same fixed point
        assert abs(ours[v].mean() / theirs[k][v].mean() - 1) < 0.02, k


def test_references_make_errors_available_on_a_generated_scene():
    sc = S.street_scene(points=6000, buildings=3)
    ctx = N.Context()
    ctx.load_bytes(S.write(sc))
    assert ctx.info()["has_ref"] == 0
    noise, iters = ctx.build_reference(block=32, max_iter=256)
    assert ctx.info()["has_ref"] == 1 and len(noise) == sc.NS
    sc2 = S.with_references(sc, ctx)
    ctx2 = N.Context()
    ctx2.load_bytes(S.write(sc2))
    for k in range(sc.NS):
        assert np.array_equal(ctx2.state_array(k, N.SA_REF), sc2.states[k].ref)
    m = M.by_name(M.timing_methods(), "v4-A2C suivi 1/4")
    errs = ctx2.run(m, [0] * 30 + [1] * 30, 3, want_err=True)
    assert np.isfinite(errs).all() and max(errs) < 1.0
