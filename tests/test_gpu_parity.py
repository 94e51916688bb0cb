"""GPU parity: the product kernels against the reference's own kernels and the CPU oracle.

* Against the reference kernels (cuda/poc_gpu.cu compiled for sm_103a, driven by
  oracle/refrun.cpp): the per-state build (direct light, shadow-voxel masks) and every frame
  of full method runs are compared BIT FOR BIT, each frame starting from identical state
  (the product's state is copied into the reference before the frame).  The only tolerated
  differences come from sums the reference accumulates with float atomics in an undefined
  order (see _frames_vs_reference).
* Against the CPU oracle: per-ray hit records (primitive id, cache point, distance) and
  the 10-seed error curves published by the reference (RTX 4060).
* The plane-culled trace against a brute-force trace of every triangle on the same rays:
  zero disagreements.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from oracle import pyref
from render_engine_gb300 import methods as M
from render_engine_gb300 import native as N
from render_engine_gb300 import scene as S

pytestmark = pytest.mark.gpu

SYNC = [N.A_LC, N.A_N, N.A_C0, N.A_PENDING, N.A_CUR, N.A_PREV, N.A_STALE, N.A_AGE, N.A_SNAP, N.A_NEQ, N.A_COEF,
        N.A_RSTAT, N.A_DSTAT, N.A_SUMPR, N.A_NPEND]


@pytest.fixture(scope="session", autouse=True)
def built():
    from render_engine_gb300 import build
    build.build()
    from oracle import build as ob
    ob.build()


def _ctx(data, **kw):
    c = N.Context(**kw)
    c.load_bytes(data)
    return c


def _sync_to_ref(ctx, ref):
    for a in SYNC:
        v = ctx.array(a)
        if a == N.A_STALE:
            v = v.astype(np.uint8)
        ref.set_array(a, v)
    for s in range(7):
        ref.set_scalar(s, ctx.scalar(s))


def test_state_build_bitexact_vs_reference(scene_main_bytes):
    if not pyref.available(3):
        pytest.skip("reference kernels not built")
    ctx = _ctx(scene_main_bytes)
    ref = pyref.RefRunner(3, scene_main_bytes)
    for s in range(ctx.info()["ns"]):
        assert np.array_equal(ctx.state_array(s, N.SA_EDIR).view(np.uint32), ref.state_array(s, 0).view(np.uint32))
        assert np.array_equal(ctx.state_array(s, N.SA_SV), ref.state_array(s, 1))


def _frames_vs_reference(data, nl, method, seq, seed, grid=(8, 4, 4)):
    """Run both implementations frame by frame from identical state and compare.

    A frame is compared BIT FOR BIT unless one of its inputs is a float sum that the
    reference accumulates with atomics in an undefined order (so the reference itself differs
    from run to run there):
      * the region statistics of a verification frame (k_decide) or a projection window,
        and the DDGI region sums, move the decided histories by an ulp or so;
      * Sum 1/(n+1) recomputed after an event in adaptive mode can move a ray budget by one
        on a few points.
    On those frames 99.8 % of the points must still agree: exactly for ray counts, masks and
    flags, to 1e-5 for histories and 1e-4 for the cache.  A projection window is looser: its
    per-region normal equations (float sums, compared to 1e-5 relative) go through a
    Gauss-Jordan solve whose conditioning amplifies their last-bit differences, and two runs
    of the reference itself leave up to 0.1 % of the points more than 1e-4 apart there (up to
    5e-3); 99 % must agree to 1e-4 and all to 1e-2.  Dependency masks of an exact frame are
    equal bit for bit, ties at voxel edges included (cache points on voxel faces walk from a
    coordinate that is an exact integer, and the walk rounds it before subtracting)."""
    ctx = _ctx(data, grid=grid)
    ref = pyref.RefRunner(nl, data, grid=grid)
    ctx.begin(method, seq[0], seed)
    ref.begin(method, seq[0], seed)
    exact_frames = 0
    for f, s in enumerate(seq):
        _sync_to_ref(ctx, ref)
        pend_before = ctx.scalar(N.S_PEND_LEFT)
        proj_before = ctx.scalar(N.S_PROJ_LEFT)
        event = f > 0 and seq[f - 1] != s
        ctx.frame(s)
        ref.frame(s)
        pend_after = ctx.scalar(N.S_PEND_LEFT)
        assert pend_after == ref.scalar(N.S_PEND_LEFT) and ctx.scalar(N.S_DORMANT) == ref.scalar(N.S_DORMANT), f
        a, b = ctx.array(N.A_LC).reshape(-1, nl), ref.array(N.A_LC).reshape(-1, nl)
        na, nb = ctx.array(N.A_N), ref.array(N.A_N)
        ca, cb = ctx.array(N.A_CUR).reshape(-1, na.size), ref.array(N.A_CUR).reshape(-1, na.size)
        same_lc = np.mean((a.view(np.uint32) == b.view(np.uint32)).all(axis=1))
        same_n = np.mean(na.view(np.uint32) == nb.view(np.uint32))
        mask_diff = int((ca != cb).any(axis=0).sum())
        same_p = np.mean(ctx.array(N.A_PENDING) == ref.array(N.A_PENDING))
        assert np.array_equal(ctx.array(N.A_STALE).astype(np.uint8), ref.array(N.A_STALE)), f
        loose = (pend_before > 0 or (event and (method.mode == 1 or pend_after > 0)) or method.ddgi
                 or proj_before > 0 or ctx.scalar(N.S_PROJ_LEFT) > 0)
        if not loose:
            assert same_lc == 1.0 and same_n == 1.0 and same_p == 1.0, (f, same_lc, same_n, same_p)
            assert mask_diff == 0, (f, mask_diff)
            exact_frames += 1
        else:
            proj = proj_before > 0 or ctx.scalar(N.S_PROJ_LEFT) > 0
            close_lc = np.mean(np.isclose(a, b, rtol=1e-4, atol=1e-6).all(axis=1))
            close_n = np.mean(np.isclose(na, nb, rtol=1e-5, atol=1e-7))
            if proj:
                qa, qb = ctx.array(N.A_NEQ), ref.array(N.A_NEQ)
                assert np.allclose(qa, qb, rtol=1e-5, atol=1e-3), f
                assert np.allclose(a, b, rtol=1e-2, atol=1e-5), f
                assert close_lc >= 0.99, (f, close_lc)
                close_lc = 1.0
            assert min(close_lc, close_n, same_p, 1.0 - mask_diff / na.size) >= 0.998, (f, close_lc, close_n, same_p, mask_diff)
        assert abs(float(a.sum()) - float(b.sum())) <= 1e-3 * abs(float(b.sum())) + 1e-6, f
    if not method.ddgi:
        assert exact_frames >= len(seq) // 3, exact_frames


@pytest.mark.parametrize("name", ["Classique 1.0x", "SHaRC responsive 1.0x", "v3 complet", "v4-A2C suivi 1/4", "DDGI 1.0x"])
def test_timing_methods_bitexact_vs_reference(scene_main_bytes, name):
    if not pyref.available(3):
        pytest.skip("reference kernels not built")
    m = M.by_name(M.timing_methods(), name)
    seq = [0] * 35 + [1] * 12 + [2] * 12 + [3] * 12 + [0] * 12
    _frames_vs_reference(scene_main_bytes, 3, m, seq, 11)


@pytest.mark.parametrize("name", ["v5-A instantanes verifies", "v5-AB instantanes+projection", "Oracle",
                                  "SHaRC + memoire + instantanes, 1.57x", "v4-A2 memoire verifiee"])
def test_event_methods_vs_reference(scene_main_bytes, name):
    if not pyref.available(3):
        pytest.skip("reference kernels not built")
    m = M.by_name(M.scen_methods(), name)
    seq = M.sequence([(0, 25), (1, 22), (2, 22), (3, 12), (0, 24), (1, 6)])
    _frames_vs_reference(scene_main_bytes, 3, m, seq, 2001)


def test_eight_lights_vs_reference(scene_stress_bytes):
    if not pyref.available(8):
        pytest.skip("reference kernels not built")
    m = M.by_name(M.timing_methods(), "v4-A2C suivi 1/4")
    seq = [0] * 25 + [3] * 10 + [0] * 10 + [2] * 10 + [4] * 8
    _frames_vs_reference(scene_stress_bytes, 8, m, seq, 3)


def test_large_generated_scene_vs_reference():
    if not pyref.available(3):
        pytest.skip("reference kernels not built")
    data = S.write(S.box_room(points=300_000, seed=7))
    m = M.by_name(M.timing_methods(), "v3 complet")
    seq = [0] * 6 + [1] * 4 + [2] * 4 + [3] * 4
    _frames_vs_reference(data, 3, m, seq, 12)


def test_culled_trace_equals_brute_force(scene_main_bytes):
    for data in (scene_main_bytes, S.write(S.box_room(points=200_000, seed=2))):
        ctx = _ctx(data, flags=N.FLAG_CHECK_TRACE)
        m = M.by_name(M.timing_methods(), "Classique 2.0x")
        ctx.run(m, [0] * 8 + [2] * 8 + [4] * 8, 21, want_err=False)
        bad, rays = ctx.check_count()
        assert rays > 0 and bad == 0, (bad, rays)


def test_probe_hits_vs_oracle(scene_main_bytes):
    ctx = _ctx(scene_main_bytes)
    orc = po.Scene(data=scene_main_bytes)
    run = po.Run(orc)
    m = M.by_name(M.timing_methods(), "Classique 2.0x")
    ctx.begin(m, 0, 99)
    run.begin(m, 0, 99)
    pts = list(range(0, 10728, 3))
    for state in (0, 2, 4):
        a = ctx.probe(state, pts)
        b = sorted(run.probe(state, pts))
        assert len(a) == len(b)
        ga = np.array([(r[0], r[1], r[2], r[3], r[4]) for r in a])
        gb = np.array([(r[0], r[1], r[2], r[3], r[4]) for r in b])
        same = np.all(ga == gb, axis=1)
        assert same.mean() > 0.999, same.mean()
        ta = np.array([r[5] for r in a])[same]
        tb = np.array([r[5] for r in b])[same]
        fin = np.isfinite(ta)
        assert np.all(np.abs(ta[fin] - tb[fin]) <= 1e-5 * np.abs(tb[fin]) + 1e-7)


@pytest.mark.parametrize("scen,method", [("R1 allumee-eteinte-rallumee", "Accumulation+parlampe N=32, 1.53x"),
                                         ("R1 allumee-eteinte-rallumee", "v4-A2C memoire verifiee+rampe"),
                                         ("R3 porte ouverte-fermee-rouverte", "v5-AB instantanes+projection")])
def test_gpu_matches_rtx4060_curves(scene_main_bytes, golden_main, scen, method):
    ctx = _ctx(scene_main_bytes)
    seq = M.sequence(dict(M.SCEN_SCENARIOS)[scen])
    m = M.by_name(M.scen_methods(), method)
    curve = np.zeros(len(seq))
    for sd in range(golden_main["nseeds"]):
        curve += ctx.run(m, seq, golden_main["seed0"] + sd) / golden_main["nseeds"]
    gold = [r for r in golden_main["rows"] if r["scen"] == scen and r["name"] == method][0]
    g = np.asarray(gold["curve"])
    rel = np.abs(curve - g) / g
    assert rel.max() < 2e-3, rel.max()


def test_million_point_scene_runs_clean():
    data = S.write(S.box_room(points=1_082_802, seed=0))
    ctx = _ctx(data)
    info = ctx.info()
    assert abs(info["np"] - 1_082_802) < 30_000
    m = M.by_name(M.timing_methods(), "v4-A2C suivi 1/4")
    seq = [s for s in range(5) for _ in range(12)]
    ctx.run(m, seq, 11, want_err=False)
    lc = ctx.array(N.A_LC)
    assert np.isfinite(lc).all() and lc.max() > 0
    assert ctx.device_flags() == 0


def test_image_pass_vs_oracle(scene_main_bytes):
    """The 1920x1080-class image pass (no reference counterpart) against the CPU oracle's
    restatement on the same cache: same pixel values except at geometric edges."""
    ctx = _ctx(scene_main_bytes)
    orc = po.Run(po.Scene(data=scene_main_bytes))
    m = M.by_name(M.timing_methods(), "v4-A2C suivi 1/4")
    seq = [0] * 6 + [1] * 4
    ctx.begin(m, 0, 5)
    orc.begin(m, 0, 5)
    for s in seq:
        ctx.frame(s)
    orc.array(po.A_LC)[...] = ctx.array(N.A_LC)
    orc.set_scalar(N.S_DORMANT, ctx.scalar(N.S_DORMANT))
    cam = N.camera(eye=(0.5, 0.6, 1.6), at=(7.5, 3.0, 1.0), fov_y_deg=70.0, width=640, height=360)
    img = ctx.render(1, cam)
    ref = orc.render(1, N.camera_basis(cam), 640, 360)
    assert np.isfinite(img).all() and img.max() > 0
    close = np.isclose(img, ref, rtol=1e-4, atol=1e-6)
    assert close.mean() > 0.995, close.mean()


@pytest.fixture(scope="module")
def street_bytes():
    return S.write(S.street_scene(points=20000, buildings=8, size=60.0))


def test_format3_state_build_bitexact_vs_reference(street_bytes):
    if not pyref.available(3):
        pytest.skip("reference kernels not built")
    ctx = _ctx(street_bytes)
    ref = pyref.RefRunner(3, street_bytes)
    for s in range(ctx.info()["ns"]):
        assert np.array_equal(ctx.state_array(s, N.SA_EDIR).view(np.uint32), ref.state_array(s, 0).view(np.uint32)), s
        assert np.array_equal(ctx.state_array(s, N.SA_SV), ref.state_array(s, 1)), s


@pytest.mark.parametrize("name", ["Classique 2.0x", "v3 complet", "v4-A2C suivi 1/4"])
def test_format3_frames_vs_reference(street_bytes, name):
    """BVH traversal, hash-table cache lookups and the whole frame on a format-3 scene."""
    if not pyref.available(3):
        pytest.skip("reference kernels not built")
    m = M.by_name(M.timing_methods(), name)
    seq = [0] * 10 + [1] * 6 + [2] * 6 + [3] * 6 + [4] * 6
    _frames_vs_reference(street_bytes, 3, m, seq, 7)


def test_format3_probe_vs_oracle(street_bytes):
    ctx = _ctx(street_bytes)
    run = po.Run(po.Scene(data=street_bytes))
    m = M.by_name(M.timing_methods(), "Classique 2.0x")
    ctx.begin(m, 0, 4)
    run.begin(m, 0, 4)
    pts = list(range(0, ctx.info()["np"], 5))
    for state in (0, 2):
        a = ctx.probe(state, pts)
        b = sorted(run.probe(state, pts))
        ga = np.array([r[:5] for r in a])
        gb = np.array([r[:5] for r in b])
        same = np.all(ga == gb, axis=1)
        assert same.mean() > 0.999, same.mean()
        assert (ga[:, 2] <= -2).mean() > 0.2    # most hits go through the BVH
    assert ctx.device_flags() == 0


def test_fine_transit_grid_vs_reference():
    """The 768-voxel transit grid (NW = 24) against the reference compiled with that grid."""
    if not pyref.available(3, (16, 8, 6)):
        pytest.skip("reference kernels not built")
    data = S.write(S.box_room(points=20000, seed=6))
    for name in ("v3 complet", "v4-A2C suivi 1/4"):
        m = M.by_name(M.timing_methods(), name)
        _frames_vs_reference(data, 3, m, [0] * 10 + [1] * 6 + [2] * 6 + [4] * 6, 21, grid=(16, 8, 6))


@pytest.mark.parametrize("points", [40, 300, 2500])
def test_ragged_point_counts_vs_reference(points):
    """Point counts that fill no block or tile evenly (65, 285, 2,527 points), bit for bit."""
    if not pyref.available(3):
        pytest.skip("reference kernels not built")
    data = S.write(S.box_room(points=points, seed=5))
    for name in ("Classique 1.0x", "v3 complet"):
        m = M.by_name(M.timing_methods(), name)
        _frames_vs_reference(data, 3, m, [0] * 8 + [1] * 6 + [2] * 6 + [4] * 4, 13)
