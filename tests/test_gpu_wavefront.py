"""The ray-queue traversal of static-mesh scenes (k_ray_queue, k_trace_queue; RC_FLAG_RAY_QUEUE)
against the one-thread-per-point traversal (k_pretrace, the default): the same rays
with the same per-ray visit order.  The two contexts run in lockstep, the second one given the
first one's run state before every frame, as the parity tests do with the reference, so a frame
is compared from identical inputs: bit for bit, except on the frames whose own outputs depend on
float sums taken with atomics in an undefined order (verification and event frames of the
adaptive methods), held to the parity tests' bound.  Reference mode and watertight mode, on a
median-split tree and on the preparation's linear BVH.  Frames against the reference's own
kernels are in test_gpu_parity.py."""
import numpy as np
import pytest

from render_engine_gb300 import methods as M
from render_engine_gb300 import native as N
from render_engine_gb300 import scene as S

pytestmark = pytest.mark.gpu

SEQ = [0] * 8 + [1] * 5 + [2] * 5 + [3] * 4 + [4] * 4
SYNC = [N.A_LC, N.A_N, N.A_C0, N.A_PENDING, N.A_CUR, N.A_PREV, N.A_STALE, N.A_AGE, N.A_SNAP, N.A_NEQ, N.A_COEF,
        N.A_RSTAT, N.A_DSTAT, N.A_SUMPR, N.A_NPEND]


def _lockstep(data, flags, method, seq, seed):
    a = N.Context(flags=flags | N.FLAG_RAY_QUEUE)
    b = N.Context(flags=flags)
    for c in (a, b):
        c.load_bytes(data)
        c.begin(method, seq[0], seed)
    exact = 0
    for f, s in enumerate(seq):
        for w in SYNC:
            b.set_array(w, a.array(w))
        for k in range(7):
            b.set_scalar(k, a.scalar(k))
        pend_before = a.scalar(N.S_PEND_LEFT)
        event = f > 0 and seq[f - 1] != s
        a.frame(s)
        b.frame(s)
        pend_after = a.scalar(N.S_PEND_LEFT)
        loose = pend_before > 0 or (event and (method.mode == 1 or pend_after > 0))
        if not loose:
            for w in (N.A_LC, N.A_N, N.A_KK, N.A_CUR, N.A_PENDING):
                x, y = a.array(w), b.array(w)
                assert np.array_equal(x.view(np.uint8), y.view(np.uint8)), (f, w)
            exact += 1
        else:
            x, y = a.array(N.A_LC), b.array(N.A_LC)
            assert np.isclose(x, y, rtol=1e-4, atol=1e-6).mean() >= 0.998, f
    ra, rb = a.stats()["rays"], b.stats()["rays"]
    assert a.device_flags() == 0 and b.device_flags() == 0
    a.close()
    b.close()
    return exact, ra, rb


@pytest.fixture(scope="module")
def street_median():
    return S.write(S.street_scene(points=30000, buildings=10, size=80.0))


@pytest.fixture(scope="module")
def street_prepared(tmp_path_factory):
    d = tmp_path_factory.mktemp("wq")
    V, alb, ds = S.street_mesh(buildings=10, seed=4, facade_cell=1.5, size=80.0)
    mesh = d / "m.msh"
    mesh.write_bytes(S.write_msh1(V, alb, ds))
    ctx = N.Context()
    ctx.prep_mesh(str(mesh), str(d / "s.bin"), points=30000)
    ctx.close()
    return (d / "s.bin").read_bytes()


@pytest.mark.parametrize("which", ["street_median", "street_prepared"])
@pytest.mark.parametrize("name", ["Classique 2.0x", "v3 complet", "v4-A2C suivi 1/4"])
def test_queue_equals_thread_per_point(request, which, name):
    data = request.getfixturevalue(which)
    m = M.by_name(M.timing_methods(), name)
    exact, ra, rb = _lockstep(data, 0, m, SEQ, 9)
    assert exact >= len(SEQ) // 2 and ra > 0
    if m.mode == 0:
        assert exact == len(SEQ) and ra == rb


def test_queue_equals_thread_per_point_watertight(street_prepared):
    m = M.by_name(M.timing_methods(), "Classique 2.0x")
    exact, ra, rb = _lockstep(street_prepared, N.FLAG_WATERTIGHT, m, SEQ[:16], 3)
    assert exact == 16 and ra == rb
