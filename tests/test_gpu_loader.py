"""Scene loading on the GPU: the per-point arrays are copied to the device as they lie in the
file (from pinned or pageable host memory) and re-laid out there, and the range checks of
region ids and hash values run on the device before the load returns.  A scene that fails a
check is rejected with a format error and leaves the context usable."""
import numpy as np
import pytest
import torch

from render_engine_gb300 import methods as M
from render_engine_gb300 import native as N
from render_engine_gb300 import scene as S

pytestmark = pytest.mark.gpu


def _run_frames(ctx, n=3):
    m = M.by_name(M.timing_methods(), "v4-A2C suivi 1/4")
    ctx.begin(m, 0, 5)
    for _ in range(n):
        ctx.frame(0)
    return ctx.array(N.A_LC)


def test_pinned_and_pageable_sources_load_the_same_scene(scene_main_bytes):
    a = N.Context()
    a.load_bytes(scene_main_bytes)
    pinned = torch.frombuffer(bytearray(scene_main_bytes), dtype=torch.uint8).pin_memory()
    b = N.Context()
    b.load_bytes(pinned.numpy())
    for s in range(a.info()["ns"]):
        for which in (N.SA_EDIR, N.SA_SV, N.SA_REF, N.SA_VALID, N.SA_PW):
            assert np.array_equal(a.state_array(s, which), b.state_array(s, which)), (s, which)
    assert np.array_equal(_run_frames(a).view(np.uint32), _run_frames(b).view(np.uint32))


def test_bad_region_id_rejected_and_context_reusable(scene_main_bytes):
    sc = S.read(scene_main_bytes)
    sc.region = sc.region.copy()
    sc.region[len(sc.region) // 2] = sc.NR
    ctx = N.Context()
    with pytest.raises(N.RCError, match="region index out of range"):
        ctx.load_bytes(S.write(sc))
    sc.region[len(sc.region) // 2] = -1
    with pytest.raises(N.RCError, match="region index out of range"):
        ctx.load_bytes(S.write(sc))
    ctx.load_bytes(scene_main_bytes)
    assert np.isfinite(_run_frames(ctx)).all()


def test_bad_hash_value_rejected():
    sc = S.street_scene(points=4000, buildings=3)
    hv = sc.mesh["HV"].copy()
    k = int(np.flatnonzero(hv >= 0)[0])
    hv[k] = 10 ** 8
    sc.mesh = dict(sc.mesh, HV=hv)
    ctx = N.Context()
    with pytest.raises(N.RCError, match="hash value out of range"):
        ctx.load_bytes(S.write(sc))


def test_truncated_scene_rejected(scene_main_bytes):
    ctx = N.Context()
    for cut in (16, len(scene_main_bytes) // 3, len(scene_main_bytes) - 7):
        with pytest.raises(N.RCError):
            ctx.load_bytes(scene_main_bytes[:cut])
    ctx.load_bytes(scene_main_bytes)
    assert np.isfinite(_run_frames(ctx)).all()


def test_states_built_ahead_of_use_give_the_same_frames(scene_main_bytes):
    """States built ahead of use on the second stream in another order (rc_scene_build_states for
    all of them before the run, against the load's build of state 0 and the look-ahead of the next
    state during a run that jumps between states, where a state can be built on the context's
    stream at first use) hold the same direct light and give the same frames, bit for bit."""
    m = M.by_name(M.timing_methods(), "Classique 2.0x")   # no float-atomic sums: runs are bit-reproducible
    seq = [0] * 6 + [3] * 5 + [1] * 5 + [4] * 4 + [2] * 4
    out = []
    for ahead in (False, True):
        ctx = N.Context()
        ctx.load_bytes(scene_main_bytes)
        if ahead:
            ctx.build_states()
            ctx.sync()
        ctx.begin(m, seq[0], 7)
        for s in seq:
            ctx.frame(s)
        ctx.sync()
        assert ctx.device_flags() == 0
        out.append((ctx.array(N.A_LC).copy(), [ctx.state_array(k, N.SA_EDIR).copy() for k in range(5)]))
        ctx.close()
    assert np.array_equal(out[0][0], out[1][0])
    for a, b in zip(out[0][1], out[1][1]):
        assert np.array_equal(a, b)


def test_async_load_gives_the_same_states_and_frames(scene_main_bytes):
    """RC_FLAG_LOAD_ASYNC (the states after the first copied on the second stream behind the load,
    from a buffer the caller keeps): the same state arrays and the same frames as a plain load,
    whether a state is first built ahead of use or on demand."""
    m = M.by_name(M.timing_methods(), "Classique 2.0x")
    seq = [0] * 4 + [3] * 4 + [1] * 4 + [4] * 3 + [2] * 3
    pinned = torch.frombuffer(bytearray(scene_main_bytes), dtype=torch.uint8).pin_memory()
    out = []
    for flags in (0, N.FLAG_LOAD_ASYNC):
        ctx = N.Context(flags=flags)
        ctx.load_bytes(pinned.numpy())
        ctx.begin(m, seq[0], 9)
        for s in seq:
            ctx.frame(s)
        ctx.sync()
        assert ctx.device_flags() == 0
        states = [[ctx.state_array(k, w).copy() for w in (N.SA_EDIR, N.SA_SV, N.SA_REF, N.SA_VALID, N.SA_PW)] for k in range(5)]
        out.append((ctx.array(N.A_LC).copy(), states))
        ctx.close()
    assert np.array_equal(out[0][0], out[1][0])
    for a, b in zip(out[0][1], out[1][1]):
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
