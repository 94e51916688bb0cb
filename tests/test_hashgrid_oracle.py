"""CPU checks of the hash-grid oracle (oracle/hg_oracle.c) and of the library's host-only
event mask.

Known answers worked by hand from the HLSL of windows/patch/rtxgi_bench.patch
(DepMarkPoint / DepMarkSegment / DepOr / the path loop / the resolve invalidation /
BenchObjVoxels / BenchSnap), and numpy's float16 as the independent check of the fp16
rounding.  No GPU needed."""
import numpy as np

from oracle import pyhg
from render_engine_gb300 import hashgrid as H


def cfg(**kw):
    return pyhg.config_from(H.make_config(**kw))


def bits(m):
    out = set()
    for w, x in enumerate(m):
        for b in range(32):
            if int(x) >> b & 1:
                out.add(32 * w + b)
    return out


def zone(x, y, z):
    return x + 6 * (y + 4 * z)


def test_fp16_rounding_matches_numpy():
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.normal(0, 1, 20000), rng.normal(0, 1e-5, 5000), rng.normal(0, 1e-7, 5000),
                         rng.uniform(6e4, 7e4, 2000), [0.0, -0.0, 65504.0, 65519.99, 65520.0, 2.0 ** -24, 2.0 ** -25,
                                                     3 * 2.0 ** -26, 1.0 + 2.0 ** -11, 1.0 + 3 * 2.0 ** -11]]).astype(np.float32)
    with np.errstate(over="ignore"):
        want = xs.astype(np.float16).view(np.uint16)
    got = np.array([pyhg.f2h(float(x)) for x in xs], np.uint16)
    assert np.array_equal(got, want)
    hs = np.arange(0, 0x7C00, 7, dtype=np.uint16)
    back = np.array([pyhg.h2f(int(h)) for h in hs], np.float32)
    assert np.array_equal(back, hs.view(np.float16).astype(np.float32))


def test_mark_point_known_answers():
    c = cfg()   # zones over [0,8] x [0,4] x [0,3]: 6 x 4 x 4 cells of 1.333 x 1 x 0.75
    assert bits(pyhg.mark_point(c, [0.1, 0.1, 0.1])) == {0}
    assert bits(pyhg.mark_point(c, [7.9, 3.9, 2.9])) == {zone(5, 3, 3)} == {95}
    assert bits(pyhg.mark_point(c, [1.4, 2.5, 0.8])) == {zone(1, 2, 1)}
    assert bits(pyhg.mark_point(c, [8.0, 1.0, 1.0])) == set()          # c == G is outside
    assert bits(pyhg.mark_point(c, [-0.01, 1.0, 1.0])) == set()


def test_mark_segment_known_answers():
    c = cfg()
    assert bits(pyhg.mark_segment(c, [0.1, 0.5, 0.3], [7.9, 0.5, 0.3])) == {zone(x, 0, 0) for x in range(6)}
    assert bits(pyhg.mark_segment(c, [9.0, 5.0, 4.0], [12.0, 6.0, 5.0])) == set()   # misses the box
    # clipped to the box: only the part inside is marked
    assert bits(pyhg.mark_segment(c, [-5.0, 0.5, 0.3], [0.5, 0.5, 0.3])) == {0}
    # a zero-length segment marks its point
    assert bits(pyhg.mark_segment(c, [1.4, 2.5, 0.8], [1.4, 2.5, 0.8])) == {zone(1, 2, 1)}


def test_mark_segment_marks_only_zones_on_the_segment():
    c = cfg()
    rng = np.random.default_rng(1)
    lo, hi = np.array([0, 0, 0]), np.array([8, 4, 3])
    for _ in range(300):
        a = rng.uniform(-2, 10, 3) * np.array([1, 0.5, 0.4])
        b = rng.uniform(-2, 10, 3) * np.array([1, 0.5, 0.4])
        got = bits(pyhg.mark_segment(c, a, b))
        ts = np.linspace(0, 1, 4001)[:, None]
        pts = a[None] + (b - a)[None] * ts
        cc = (pts - lo) / (hi - lo) * np.array([6, 4, 4])
        ok = np.all((cc >= 0) & (cc < np.array([6, 4, 4])), axis=1)
        v = cc[ok].astype(int)
        dense = set((v[:, 0] + 6 * (v[:, 1] + 4 * v[:, 2])).tolist())
        assert got <= dense | _neighbours(dense)


def _neighbours(zs):
    out = set()
    for z in zs:
        x, y, k = z % 6, (z // 6) % 4, z // 24
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dk in (-1, 0, 1):
                    if 0 <= x + dx < 6 and 0 <= y + dy < 4 and 0 <= k + dk < 4:
                        out.add(zone(x + dx, y + dy, k + dk))
    return out


def _vertex(origin, hit=(0, 0, 0), d=(0, 0, 1), to_light=(0, 0, 1), light_dist=1.0, light=-1, entry=H.INVALID, flags=0):
    v = np.zeros(1, H.VERTEX_DTYPE)
    v["origin"], v["dir"], v["hit"], v["to_light"] = origin, d, hit, to_light
    v["light_dist"], v["light_index"], v["entry"], v["flags"] = light_dist, light, entry, flags
    return v


def test_path_propagation_rules():
    c = cfg(capacity=64, max_depth=4, tracing_distance=100.0)
    A, B = (1.0, 0.5, 0.3), (6.0, 3.5, 2.5)
    path = np.concatenate([
        _vertex((1.0, 0.5, 2.9), hit=A, to_light=(0, 0, 1), light_dist=2.0, light=3, entry=5, flags=H.LIGHT_VISIBLE),
        _vertex(A, hit=B, to_light=(-1, 0, 0), light_dist=0.5, light=1, entry=9, flags=0),
        _vertex(B, d=(0, 0, 1), flags=H.MISS),
    ])
    cache = pyhg.Cache(c)
    cache.mark_paths(path, np.array([0, 3]))
    pt = lambda p: pyhg.mark_point(c, p)
    seg = lambda a, b: pyhg.mark_segment(c, a, b)
    # vertex 0 (entry 5): its point, its shadow segment, light 3
    cur0 = pt(A) | seg(A, (1.0, 0.5, 2.3))
    # vertex 1 (entry 9): its point and shadow segment (light 1 not visible), and entry 5 inherits them
    # with vertex 1's incoming segment
    cur1 = pt(B) | seg(B, (5.5, 3.5, 2.5))
    in1 = seg(A, B)
    sky = seg(B, (6.0, 3.5, 102.5))
    want5 = np.concatenate([cur0 | cur1 | in1 | sky, [(1 << 3) | H.SKY_BIT]]).astype(np.uint32)
    want9 = np.concatenate([cur1 | sky, [H.SKY_BIT]]).astype(np.uint32)
    assert np.array_equal(cache.bank0[5], want5)
    assert np.array_equal(cache.bank0[9], want9)
    assert not cache.bank1.any() and cache.bank0[np.r_[0:5, 6:9, 10:64]].sum() == 0


def test_stop_vertex_passes_on_its_entry_masks():
    c = cfg(capacity=64)
    cache = pyhg.Cache(c)
    cache.bank1[7] = [0, 0, 1 << 4, 1 << 9]     # what entry 7 depends on from earlier frames
    A, B = (1.0, 0.5, 0.3), (6.0, 3.5, 2.5)
    path = np.concatenate([_vertex((1.0, 0.5, 2.9), hit=A, entry=3), _vertex(A, hit=B, entry=7, flags=H.STOP),
                           _vertex(B, flags=H.MISS)])
    cache.mark_paths(path, np.array([0, 3]))
    got3 = cache.bank0[3]
    assert got3[2] & (1 << 4) and got3[3] & (1 << 9)     # inherited
    assert not got3[3] & H.SKY_BIT                        # the path stopped before the miss
    assert np.array_equal(cache.bank0[7][:3], pyhg.mark_point(c, B))


def test_depth_limits_propagation():
    c = cfg(capacity=64, max_depth=2)
    cache = pyhg.Cache(c)
    pts = [(0.5 + 1.5 * k, 0.5, 0.4) for k in range(4)]   # zones x = 0, 1, 2, 3
    path = np.concatenate([_vertex(pts[k - 1] if k else (0.5, 0.5, 2.9), hit=pts[k], entry=10 + k) for k in range(4)])
    cache.mark_paths(path, np.array([0, 4]))
    # with two kept vertices, vertex k reaches only vertex k - 1: entry 10 sees vertex 1, not vertex 2
    assert bits(cache.bank0[10][:3]) & bits(pyhg.mark_point(c, pts[1]))
    assert not bits(cache.bank0[10][:3]) & bits(pyhg.mark_point(c, pts[2]))


def test_bank_rotation():
    c = cfg(capacity=32)
    cache = pyhg.Cache(c)
    cache.bank0[:] = 1
    cache.bank1[:] = 2
    cache.begin_frame(0, 16)
    assert cache.bank == 0 and not cache.bank0.any() and (cache.bank1 == 2).all()
    cache.begin_frame(5, 16)
    assert cache.bank == 0
    cache.begin_frame(16, 16)
    assert cache.bank == 1 and not cache.bank1.any()
    cache.begin_frame(32, 16)
    assert cache.bank == 0


def _h(x):
    return int(np.float16(x).view(np.uint16))


def test_resolve_invalidation_and_accumulation():
    c = cfg(capacity=32, acc_frames=8, stale_frames=2)
    cache = pyhg.Cache(c)
    cache.keys[[1, 2, 3, 4]] = [11, 12, 13, 14]
    for e in (1, 2, 3, 4):
        cache.resolved[e] = [_h(1.0) | _h(2.0) << 16, _h(3.0) | _h(4.0) << 16, 4, 0]
    cache.bank0[1] = [1, 0, 0, 0]          # depends on zone 0
    cache.bank1[2] = [0, 0, 0, 1 << 5]     # depends on light 5
    # entry 3 has no mask at all; entry 4 depends on zone 1
    cache.bank0[4] = [2, 0, 0, 0]
    cache.accum[4] = [4 * 1024, 0, 1024, 2]
    counts = cache.resolve([1, 0, 0, 0])   # zone 0 changed
    assert counts[0] == 2                  # entry 1 (meets) and entry 3 (no mask: invalidated by prudence)
    assert cache.resolved[1, 2] == 1 << 16 and cache.resolved[1, 1] >> 16 == 0   # zeroed, then one stale frame
    assert cache.resolved[2, 2] == 4 | 1 << 16                                   # untouched, one stale frame
    # entry 4: (old 1,2,3 x 4 samples + new sums 4,0,1 over 2 samples) / 6
    r = cache.resolved[4]
    got = [np.uint16(r[0] & 0xFFFF).view(np.float16), np.uint16(r[0] >> 16).view(np.float16),
           np.uint16(r[1] & 0xFFFF).view(np.float16), np.uint16(r[1] >> 16).view(np.float16)]
    assert [float(x) for x in got] == [float(np.float16(8 / 6)), float(np.float16(8 / 6)), float(np.float16(13 / 6)), 6.0]
    assert r[2] == 6 and not cache.accum.any()
    # nothing changed: no invalidation; entries without samples age out after stale_frames
    for _ in range(3):
        cache.resolve()
    assert cache.keys[4] == H.EVICTED and cache.keys[2] == H.EVICTED and not cache.bank1[2].any()


def test_resolve_caps_the_sample_count():
    c = cfg(capacity=32, acc_frames=8)
    cache = pyhg.Cache(c)
    cache.keys[0] = 5
    cache.resolved[0] = [_h(1.0), _h(1.0) | _h(6.0) << 16, 6, 0]
    cache.accum[0] = [5 * 1024, 0, 0, 5]
    cache.resolve()
    assert cache.resolved[0, 2] == 8 and cache.resolved[0, 1] >> 16 == _h(8.0)


def test_event_mask_known_answer_and_library_agrees():
    c = cfg()
    want = np.array([0xC70001C7, 0x1, 0x0, 0x80000002], np.uint32)
    args = ([1, 1, 1], [1, 0.5, 1], 0, 1, [1, 1, 0.5, 0.5, 0.5, 0.5], [3, 1, 0.5, 0.5, 0.5, 0.5])
    assert np.array_equal(pyhg.event_mask(c, *args), want)
    assert np.array_equal(H.event_mask(H.make_config(), *args), want)
    assert not pyhg.event_mask(c, [1, 2], [1, 2], 1, 1, [1, 1, 1, 1, 1, 1], [1, 1, 1, 1, 1, 1]).any()
    rng = np.random.default_rng(3)
    for _ in range(200):
        la, lb = rng.integers(0, 2, 40).astype(float), rng.integers(0, 2, 40).astype(float)
        oa = np.r_[rng.uniform(-1, 9, 3), rng.uniform(0.1, 3, 3)]
        ob = oa if rng.random() < 0.3 else np.r_[rng.uniform(-1, 9, 3), rng.uniform(0.1, 3, 3)]
        sa, sb = int(rng.integers(0, 2)), int(rng.integers(0, 2))
        assert np.array_equal(pyhg.event_mask(c, la, lb, sa, sb, oa, ob), H.event_mask(H.make_config(), la, lb, sa, sb, oa, ob))


def test_insert_and_snapshot_round_trip():
    c = cfg(capacity=1 << 12, cell=0.5)
    cache = pyhg.Cache(c)
    rng = np.random.default_rng(4)
    pos = rng.uniform(0, 8, (3000, 3)).astype(np.float32)
    nrm = rng.normal(size=(3000, 3)).astype(np.float32)
    e = cache.insert(pos, nrm)
    assert (e != H.INVALID).all()
    assert all(cache.keys[e[i]] == pyhg.key(c, pos[i], nrm[i]) for i in range(0, 3000, 7))
    cache.accumulate(e, rng.uniform(0, 2, (3000, 3)))
    cache.resolve()
    snap = cache.snapshot(H.SNAP_DTYPE)
    assert len(snap) == len(np.unique(e)) and np.all(np.diff(snap["index"].astype(np.int64)) > 0)
    keys, res = cache.keys.copy(), cache.resolved.copy()
    cache.keys[:] = 0
    cache.resolved[:] = 0
    cache.restore(snap)
    assert np.array_equal(cache.keys, keys)
    assert np.array_equal(cache.resolved[:, :2], res[:, :2]) and np.array_equal(cache.resolved[:, 2], res[:, 2] & 0xFFFF)


def test_evicted_slot_keeps_later_keys_reachable():
    c = cfg(capacity=32, cell=1.0)
    cache = pyhg.Cache(c)
    rng = np.random.default_rng(6)
    pos = rng.uniform(0, 30, (400, 3)).astype(np.float32)
    nrm = np.tile(np.float32([0, 0, 1]), (400, 1))
    keys = np.array([pyhg.key(c, p, n) for p, n in zip(pos, nrm)], np.uint64)
    # two keys whose probes start at the same slot: the second lands one slot further
    slot = {}
    pair = None
    for i, k in enumerate(keys):
        h = int(_mix64(int(k))) & 31
        if h in slot and keys[slot[h]] != k:
            pair = (slot[h], i)
            break
        slot.setdefault(h, i)
    a, b = pair
    e = cache.insert(pos[[a, b]], nrm[[a, b]])
    assert e[1] == (e[0] + 1) % 32
    cache.keys[e[0]] = H.EVICTED                  # the first one is evicted
    again = cache.insert(pos[[b]], nrm[[b]])
    assert again[0] == e[1]                       # still found past the evicted slot
    new = cache.insert(pos[[a]], nrm[[a]])
    assert new[0] == e[0]                         # a missing key reuses the evicted slot


def _mix64(x):
    m = (1 << 64) - 1
    x ^= x >> 30; x = (x * 0xbf58476d1ce4e5b9) & m; x ^= x >> 27; x = (x * 0x94d049bb133111eb) & m; x ^= x >> 31
    return x
