"""Pins the restatement of the bench's dependency encoding to the reference's own code, extracted
unchanged from a reference checkout and compiled as C++ by oracle/build_patch_ref.sh:

* the shader functions DepMarkPoint and DepMarkSegment (rtxgi_bench.patch:825-858; HLSL's vector
  types from oracle/hlsl_compat.h, IEEE single precision, no contraction) against oracle/
  hg_oracle.c's hgo_mark_point / hgo_mark_segment, the checker of the GPU kernels in
  csrc/rc_hashgrid.cu: masks equal bit for bit on random points and segments, on points on the
  zone boundaries, on axis-aligned and degenerate segments, on segments that miss the box and on
  long ones (the 48-step cap);
* the host function Pathtracer::BenchObjVoxels (patch:592-615, the zones an object invalidates)
  against the oracle's event mask and the library's own rc_hg_event_mask (host code, no GPU):
  equal zone words for random objects, objects on zone edges and objects outside the box;
* the snapshot compute shaders of BenchSnap.hlsl (patch:1283-1345: count, pack, restore),
  dispatched one thread after another, against the oracle's snapshot and restore (the checker
  of rc_hg_snapshot / rc_hg_restore): the same records in the same (entry) order, and the same
  table after a restore, on tables with empty, evicted, sample-less and live entries.

Skipped without a reference checkout (the patch is read from there)."""
import ctypes
import os

import numpy as np
import pytest

from oracle import build as OB
from oracle import pyhg

LIB = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref", "libpatch_ref.so")


@pytest.fixture(scope="module")
def href():
    if not OB.build_patch_ref():
        pytest.skip("no reference checkout (the patch is read from there)")
    L = ctypes.CDLL(LIB)
    vp = ctypes.c_void_p
    L.href_mark_point.argtypes = [vp, vp, vp, vp]
    L.href_mark_segment.argtypes = [vp, vp, vp, vp, vp]
    L.href_obj_voxels.argtypes = [vp, vp, vp, vp]
    L.href_snapshot.argtypes = [vp, vp, ctypes.c_uint32, vp, ctypes.c_uint32]
    L.href_snapshot.restype = ctypes.c_uint32
    L.href_restore.argtypes = [vp, vp, ctypes.c_uint32, vp, ctypes.c_uint32]
    return L


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


BOXES = [((0.0, 0.0, 0.0), (8.0, 4.0, 3.0)), ((-3.5, 0.25, -1.0), (9.1, 7.0, 2.2)), ((10.0, -20.0, 0.0), (130.0, 40.0, 55.0))]


@pytest.mark.parametrize("box", BOXES)
def test_mark_point_equals_the_shader(href, box):
    lo, hi = np.array(box[0], np.float32), np.array(box[1], np.float32)
    cfg = pyhg.Config()
    cfg.zone_lo[:], cfg.zone_hi[:] = lo.tolist(), hi.tolist()
    rng = np.random.default_rng(3)
    ext = hi - lo
    pts = [rng.uniform(lo - 0.1 * ext, hi + 0.1 * ext).astype(np.float32) for _ in range(20000)]
    # zone boundaries and the box's faces, a few ulps either side
    for k in range(3):
        for z in range(int((6, 4, 4)[k]) + 1):
            c = np.float32(lo[k] + ext[k] * z / (6, 4, 4)[k])
            for e in (np.float32(-np.inf), np.float32(0), np.float32(np.inf)):
                p = rng.uniform(lo, hi).astype(np.float32)
                p[k] = c if e == 0 else np.nextafter(c, e)
                pts.append(p)
    for p in pts:
        a, b = np.zeros(3, np.uint32), np.zeros(3, np.uint32)
        href.href_mark_point(_p(lo), _p(hi), _p(a), _p(p))
        b[:] = pyhg.mark_point(cfg, p)
        assert np.array_equal(a, b), (p, a, b)


@pytest.mark.parametrize("box", BOXES)
def test_mark_segment_equals_the_shader(href, box):
    lo, hi = np.array(box[0], np.float32), np.array(box[1], np.float32)
    cfg = pyhg.Config()
    cfg.zone_lo[:], cfg.zone_hi[:] = lo.tolist(), hi.tolist()
    rng = np.random.default_rng(5)
    ext = hi - lo
    segs = []
    for _ in range(20000):
        a = rng.uniform(lo - 0.5 * ext, hi + 0.5 * ext).astype(np.float32)
        b = rng.uniform(lo - 0.5 * ext, hi + 0.5 * ext).astype(np.float32)
        segs.append((a, b))
    for _ in range(2000):   # axis-aligned, degenerate, short and very long segments
        a = rng.uniform(lo, hi).astype(np.float32)
        b = a.copy()
        k = int(rng.integers(0, 3))
        b[k] = np.float32(b[k] + rng.uniform(-2, 2) * ext[k])
        segs.append((a, b))
        segs.append((a, a.copy()))
        segs.append((a, (a + np.float32(1e-6)).astype(np.float32)))
        segs.append((a, (a + rng.normal(size=3).astype(np.float32) * np.float32(50) * ext).astype(np.float32)))
    for a, b in segs:
        m1, m2 = np.zeros(3, np.uint32), np.zeros(3, np.uint32)
        href.href_mark_segment(_p(lo), _p(hi), _p(m1), _p(a), _p(b))
        m2[:] = pyhg.mark_segment(cfg, a, b)
        assert np.array_equal(m1, m2), (a, b, m1, m2)


@pytest.mark.parametrize("box", BOXES)
def test_object_zones_equal_the_reference(href, box):
    from render_engine_gb300 import hashgrid as H
    lo, hi = np.array(box[0], np.float32), np.array(box[1], np.float32)
    cfg = pyhg.Config()
    cfg.zone_lo[:], cfg.zone_hi[:] = lo.tolist(), hi.tolist()
    lib_cfg = H.make_config(zone_lo=tuple(lo.tolist()), zone_hi=tuple(hi.tolist()))
    rng = np.random.default_rng(7)
    ext = hi - lo
    cs = ext / np.array([6, 4, 4], np.float32)
    objs = []
    for _ in range(3000):
        c = rng.uniform(lo - 0.2 * ext, hi + 0.2 * ext)
        size = rng.uniform(0.01, 0.5, 3) * ext
        objs.append(np.concatenate([c, size]).astype(np.float32))
    for _ in range(500):   # faces 0.25 (the margin) away from a zone edge, exactly
        k = int(rng.integers(0, 3))
        z = int(rng.integers(0, (6, 4, 4)[k] + 1))
        c = rng.uniform(lo, hi)
        size = rng.uniform(0.05, 0.3, 3) * ext
        c[k] = lo[k] + cs[k] * z - 0.25 - 0.5 * size[k]
        objs.append(np.concatenate([c, size]).astype(np.float32))
    for o in objs:
        want = np.zeros(4, np.uint32)
        href.href_obj_voxels(_p(lo), _p(hi), _p(o), _p(want))
        got_oracle = pyhg.event_mask(cfg, obj_a=o)
        got_lib = H.event_mask(lib_cfg, obj_a=o)
        assert np.array_equal(want[:3], got_oracle[:3]), (o, want, got_oracle)
        assert np.array_equal(want[:3], got_lib[:3]), (o, want, got_lib)


SNAP = np.dtype([("index", "<u4"), ("sample_data", "<u4"), ("key", "<u4", 2), ("radiance", "<u4", 2)])


def _table(rng, cap):
    """A table in the states the cache leaves entries in: empty (key 0, all zero), evicted (key
    all ones, resolved zero), live without samples (fp16 count 0) and live with samples."""
    keys = np.zeros(cap, np.uint64)
    res = np.zeros((cap, 4), np.uint32)
    kind = rng.choice(4, cap, p=[0.4, 0.05, 0.1, 0.45])
    live = kind >= 2
    keys[kind == 1] = np.uint64(0xFFFFFFFFFFFFFFFF)
    keys[live] = rng.integers(1, 2**63, live.sum(), dtype=np.int64).astype(np.uint64)
    n = live.sum()
    rgb = rng.random((n, 3)).astype(np.float16).view(np.uint16).astype(np.uint32)
    cnt = np.where(kind[live] == 3, rng.integers(1, 64, n), 0).astype(np.float16).view(np.uint16).astype(np.uint32)
    res[live, 0] = rgb[:, 0] | rgb[:, 1] << 16
    res[live, 1] = rgb[:, 2] | cnt << 16
    res[live, 2] = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    return keys, res


def test_snapshot_shaders_equal_the_oracle(href):
    rng = np.random.default_rng(11)
    cap = 1 << 16
    cfg = pyhg.Config()
    cfg.capacity = cap
    for trial in range(4):
        keys, res = _table(rng, cap)
        cache = pyhg.Cache(cfg)
        cache.keys[:] = keys
        cache.resolved[:] = res
        mine = cache.snapshot(SNAP)
        theirs = np.zeros(cap, SNAP)
        k2, r2 = keys.copy(), res.copy()
        n = href.href_snapshot(_p(k2), _p(r2), cap, _p(theirs), cap)
        assert n == len(mine) and n > 0
        assert np.array_equal(mine.view(np.uint32), theirs[:n].view(np.uint32))
        # a capacity below the count: both keep the first records and report the full count
        short = np.zeros(n // 2, SNAP)
        assert href.href_snapshot(_p(k2), _p(r2), cap, _p(short), n // 2) == n
        assert np.array_equal(short.view(np.uint32), mine[: n // 2].view(np.uint32))
        # restore into a table whose restored entries hold something else
        k_a, r_a = _table(rng, cap)
        cache2 = pyhg.Cache(cfg)
        cache2.keys[:] = k_a
        cache2.resolved[:] = r_a
        cache2.restore(mine)
        k_b, r_b = k_a.copy(), r_a.copy()
        href.href_restore(_p(k_b), _p(r_b), cap, _p(theirs), n)
        assert np.array_equal(cache2.keys, k_b)
        assert np.array_equal(cache2.resolved, r_b)
