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
  equal zone words for random objects, objects on zone edges and objects outside the box.

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
