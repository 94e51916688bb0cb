"""Pins the restatement of the bench's dependency marking (oracle/hg_oracle.c: hgo_mark_point,
hgo_mark_segment, the checker of the GPU kernels in csrc/rc_hashgrid.cu) to the reference's own
shader functions DepMarkPoint and DepMarkSegment (rtxgi_bench.patch:825-858), extracted unchanged
from a reference checkout and compiled as C++ by oracle/build_hlsl_ref.sh (HLSL's vector types
from oracle/hlsl_compat.h, IEEE single precision, no contraction).  The masks must be equal bit
for bit on random points and segments, on points on the zone boundaries, on axis-aligned and
degenerate segments, on segments that miss the box and on long ones (the 48-step cap).  Skipped
without a reference checkout (the shader source is read from there)."""
import ctypes
import os

import numpy as np
import pytest

from oracle import build as OB
from oracle import pyhg

LIB = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref", "libhlsl_dep.so")


@pytest.fixture(scope="module")
def href():
    if not OB.build_hlsl_ref():
        pytest.skip("no reference checkout (the shader functions are read from there)")
    L = ctypes.CDLL(LIB)
    vp = ctypes.c_void_p
    L.href_mark_point.argtypes = [vp, vp, vp, vp]
    L.href_mark_segment.argtypes = [vp, vp, vp, vp, vp]
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
