"""Camera paths feeding the hash-grid cache, and the per-voxel light masks: the CPU
restatements (oracle/rc_oracle.c osc_camera_paths, oracle/hg_oracle.c hgo_voxels_mark).
No reference exists for either (bench B has no camera; bench A's path tracer is HLSL), so
these tests state their invariants; tests/test_gpu_paths.py compares the GPU with them."""
import numpy as np
import pytest

from oracle import pyhg
from oracle import pyoracle as po
from render_engine_gb300 import hashgrid as H
from render_engine_gb300 import native as N
from render_engine_gb300 import scene as S

AREA = ((3.5, 1.5, 2.95), (1.0, 0.0, 0.0), (0.0, -1.0, 0.0), (4.0, 3.5, 3.0))   # 1 x 1 m, facing down
SUN = ((0.3, 0.2, 1.0), (0.5, 0.5, 0.45))


@pytest.fixture(scope="module")
def room(scene_main_bytes):
    return po.Scene(data=scene_main_bytes), S.read(scene_main_bytes)


def _run(o, sc, state=0, scale=1.0, bounces=2, w=64, h=48, area=AREA, sun=SUN):
    cam = N.camera((0.6, 0.5, 1.6), (6.0, 3.0, 1.0), width=w, height=h, fov_y_deg=75.0)
    a = None if area is None else (area[0], area[1], area[2], tuple(scale * x for x in area[3]))
    s = None if sun is None else (sun[0], tuple(scale * x for x in sun[1]))
    return o.camera_paths(state, N.camera_basis(cam), w, h, bounces, seed=9, frame=3, td=50.0, lpos=sc.L,
                          inten=np.asarray(sc.states[state].inten) * scale, area=a, sun=s)


def test_path_records(room):
    o, sc = room
    r = _run(o, sc)
    v, ln, S1 = r["vertices"], r["len"], r["stride"]
    assert S1 == 3 and ln.min() >= 0 and ln.max() <= 3 and (ln > 0).mean() > 0.9
    for p in range(len(ln)):
        for k in range(S1):
            x = v[p * S1 + k]
            n = r["nrm"][p * S1 + k]
            if k >= ln[p]:
                assert not n.any() and not r["rgb"][p * S1 + k].any()
            elif x["flags"] & 1:
                assert k == ln[p] - 1 and not n.any()
            else:
                assert abs(np.linalg.norm(n) - 1) < 1e-5 and -1 <= x["light_index"] <= sc.NL + 1
    assert np.isfinite(r["rgb"]).all() and (r["rgb"] >= 0).all()
    lit = r["rgb"][::S1]
    assert (lit.sum(axis=1) > 0).mean() > 0.5
    assert {int(x) for x in v["light_index"][v["light_index"] >= 0]} >= {0, sc.NL}   # point lights and the rectangle


def test_radiance_linear_in_the_lights(room):
    o, sc = room
    a, b = _run(o, sc), _run(o, sc, scale=2.0)
    assert (a["len"] == b["len"]).all()
    assert np.array_equal(2.0 * a["rgb"], b["rgb"])    # same choices, every term scaled by a power of two
    c = _run(o, sc, area=None, sun=None)
    assert c["vertices"]["light_index"].max() < sc.NL


def test_voxel_masks_by_hand():
    cfg = pyhg.config_from(H.make_config(zone_lo=(0, 0, 0), zone_hi=(8, 4, 3), tracing_distance=50.0))
    v = np.zeros(2, H.VERTEX_DTYPE)
    v[0]["hit"] = (1.05, 1.05, 0.55)
    v[0]["to_light"] = (0.0, 0.0, 1.0)
    v[0]["light_dist"] = 2.0
    v[0]["light_index"] = 5
    v[0]["flags"] = 2
    v[1] = v[0]
    v[1]["flags"] = 0        # shadow ray blocked: nothing
    vox = pyhg.voxels_mark(cfg, 8, v, np.array([2], np.int32), 2).reshape(8, 8, 8)   # z, y, x
    zs = sorted({int(z) for z, y, x in zip(*np.nonzero(vox))})
    assert set(np.unique(vox)) == {0, 1 << 5}
    assert zs == [1, 2, 3, 4, 5, 6] and set(np.nonzero(vox)[1]) == {2} and set(np.nonzero(vox)[2]) == {1}
