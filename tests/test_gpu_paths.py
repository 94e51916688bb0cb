"""Camera paths feeding the hash-grid cache (rc_hg_camera_paths) and the per-voxel light masks
on the GPU, against the CPU restatements (oracle/rc_oracle.c, oracle/hg_oracle.c).

The GPU traces with CUDA's cosf / sinf / rsqrtf and the oracle with the C library's, so a few
paths take another branch at a near-tie; everything is compared on the paths that agree, and
the voxel masks are compared bit for bit from the GPU's own vertices."""
import numpy as np
import pytest
import torch

from oracle import pyhg
from oracle import pyoracle as po
from render_engine_gb300 import hashgrid as H
from render_engine_gb300 import native as N
from render_engine_gb300 import scene as S

pytestmark = pytest.mark.gpu

AREA = ((3.5, 1.5, 2.95), (1.0, 0.0, 0.0), (0.0, -1.0, 0.0), (4.0, 3.5, 3.0))
SUN = ((0.3, 0.2, 1.0), (0.5, 0.5, 0.45))
RGB3 = [(1.0, 0.8, 0.6), (0.6, 0.8, 1.0), (1.0, 1.0, 1.0)]


def _gpu_pass(data, cam, state=0, bounces=2, res=32):
    ctx = N.Context()
    ctx.load_bytes(data)
    cfg = H.make_config(zone_lo=(0, 0, 0), zone_hi=(8, 4, 3), cell=0.1, capacity=1 << 20, max_depth=4, tracing_distance=50.0)
    hg = H.HashGrid(cfg)
    hg.voxels_init(res)
    hg.begin_frame(0, 16)
    img = torch.zeros(cam.width * cam.height * 3, device="cuda")
    prm = H.path_params(cam, bounces=bounces, seed=9, frame=3, light_rgb=RGB3, area=AREA, sun=SUN)
    hg.camera_paths(ctx, state, prm, img)
    torch.cuda.synchronize()
    arr = H.camera_arrays(ctx)
    out = {"arr": arr, "img": img.cpu().numpy().reshape(-1, 3), "keys": hg.download(H.A_KEYS), "accum": hg.download(H.A_ACCUM),
           "bank": hg.download(H.A_BANK0), "vox": hg.voxels(), "cfg": cfg,
           "box": hg.voxels_box_lights((3.0, 1.0, 0.0), (4.5, 2.5, 3.0))}
    hg.close()
    ctx.close()
    return out


def test_camera_paths_vs_oracle(scene_main_bytes):
    cam = N.camera((0.6, 0.5, 1.6), (6.0, 3.0, 1.0), width=96, height=64, fov_y_deg=75.0)
    g = _gpu_pass(scene_main_bytes, cam)
    sc = S.read(scene_main_bytes)
    o = po.Scene(data=scene_main_bytes)
    r = o.camera_paths(0, N.camera_basis(cam), 96, 64, 2, seed=9, frame=3, td=50.0, lpos=sc.L, inten=sc.states[0].inten,
                       light_rgb=RGB3, area=AREA, sun=SUN)
    a, S1 = g["arr"], r["stride"]
    assert a["stride"] == S1 and a["npaths"] == 96 * 64
    same_len = a["len"] == r["len"]
    assert same_len.mean() > 0.99
    gv, ov = a["vertices"], r["vertices"]
    agree = np.zeros(len(same_len), bool)
    for p in np.flatnonzero(same_len):
        sl = slice(p * S1, p * S1 + a["len"][p])
        agree[p] = (np.array_equal(gv[sl]["flags"], ov[sl]["flags"]) and np.array_equal(gv[sl]["light_index"], ov[sl]["light_index"])
                    and np.allclose(gv[sl]["hit"], ov[sl]["hit"], rtol=0, atol=1e-4))
    assert agree.mean() > 0.99
    slots = np.concatenate([np.arange(p * S1, (p + 1) * S1) for p in np.flatnonzero(agree)])
    assert np.allclose(a["rgb"][slots], r["rgb"][slots], rtol=1e-4, atol=1e-6)
    px = np.flatnonzero(agree)
    assert np.allclose(g["img"][px], r["image"][px], rtol=1e-4, atol=1e-6)
    # the cache: every slot with a surface vertex has an entry, keyed as the oracle keys the GPU's
    # own hit (hits on the room's walls lie on cell boundaries, where an ulp picks the cell)
    ent = a["entry"]
    surf = np.linalg.norm(r["nrm"], axis=1) > 0
    assert ((ent != H.INVALID) == surf)[slots].all()
    cfg = pyhg.config_from(g["cfg"])
    oc = pyhg.Cache(cfg)
    hit_g = np.where(surf[:, None], gv["hit"], 0.0).astype(np.float32)
    e_o = oc.insert(hit_g[slots], r["nrm"][slots])
    keys_o = {int(oc.keys[e]) for e in e_o if e != H.INVALID}
    keys_g = {int(g["keys"][e]) for e in ent[slots] if e != H.INVALID}
    assert keys_o == keys_g
    # samples: counts per key equal to the number of slots with that key
    cnt_g = {int(g["keys"][e]): int(g["accum"][e, 3]) for e in set(ent[ent != H.INVALID].tolist())}
    assert sum(cnt_g.values()) == int((ent != H.INVALID).sum())
    # voxel masks: bit for bit from the GPU's own vertices
    vox_o = pyhg.voxels_mark(cfg, 32, a["vertices"], a["len"], S1)
    assert np.array_equal(g["vox"], vox_o)
    assert g["vox"].any()
    v3 = g["vox"].reshape(32, 32, 32)
    sx, sy = np.float32(32) / np.float32(8), np.float32(32) / np.float32(4)
    xs = slice(int(np.float32(3.0) * sx), int(np.float32(4.5) * sx) + 1)
    ys = slice(int(np.float32(1.0) * sy), int(np.float32(2.5) * sy) + 1)
    m = np.bitwise_or.reduce(v3[:, ys, xs].reshape(-1))
    assert g["box"] == int(m)


def test_dependency_masks_of_camera_paths(scene_main_bytes):
    """The GPU's masks of its own paths equal the oracle's marking of the same vertices."""
    cam = N.camera((0.6, 0.5, 1.6), (6.0, 3.0, 1.0), width=64, height=48, fov_y_deg=75.0)
    g = _gpu_pass(scene_main_bytes, cam)
    a = g["arr"]
    cfg = pyhg.config_from(g["cfg"])
    oc = pyhg.Cache(cfg)
    oc.keys[:] = g["keys"]
    ln = a["len"]
    S1 = a["stride"]
    ps = np.concatenate([[0], np.cumsum(ln)]).astype(np.int32)
    verts = np.concatenate([a["vertices"][p * S1: p * S1 + ln[p]] for p in range(len(ln))])
    oc.mark_paths(verts, ps)
    assert np.array_equal(g["bank"], oc.bank0)
    assert g["bank"].any()


def test_camera_paths_street_format3():
    data = S.write(S.street_scene(points=12000, buildings=6, seed=2, lights=8))
    cam = N.camera((-20.0, -2.0, 2.0), (10.0, 0.0, 3.0), width=128, height=72, fov_y_deg=70.0)
    ctx = N.Context()
    ctx.load_bytes(data)
    cfg = H.make_config(zone_lo=(-60, -60, 0), zone_hi=(60, 60, 40), cell=0.5, capacity=1 << 20, tracing_distance=200.0)
    hg = H.HashGrid(cfg)
    img = torch.zeros(128 * 72 * 3, device="cuda")
    prm = H.path_params(cam, bounces=2, seed=1, sun=((0.2, 0.3, 1.0), (1.0, 0.95, 0.9)), sky=(0.2, 0.3, 0.5))
    hg.camera_paths(ctx, 0, prm, img)
    counts = torch.zeros(3, dtype=torch.int32, device="cuda")
    hg.resolve(None, counts)
    torch.cuda.synchronize()
    im = img.cpu().numpy()
    assert np.isfinite(im).all() and (im >= 0).all() and im.max() > 0
    assert int(counts[2]) > 100          # valid entries after the resolve
    a = H.camera_arrays(ctx)
    assert (a["vertices"]["flags"] & 1).any()   # some rays escape to the sky
    hg.close()
    ctx.close()
