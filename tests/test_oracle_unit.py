"""Unit checks of the oracle's integer building blocks and loader (no GPU)."""
import numpy as np
import pytest

from oracle import pyoracle as po
from render_engine_gb300 import methods as M
from render_engine_gb300 import scene as S


def hash32(x):
    x &= 0xFFFFFFFF
    x ^= x >> 16; x = (x * 0x7FEB352D) & 0xFFFFFFFF
    x ^= x >> 15; x = (x * 0x846CA68B) & 0xFFFFFFFF
    x ^= x >> 16
    return x


def test_scene_roundtrip(scene_main_bytes):
    sc = S.read(scene_main_bytes)
    assert S.write(sc) == scene_main_bytes
    assert sc.Np == 10728 and sc.NL == 3 and sc.NS == 5


def test_truncated_scene_rejected(scene_main_bytes):
    for cut in (10, 1000, len(scene_main_bytes) // 2, len(scene_main_bytes) - 3):
        with pytest.raises(ValueError):
            po.Scene(data=scene_main_bytes[:cut])


def test_bad_region_rejected(scene_main_bytes):
    sc = S.read(scene_main_bytes)
    sc.region = sc.region.copy()
    sc.region[5] = sc.NR + 3
    with pytest.raises(ValueError):
        po.Scene(data=S.write(sc))


def test_generated_room_loads_and_builds():
    sc = S.box_room(points=20000, seed=3)
    data = S.write(sc)
    o = po.Scene(data=data)
    assert o.Np == sc.Np and o.NL == 3 and o.NS == 5
    o.build()
    ed = o.state_array(0, 0).reshape(-1, 3)
    assert np.isfinite(ed).all() and (ed >= 0).all() and ed.max() > 0
    # light 0 is off in state 1: its direct light vanishes, the others stay
    ed1 = o.state_array(1, 0).reshape(-1, 3)
    assert ed1[:, 0].max() == 0 and np.array_equal(ed1[:, 1:], ed[:, 1:])
    # the box moves between states 1 and 2: occluder voxels listed for that pair
    assert len(o.event_list(1 * 5 + 2, 0)) > 0
    # light 0 comes on between 2 and 3: its voxel is listed
    assert len(o.event_list(2 * 5 + 3, 1)) == 1


def test_run_is_deterministic():
    sc = po.Scene(data=S.write(S.box_room(points=8000, seed=1)))
    run = po.Run(sc)
    m = M.by_name(M.timing_methods(), "v4-A2C suivi 1/4")
    seq = [0] * 12 + [1] * 12 + [2] * 12
    run.begin(m, 0, 5)
    for s in seq:
        run.frame(s)
    a = run.array(po.A_LC).copy()
    run.begin(m, 0, 5)
    for s in seq:
        run.frame(s)
    assert np.array_equal(a, run.array(po.A_LC))
    assert np.isfinite(a).all()


def test_street_scene_tables():
    """Format-3 writer: BVH covers every triangle once with nested bounds; every static cache
    point is found in the hash table under its own cell key (linear probing from mix64)."""
    sc = S.street_scene(points=6000, buildings=4, size=40.0)
    m = sc.mesh
    BN = m["BN"]
    lf = BN[:, 3].view(np.int32)
    cnt = BN[:, 7].view(np.int32)
    seen = np.zeros(len(m["ST"]), int)
    stack = [0]
    while stack:
        k = stack.pop()
        if cnt[k] > 0:
            seen[lf[k]: lf[k] + cnt[k]] += 1
        else:
            for ch in (lf[k], lf[k] + 1):
                assert (BN[ch, 0:3] >= BN[k, 0:3]).all() and (BN[ch, 4:7] <= BN[k, 4:7]).all()
                stack.append(ch)
    assert (seen == 1).all()
    HK, HV = m["HK"], m["HV"]
    mask = len(HK) - 1
    npst = m["npst"]
    lo = m["lo"]
    h = np.float32(m["hcell"])
    P = sc.states[0].P[:npst]
    N = sc.states[0].N[:npst]
    c = np.floor((P - lo) * (np.float32(1) / h)).astype(np.int64)
    keys = S._cell_key(c[:, 0], c[:, 1], c[:, 2], S._normal_bucket(N))
    h0 = (S._mix64(keys) & np.uint64(0xFFFFFFFF)).astype(np.int64) & mask
    for i in range(0, npst, 7):
        j = int(h0[i])
        for _ in range(64):
            if HK[j] == keys[i] or HK[j] == 0:
                break
            j = (j + 1) & mask
        assert HK[j] == keys[i] and HV[j] == i


def test_street_scene_runs_in_oracle():
    data = S.write(S.street_scene(points=5000, buildings=4, size=40.0))
    o = po.Scene(data=data)
    assert o.fmt == 3 and o.nst > 0
    run = po.Run(o)
    m = M.by_name(M.timing_methods(), "v4-A2C suivi 1/4")
    run.begin(m, 0, 1)
    for s in [0] * 4 + [1] * 4 + [2] * 4 + [3] * 4:
        run.frame(s)
    lc = run.array(po.A_LC)
    assert np.isfinite(lc).all() and lc.max() > 0
    recs = run.probe(0, list(range(0, o.Np, 11)))
    assert any(r[2] <= -2 for r in recs)   # static (BVH) hits resolved through the hash table


def test_walk_restatement_breaks_edge_ties_like_the_reference():
    """A walk starting exactly on a voxel edge (x = 5, z = 2.25 -> grid z 3.0 with sz = 4/3)
    going -x and -z: both crossing distances are 0 and the reference's if / else-if chain steps
    z first (voxel 101 -> 69), which needs the grid coordinate rounded before the voxel index
    is subtracted from it."""
    v = po.dda_voxels((5.0, 0.001, 2.25), (3.5884497, 3.9999998, 1.8764427))
    assert v[:2] == [101, 69]
    assert po.dda_voxels((1.0, 0.5, 0.375), (1.0, 0.5, 0.375)) == [1]   # a point: its own voxel
