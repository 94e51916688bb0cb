"""GPU parity of the hash-grid cache with dependency masks (include/rc_hashgrid.h) against its
CPU oracle (oracle/hg_oracle.c), bit for bit:

* dependency marking of random path batches, both banks, inheritance from cached answers;
* resolve: invalidation by event masks, accumulation into fp16, sample cap, eviction;
* insert (per key: the GPU may place colliding keys in other slots) and accumulate;
* snapshots (records in entry order) and restore;
* a multi-frame run with bank rotation and an event, compared per key every frame.

Vertices answered from the cache (STOP) use entries no other path touches, so their
inherited masks do not depend on the order in which paths run."""
import numpy as np
import pytest
import torch

from oracle import pyhg
from render_engine_gb300 import hashgrid as H

pytestmark = pytest.mark.gpu


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _paths(rng, npaths, cap, stop_base, max_len=5, p_miss=0.15, p_stop=0.1):
    lens = rng.integers(1, max_len + 1, npaths)
    start = np.zeros(npaths + 1, np.int32)
    start[1:] = np.cumsum(lens)
    n = int(start[-1])
    v = np.zeros(n, H.VERTEX_DTYPE)
    lo, hi = np.array([-1.0, -1.0, -1.0]), np.array([9.0, 5.0, 4.0])
    v["origin"] = rng.uniform(lo, hi, (n, 3))
    v["hit"] = rng.uniform(lo, hi, (n, 3))
    d = rng.normal(size=(n, 3))
    v["dir"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    t = rng.normal(size=(n, 3))
    v["to_light"] = t / np.linalg.norm(t, axis=1, keepdims=True)
    v["light_dist"] = rng.uniform(0.05, 30.0, n)
    v["light_index"] = rng.integers(-1, 40, n)
    v["entry"] = rng.integers(0, stop_base, n)
    v["entry"][rng.random(n) < 0.05] = H.INVALID
    flags = np.where(rng.random(n) < 0.5, H.LIGHT_VISIBLE, 0)
    flags |= np.where(rng.random(n) < p_miss, H.MISS, 0)
    stop = rng.random(n) < p_stop
    flags |= np.where(stop, H.STOP, 0)
    v["flags"] = flags
    # cached answers: an entry of their own (no other vertex uses it)
    ns = int(stop.sum())
    assert stop_base + ns <= cap
    v["entry"][stop] = stop_base + np.arange(ns)
    return v, start


def _rand_banks(rng, cap, p=0.3):
    b = rng.integers(0, 2 ** 32, (cap, 4), dtype=np.uint64).astype(np.uint32)
    b &= rng.integers(0, 2 ** 32, (cap, 4), dtype=np.uint64).astype(np.uint32)
    b[rng.random(cap) > p] = 0
    return b


@pytest.mark.parametrize("bank", [0, 1])
def test_mark_paths_bitexact(bank):
    rng = np.random.default_rng(10 + bank)
    cap = 1 << 16
    cfg = H.make_config(capacity=cap, max_depth=4, tracing_distance=50.0)
    hg = H.HashGrid(cfg)
    orc = pyhg.Cache(pyhg.config_from(cfg))
    if bank:
        hg.begin_frame(16, 16)
        orc.begin_frame(16, 16)
    b0, b1 = _rand_banks(rng, cap), _rand_banks(rng, cap)
    hg.upload(H.A_BANK0, b0)
    hg.upload(H.A_BANK1, b1)
    orc.bank0[:], orc.bank1[:] = b0, b1
    v, start = _paths(rng, 30000, cap, stop_base=cap // 2)
    dv, ds = _dev(v.view(np.uint8)), _dev(start)
    hg.mark_paths(dv, ds, len(start) - 1)
    orc.mark_paths(v, start)
    assert np.array_equal(hg.download(H.A_BANK0), orc.bank0)
    assert np.array_equal(hg.download(H.A_BANK1), orc.bank1)
    assert orc.bank0.any() and orc.bank1.any()


def _rand_state(rng, cap, stale_frames):
    keys = rng.integers(1, 2 ** 63, cap, dtype=np.uint64)
    keys[rng.random(cap) < 0.4] = 0
    accum = np.zeros((cap, 4), np.uint32)
    has = rng.random(cap) < 0.5
    cnt = rng.integers(1, 6, cap)
    accum[has, 3] = cnt[has]
    accum[has, :3] = (rng.uniform(0, 50, (int(has.sum()), 3)) * 1024 * cnt[has, None]).astype(np.uint32)
    res = np.zeros((cap, 4), np.uint32)
    n0 = rng.integers(0, 40, cap).astype(np.uint32)
    rgb = rng.uniform(0, 100, (cap, 3)).astype(np.float16).view(np.uint16).astype(np.uint32)
    res[:, 0] = rgb[:, 0] | rgb[:, 1] << 16
    res[:, 1] = rgb[:, 2] | n0.astype(np.float16).view(np.uint16).astype(np.uint32) << 16
    res[:, 2] = n0 | rng.integers(0, stale_frames + 2, cap).astype(np.uint32) << 16
    empty = keys == 0            # an empty slot holds no data (the cache keeps it so)
    accum[empty] = 0
    res[empty] = 0
    return keys, accum, res


@pytest.mark.parametrize("inv", [None, (1 << 3, 0, 1 << 7, 0), (0, 0, 0, 1 << 5), (0, 0, 0, H.SKY_BIT)])
def test_resolve_bitexact(inv):
    rng = np.random.default_rng(20)
    cap = 1 << 16
    cfg = H.make_config(capacity=cap, acc_frames=32, stale_frames=3)
    hg = H.HashGrid(cfg)
    orc = pyhg.Cache(pyhg.config_from(cfg))
    keys, accum, res = _rand_state(rng, cap, 3)
    b0, b1 = _rand_banks(rng, cap, 0.5), _rand_banks(rng, cap, 0.5)
    b0[keys == 0] = 0
    b1[keys == 0] = 0
    for which, a in ((H.A_KEYS, keys), (H.A_ACCUM, accum), (H.A_RESOLVED, res), (H.A_BANK0, b0), (H.A_BANK1, b1)):
        hg.upload(which, a)
    orc.keys[:], orc.accum[:], orc.resolved[:], orc.bank0[:], orc.bank1[:] = keys, accum, res, b0, b1
    counts = torch.zeros(3, dtype=torch.int32, device="cuda")
    hg.resolve(inv, counts)
    want = orc.resolve(inv)
    assert np.array_equal(counts.cpu().numpy().astype(np.uint32), want)
    for which, a in ((H.A_KEYS, orc.keys), (H.A_ACCUM, orc.accum), (H.A_RESOLVED, orc.resolved), (H.A_BANK0, orc.bank0),
                     (H.A_BANK1, orc.bank1)):
        assert np.array_equal(hg.download(which), a), which
    if inv is not None:
        assert want[0] > 0
    assert want[1] > 0 and want[2] > 0


def _by_key(keys, *arrays):
    out = {}
    for e in np.flatnonzero((keys != 0) & (keys != H.EVICTED)):
        assert int(keys[e]) not in out        # one entry per key
        out[int(keys[e])] = tuple(tuple(a[e].tolist()) for a in arrays)
    return out


def test_insert_and_accumulate_per_key():
    rng = np.random.default_rng(30)
    cap = 1 << 15
    cfg = H.make_config(capacity=cap, cell=0.5)
    hg = H.HashGrid(cfg)
    orc = pyhg.Cache(pyhg.config_from(cfg))
    n = 20000
    pos = (rng.integers(0, 24, (n, 3)) * np.array([0.34, 0.17, 0.13]) + rng.uniform(0, 0.02, (n, 3))).astype(np.float32)
    nrm = rng.normal(size=(n, 3)).astype(np.float32)
    entry = torch.zeros(n, dtype=torch.int32, device="cuda")
    hg.insert(_dev(pos), _dev(nrm), entry)
    e_gpu = entry.cpu().numpy().view(np.uint32)
    e_orc = orc.insert(pos, nrm)
    keys = hg.download(H.A_KEYS)
    assert (e_gpu != H.INVALID).all()
    assert np.array_equal(keys[e_gpu], orc.keys[e_orc])            # every point found its own key
    live = lambda k: set(k[(k != 0) & (k != H.EVICTED)].tolist())
    assert live(keys) == live(orc.keys)
    rgb = rng.uniform(0, 3, (n, 3)).astype(np.float32)
    hg.accumulate(entry, _dev(rgb))
    orc.accumulate(e_orc, rgb)
    acc = hg.download(H.A_ACCUM)
    assert _by_key(keys, acc) == _by_key(orc.keys, orc.accum)


def test_snapshot_and_restore_bitexact():
    rng = np.random.default_rng(40)
    cap = 1 << 16
    cfg = H.make_config(capacity=cap, acc_frames=32, stale_frames=3)
    hg = H.HashGrid(cfg)
    orc = pyhg.Cache(pyhg.config_from(cfg))
    keys, accum, res = _rand_state(rng, cap, 3)
    for which, a in ((H.A_KEYS, keys), (H.A_ACCUM, accum), (H.A_RESOLVED, res)):
        hg.upload(which, a)
    orc.keys[:], orc.accum[:], orc.resolved[:] = keys, accum, res
    hg.resolve()
    orc.resolve()
    recs = torch.zeros(cap * H.SNAP_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    n = hg.snapshot(recs, cap)
    want = orc.snapshot(H.SNAP_DTYPE)
    assert n == len(want) > 0
    got = recs.cpu().numpy()[: n * H.SNAP_DTYPE.itemsize].view(H.SNAP_DTYPE)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    # a short buffer receives the first records, the count is still the total
    short = torch.zeros(100 * H.SNAP_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    assert hg.snapshot(short, 100) == n
    assert np.array_equal(short.cpu().numpy().view(H.SNAP_DTYPE).view(np.uint32), want[:100].view(np.uint32))
    k_before, r_before = hg.download(H.A_KEYS), hg.download(H.A_RESOLVED)
    hg.clear()
    hg.restore(recs, n)
    orc.keys[:] = 0
    orc.resolved[:] = 0
    orc.restore(want)
    assert np.array_equal(hg.download(H.A_KEYS), orc.keys)
    assert np.array_equal(hg.download(H.A_RESOLVED), orc.resolved)
    valid = (k_before != 0) & ((r_before[:, 1] >> 16) != 0)
    assert np.array_equal(orc.keys[valid], k_before[valid])


def test_frames_with_rotation_and_event_per_key():
    rng = np.random.default_rng(50)
    cap = 1 << 16
    cfg = H.make_config(capacity=cap, cell=0.25, max_depth=3, acc_frames=16, stale_frames=4, tracing_distance=40.0)
    hg = H.HashGrid(cfg)
    orc = pyhg.Cache(pyhg.config_from(cfg))
    npts = 6000
    pos = rng.uniform([0, 0, 0], [8, 4, 3], (npts, 3)).astype(np.float32)
    nrm = rng.normal(size=(npts, 3)).astype(np.float32)
    counts = torch.zeros(3, dtype=torch.int32, device="cuda")
    for f in range(24):
        hg.begin_frame(f, 4)
        orc.begin_frame(f, 4)
        pick = rng.choice(npts, 3000, replace=False)
        entry = torch.zeros(len(pick), dtype=torch.int32, device="cuda")
        hg.insert(_dev(pos[pick]), _dev(nrm[pick]), entry)
        e_orc = orc.insert(pos[pick], nrm[pick])
        rgb = rng.uniform(0, 2, (len(pick), 3)).astype(np.float32)
        hg.accumulate(entry, _dev(rgb))
        orc.accumulate(e_orc, rgb)
        # paths through the picked points (no cached answers: entries are shared between paths)
        e_gpu = entry.cpu().numpy().view(np.uint32)
        v, start = _paths(rng, 1000, cap, stop_base=1, p_stop=0.0)
        sel = rng.integers(0, len(pick), len(v))
        v["hit"] = pos[pick][sel]
        v_gpu = v.copy()
        v_gpu["entry"] = e_gpu[sel]
        v["entry"] = e_orc[sel]
        hg.mark_paths(_dev(v_gpu.view(np.uint8)), _dev(start), len(start) - 1)
        orc.mark_paths(v, start)
        inv = H.event_mask(cfg, [1, 1, 1], [1, 0.5, 1], 0, 0, [2, 1, 1, 1, 1, 1], [5, 2, 1, 1, 1, 1]) if f == 15 else None
        hg.resolve(inv, counts)
        want = orc.resolve(inv)
        assert np.array_equal(counts.cpu().numpy().astype(np.uint32), want), f
        keys = hg.download(H.A_KEYS)
        got = _by_key(keys, hg.download(H.A_ACCUM), hg.download(H.A_RESOLVED), hg.download(H.A_BANK0), hg.download(H.A_BANK1))
        assert got == _by_key(orc.keys, orc.accum, orc.resolved, orc.bank0, orc.bank1), f
