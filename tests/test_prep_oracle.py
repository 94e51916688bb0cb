"""The CPU restatement of the preparation's tree builder and lookup table (oracle/prep_oracle.py)
on its own: a valid tree in the format-3 layout, a bounded SAH cost, and a table whose keys
linear probing finds within 64 steps."""
import numpy as np

from oracle import prep_oracle as PO
from render_engine_gb300 import scene as S


def _check_tree(BN, nt):
    lf = BN[:, 3].view(np.int32)
    cnt = BN[:, 7].view(np.int32)
    cover = np.zeros(nt, np.int64)
    seen = np.zeros(len(BN), np.int64)
    seen[0] = 1
    stack = [0]
    while stack:
        k = stack.pop()
        if cnt[k] > 0:
            cover[lf[k]:lf[k] + cnt[k]] += 1
            continue
        for c in (lf[k], lf[k] + 1):
            assert (BN[c, 0:3] >= BN[k, 0:3]).all() and (BN[c, 4:7] <= BN[k, 4:7]).all()
            seen[c] += 1
            stack.append(c)
    assert (cover == 1).all()          # every triangle in exactly one leaf
    assert (seen == 1).all()           # every node reached once: a tree, children adjacent
    assert cnt.max() <= PO.MAX_LEAF


def test_lbvh_is_a_valid_tree_in_the_format_layout():
    V, _, _ = S.street_mesh(buildings=4, seed=1, facade_cell=3.0, size=40.0)
    BN, order = PO.lbvh(V)
    assert sorted(order.tolist()) == list(range(len(V)))
    _check_tree(BN, len(V))
    # the root box holds every triangle
    assert (BN[0, 0:3] <= V.reshape(-1, 3).min(0)).all() and (BN[0, 4:7] >= V.reshape(-1, 3).max(0)).all()


def test_lbvh_small_and_degenerate_inputs():
    rng = np.random.default_rng(0)
    for n in (1, 2, 3, 5, 17):
        V = rng.uniform(-1, 1, (n, 3, 3)).astype(np.float32)
        BN, _ = PO.lbvh(V)
        _check_tree(BN, n)
    V = np.repeat(rng.uniform(-1, 1, (1, 3, 3)).astype(np.float32), 40, axis=0)   # every centroid the same
    BN, _ = PO.lbvh(V)
    _check_tree(BN, 40)


def test_lbvh_sah_against_binned_sah():
    V, _, _ = S.street_mesh(buildings=6, seed=2, facade_cell=2.0, size=60.0)
    BN, _ = PO.lbvh(V)
    ours, yard = PO.sah_cost(BN), PO.binned_sah_cost(V)
    assert yard <= ours <= 1.45 * yard, (ours, yard)


def test_canonical_table_lookups():
    rng = np.random.default_rng(3)
    keys = np.unique(rng.integers(1, 1 << 62, 3000, dtype=np.int64)).astype(np.uint64)
    hs = 8192
    HK, HV = PO.canonical_table(keys, hs)
    home = (PO.mix64(keys) & np.uint64(hs - 1)).astype(np.int64)
    for i, k in enumerate(keys):
        s = int(home[i])
        for step in range(64):
            if HK[s] == k:
                break
            assert HK[s] != 0
            s = (s + 1) % hs
        assert HK[s] == k and HV[s] == i
