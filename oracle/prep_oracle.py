"""CPU restatement of the scene preparation's tree builder and lookup table (rc_prep.cu) --
TEST INFRASTRUCTURE ONLY: the GPU-built scene is compared with it bit for bit.

* ``lbvh(V)``: the linear BVH over 63-bit Morton codes of the triangle centroids (Karras, HPG
  2012: radix tree over the sorted codes, equal codes ordered by index), boxes and SAH costs
  fitted bottom-up with every float operation rounded on its own, subtrees of at most four
  triangles collapsed where the leaf's SAH cost is not above the split's, laid out with the
  children of a node adjacent.  Returns the node array in the format-3 layout and the
  triangle order.
* ``sah_cost(BN)``: the SAH cost of a node array (inner node 1, triangle 1, relative to the
  root's area).
* ``binned_sah_cost(V)``: the cost of a greedy top-down binned-SAH tree (16 bins on each axis,
  leaves of at most four triangles): the yardstick the GPU tree is held to.
* ``canonical_table(keys, hs)``: the linear-probing table placed in home-slot order.

There is no reference counterpart for these (the reference builds its tree on the host with a
binned SAH, cuda/prep_mesh.cuh:42-114): parity of the preparation with the reference is by
what the frames do on the prepared scene, not by its bytes.
"""
from __future__ import annotations

import numpy as np

F = np.float32
MAX_LEAF = 4


def _spread3(x: np.ndarray) -> np.ndarray:
    x = x.astype(np.uint64) & np.uint64(0x1FFFFF)
    x = (x | (x << np.uint64(32))) & np.uint64(0x1F00000000FFFF)
    x = (x | (x << np.uint64(16))) & np.uint64(0x1F0000FF0000FF)
    x = (x | (x << np.uint64(8))) & np.uint64(0x100F00F00F00F00F)
    x = (x | (x << np.uint64(4))) & np.uint64(0x10C30C30C30C30C3)
    x = (x | (x << np.uint64(2))) & np.uint64(0x1249249249249249)
    return x


def morton_codes(V: np.ndarray) -> np.ndarray:
    V = np.asarray(V, F).reshape(-1, 3, 3)
    lo, hi = V.min(axis=1), V.max(axis=1)
    c = (F(0.5) * (lo + hi)).astype(F)
    clo, chi = c.min(axis=0), c.max(axis=0)
    e = (chi - clo).astype(F)
    with np.errstate(divide="ignore", invalid="ignore"):
        u = np.where(e > 0, ((c - clo) / np.where(e > 0, e, F(1))).astype(F), F(0)).astype(F)
    q = np.clip((u * F(2097152.0)).astype(F), F(0), F(2097151.0)).astype(np.uint64)
    return _spread3(q[:, 0]) | (_spread3(q[:, 1]) << np.uint64(1)) | (_spread3(q[:, 2]) << np.uint64(2))


def _lcp(c, n, i, j):
    if j < 0 or j >= n:
        return -1
    x = int(c[i]) ^ int(c[j])
    if x:
        return 64 - x.bit_length()
    return 64 + (32 - (i ^ j).bit_length())


def _area(lo, hi):
    d = [max(F(hi[k] - lo[k]), F(0)) for k in range(3)]
    return F(F(2) * F(F(F(d[0] * d[1]) + F(d[1] * d[2])) + F(d[2] * d[0])))


def lbvh(V: np.ndarray):
    """(nodes (K, 8) float32 in the format-3 layout, triangle order) of the preparation's tree."""
    V = np.asarray(V, F).reshape(-1, 3, 3)
    n = len(V)
    tlo, thi = V.min(axis=1), V.max(axis=1)
    code = morton_codes(V)
    order = np.argsort(code, kind="stable")
    sc = code[order]
    if n == 1:
        out = np.zeros((1, 8), F)
        out[0, 0:3], out[0, 4:7] = tlo[0], thi[0]
        out[0, 7] = np.array([1], np.int32).view(F)[0]
        return out, order
    child = np.zeros((n - 1, 2), np.int64)
    first = np.zeros(n - 1, np.int64)
    for i in range(n - 1):
        d = 1 if _lcp(sc, n, i, i + 1) - _lcp(sc, n, i, i - 1) > 0 else -1
        dmin = _lcp(sc, n, i, i - d)
        lmax = 2
        while _lcp(sc, n, i, i + lmax * d) > dmin:
            lmax *= 2
        l, t = 0, lmax // 2
        while t >= 1:
            if _lcp(sc, n, i, i + (l + t) * d) > dmin:
                l += t
            t //= 2
        j = i + l * d
        dnode = _lcp(sc, n, i, j)
        s, div = 0, 2
        while True:
            t = (l + div - 1) // div
            if _lcp(sc, n, i, i + (s + t) * d) > dnode:
                s += t
            if t <= 1:
                break
            div *= 2
        g = i + s * d + min(d, 0)
        lo_, hi_ = min(i, j), max(i, j)
        child[i] = (n - 1 + g if lo_ == g else g, n - 1 + g + 1 if hi_ == g + 1 else g + 1)
        first[i] = lo_
    box_lo = np.zeros((2 * n - 1, 3), F)
    box_hi = np.zeros((2 * n - 1, 3), F)
    cost = np.zeros(2 * n - 1, F)
    count = np.zeros(2 * n - 1, np.int64)
    desc = np.zeros(2 * n - 1, np.int64)
    coll = np.zeros(2 * n - 1, bool)
    box_lo[n - 1:] = tlo[order]
    box_hi[n - 1:] = thi[order]
    count[n - 1:] = 1
    for k in range(n - 1, 2 * n - 1):
        cost[k] = _area(box_lo[k], box_hi[k])
    # post order: children before parents
    post, stack = [], [(0, False)]
    while stack:
        x, done = stack.pop()
        if x >= n - 1:
            continue
        if done:
            post.append(x)
            continue
        stack.append((x, True))
        stack.append((int(child[x, 1]), False))
        stack.append((int(child[x, 0]), False))
    for x in post:
        a, b = int(child[x, 0]), int(child[x, 1])
        box_lo[x] = np.minimum(box_lo[a], box_lo[b])
        box_hi[x] = np.maximum(box_hi[a], box_hi[b])
        A = _area(box_lo[x], box_hi[x])
        count[x] = count[a] + count[b]
        split = F(F(F(F(1) * A) + cost[a]) + cost[b])
        leaf = F(F(count[x]) * A)
        coll[x] = count[x] <= MAX_LEAF and leaf <= split
        cost[x] = leaf if coll[x] else split
        desc[x] = 0 if coll[x] else 2 + desc[a] + desc[b]
    out = np.zeros((1 + desc[0], 8), F)
    as_f = lambda v: np.array([v], np.int32).view(F)[0]
    stack = [(0, 0, 1)]   # node, position, children block start
    while stack:
        x, pos, cb = stack.pop()
        leaf = x >= n - 1 or coll[x]
        out[pos, 0:3], out[pos, 4:7] = box_lo[x], box_hi[x]
        if leaf:
            out[pos, 3] = as_f(x - (n - 1) if x >= n - 1 else first[x])
            out[pos, 7] = as_f(count[x])
        else:
            out[pos, 3] = as_f(cb)
            out[pos, 7] = as_f(0)
            a, b = int(child[x, 0]), int(child[x, 1])
            stack.append((a, cb, cb + 2))
            stack.append((b, cb + 1, cb + 2 + desc[a]))
    return out, order


def sah_cost(BN: np.ndarray) -> float:
    """SAH cost of a format-3 node array: 1 per inner node visit and 1 per triangle test,
    weighted by area relative to the root's."""
    BN = np.asarray(BN, F).reshape(-1, 8)
    cnt = BN[:, 7].view(np.int32)
    d = np.maximum(BN[:, 4:7].astype(np.float64) - BN[:, 0:3], 0)
    A = 2 * (d[:, 0] * d[:, 1] + d[:, 1] * d[:, 2] + d[:, 2] * d[:, 0])
    return float((np.where(cnt > 0, cnt, 1) * A).sum() / A[0])


def binned_sah_cost(V: np.ndarray, bins: int = 16, leaf: int = MAX_LEAF) -> float:
    """Cost (as sah_cost counts it) of a greedy top-down binned-SAH tree over V: at every node
    the best of 16 bins on each axis, a leaf when it holds at most `leaf` triangles and its
    cost is not above the split's."""
    V = np.asarray(V, np.float64).reshape(-1, 3, 3)
    lo, hi = V.min(axis=1), V.max(axis=1)
    cen = 0.5 * (lo + hi)

    def area(l, h):
        d = np.maximum(h - l, 0)
        return 2 * (d[..., 0] * d[..., 1] + d[..., 1] * d[..., 2] + d[..., 2] * d[..., 0])

    root = area(lo.min(0), hi.max(0))
    total = 0.0
    stack = [np.arange(len(V))]
    while stack:
        idx = stack.pop()
        l, h = lo[idx].min(0), hi[idx].max(0)
        A = area(l, h)
        n = len(idx)
        best, choice = np.inf, None
        c = cen[idx]
        cl, ch = c.min(0), c.max(0)
        for ax in range(3):
            if ch[ax] - cl[ax] <= 0:
                continue
            b = np.minimum(((c[:, ax] - cl[ax]) / (ch[ax] - cl[ax]) * bins).astype(int), bins - 1)
            cnt = np.bincount(b, minlength=bins)
            blo = np.full((bins, 3), np.inf)
            bhi = np.full((bins, 3), -np.inf)
            np.minimum.at(blo, b, lo[idx])
            np.maximum.at(bhi, b, hi[idx])
            llo = np.minimum.accumulate(blo, 0)
            lhi = np.maximum.accumulate(bhi, 0)
            rlo = np.minimum.accumulate(blo[::-1], 0)[::-1]
            rhi = np.maximum.accumulate(bhi[::-1], 0)[::-1]
            nl = np.cumsum(cnt)
            for s in range(1, bins):
                L, R = nl[s - 1], n - nl[s - 1]
                if L == 0 or R == 0:
                    continue
                cost = L * area(llo[s - 1], lhi[s - 1]) + R * area(rlo[s], rhi[s])
                if cost < best:
                    best, choice = cost, (ax, b < s)
        if n <= leaf and (choice is None or n * A <= A + best):
            total += n * A
            continue
        if choice is None:   # coincident centroids: split in half
            half = n // 2
            left = np.zeros(n, bool)
            left[:half] = True
        else:
            left = choice[1]
        total += A
        stack.append(idx[left])
        stack.append(idx[~left])
    return float(total / root)


def mix64(x: np.ndarray) -> np.ndarray:
    x = np.asarray(x, np.uint64)
    with np.errstate(over="ignore"):
        x = x ^ (x >> np.uint64(30))
        x = x * np.uint64(0xBF58476D1CE4E5B9)
        x = x ^ (x >> np.uint64(27))
        x = x * np.uint64(0x94D049BB133111EB)
        x = x ^ (x >> np.uint64(31))
    return x


def canonical_table(keys: np.ndarray, hs: int):
    """(HK, HV) of the linear-probing table with the keys placed in the order of their home slot
    mix64(key) & (hs - 1), ties by point index: the table the preparation writes."""
    keys = np.asarray(keys, np.uint64)
    home = (mix64(keys) & np.uint64(hs - 1)).astype(np.int64)
    order = np.lexsort((np.arange(len(keys)), home))
    HK = np.zeros(hs, np.uint64)
    HV = np.full(hs, -1, np.int32)
    last = -1
    for i in order:
        s = max(int(home[i]), last + 1)
        if s >= hs:
            s = int(home[i])
            while HK[s % hs] != 0:
                s += 1
            s %= hs
        else:
            last = s
        HK[s] = keys[i]
        HV[s] = i
    return HK, HV
