"""Edge cases of the frame loop on the GPU against the CPU oracle: every compiled light count,
point counts that fill no block or tile evenly, and the 768-voxel transit grid (NW = 24).
The reference's kernels exist for 3 and 8 lights and the 8 x 4 x 4 grid only (its compile-time
constants), so these are checked against the CPU restatement: the same rays except at ulp
ties of the C library's cosf / sinf, hence the per-point agreement thresholds."""
import numpy as np
import pytest

from oracle import pyoracle as po
from render_engine_gb300 import methods as M
from render_engine_gb300 import native as N
from render_engine_gb300 import scene as S

pytestmark = pytest.mark.gpu

SEQ = [0] * 8 + [1] * 6 + [2] * 6 + [4] * 4


def _compare(data, method, grid=(8, 4, 4), frames=SEQ, mask_check=False):
    ctx = N.Context(grid=grid)
    info = ctx.load_bytes(data)
    orc = po.Run(po.Scene(data=data, grid=grid))
    m = M.by_name(M.timing_methods(), method)
    ctx.begin(m, frames[0], 7)
    orc.begin(m, frames[0], 7)
    for s in frames:
        ctx.frame(s)
        orc.frame(s)
    a, b = ctx.array(N.A_LC), orc.array(po.A_LC)
    close = np.isclose(a, b, rtol=1e-3, atol=1e-5 * max(1.0, float(np.abs(b).max())))
    assert np.isfinite(a).all() and close.mean() > 0.99, close.mean()
    assert abs(float(a.sum()) - float(b.sum())) <= 2e-3 * abs(float(b.sum())) + 1e-6
    if mask_check:
        cur, cur_o = ctx.array(N.A_CUR), orc.array(po.A_CUR)
        assert cur.size == info["nw"] * info["np"]
        # masks or together every ray of the run, so each ulp-level direction difference that
        # moves a voxel crossing stays; bit for bit they are checked against the reference's
        # kernels (tests/test_gpu_parity.py, also on the 16 x 8 x 6 grid)
        assert (cur == cur_o).mean() > 0.99
        diff_bits = sum(bin(int(x)).count("1") for x in (cur ^ cur_o)[cur != cur_o])
        set_bits = int(np.unpackbits(cur.view(np.uint8)).sum())
        assert diff_bits <= 0.005 * set_bits, (diff_bits, set_bits)
        assert cur.any()
    assert ctx.device_flags() == 0
    ctx.close()
    return info


@pytest.mark.parametrize("lights", [1, 2, 4, 32])
def test_light_counts(lights):
    data = S.write(S.box_room(points=6000, seed=4, lights=lights))
    info = _compare(data, "v4-A2C suivi 1/4")
    assert info["nl"] == lights


@pytest.mark.parametrize("points", [40, 300, 2500])
def test_ragged_point_counts(points):
    """The cache against the oracle; the masks of these scenes are compared with the
    reference's kernels instead (tests/test_gpu_parity.py): on coarse point grids many shadow
    samples fall exactly on voxel boundaries, where the reference's contracted a + (b - a) t
    (the GPU's, bit for bit) and the oracle's uncontracted one pick different voxels."""
    data = S.write(S.box_room(points=points, seed=5))
    info = _compare(data, "v3 complet")
    assert info["np"] % 256 != 0


def test_fine_transit_grid():
    data = S.write(S.box_room(points=8000, seed=6))
    info = _compare(data, "v3 complet", grid=(16, 8, 6))
    assert info["nw"] == 24
    _compare(data, "v3 complet", grid=(16, 8, 6), frames=[0] * 12, mask_check=True)


@pytest.mark.parametrize("points", [40, 300])
def test_dependency_masks_replay_probe_records(points):
    """Frame 0 of a method tracked every frame writes, per point, the OR of its rays' shadow-voxel
    masks (at the hit point, or the point's own for a ray that does not count) and of the walks
    O -> H.  Replayed on the CPU from the rc_probe_rays records (direction, end point) with the
    float restatement of the walk, it equals the GPU's mask bit for bit, on rooms whose cache
    points lie on voxel faces (ties at voxel edges included)."""
    data = S.write(S.box_room(points=points, seed=5))
    ctx = N.Context()
    info = ctx.load_bytes(data)
    Np, NW = info["np"], info["nw"]
    m = M.by_name(M.timing_methods(), "v3 complet")
    ctx.begin(m, 0, 13)
    recs = ctx.probe_full(0, list(range(Np)))
    ctx.frame(0)
    cur = ctx.array(N.A_CUR).reshape(NW, Np)
    sv = ctx.state_array(0, N.SA_SV).reshape(Np, NW)
    st = S.read(data).states[0]
    eps = np.float64(np.float32(1e-3))
    by_point = {}
    for r in recs:
        by_point.setdefault(r["point"], []).append(r)
    for i in range(Np):
        want = np.zeros(NW, np.uint32)
        rays = by_point.get(i, [])
        # O = P + N * 1e-3 as one fused multiply-add: exact product and sum in double, one rounding
        O = (st.P[i].astype(np.float64) + st.N[i].astype(np.float64) * eps).astype(np.float32)
        for r in rays:
            want |= sv[i if r["back"] else r["pi"]]
            for v in po.dda_voxels(O, r["hit"]):
                want[v >> 5] |= np.uint32(1 << (v & 31))
        np.testing.assert_array_equal(cur[:, i], want, err_msg="point %d, %d rays" % (i, len(rays)))
