"""The state build's voxel index of a shadow-segment sample (vox_axis in
render_engine_gb300/csrc/rc_device.cuh) against the reference's expression it replaces
(vox_of, poc_gpu.cu:137-142): int((x - lo) / ext * n) clamped to [0, n - 1], with an IEEE
division.  The fast path truncates qf = (x - lo) * s, s = n / ext rounded to float, and falls back
to the division when qf is within 1e-5 * max(1, |qf|) of an integer; both are restated here in
float32 arithmetic (IEEE, round to nearest, as the GPU's) and must give the same index on random
samples, on samples packed around every voxel boundary, and far outside the grid."""
import numpy as np
import pytest

F = np.float32


def ref_axis(x, lo, ext, n):
    d = (x - F(lo)).astype(F)
    q = ((d / F(ext)).astype(F) * F(n)).astype(F)
    with np.errstate(invalid="ignore"):
        v = np.trunc(q)
        v = np.where(np.isfinite(v), v, 0).astype(np.int64)
    return np.clip(v, 0, n - 1)


def fast_axis(x, lo, ext, n):
    d = (x - F(lo)).astype(F)
    s = F(F(n) / F(ext))
    qf = (d * s).astype(F)
    r = np.rint(qf).astype(F)
    with np.errstate(invalid="ignore"):   # inf - inf: the comparison is false, as on the GPU
        far = np.abs((qf - r).astype(F)) > F(1e-5) * np.maximum(F(1.0), np.abs(qf))
    with np.errstate(invalid="ignore"):
        v_fast = np.trunc(qf)
        v_fast = np.where(np.isfinite(v_fast), v_fast, 0).astype(np.int64)
    v = np.where(far, v_fast, ref_axis(x, lo, ext, n))
    return np.clip(v, 0, n - 1), far


@pytest.mark.parametrize("lo,ext,n", [(0.0, 8.0, 8), (0.0, 4.0, 4), (0.0, 3.0, 4), (-12.5, 37.0, 16), (3.25, 1.7, 128),
                                      (-100.0, 200.0, 256), (0.1, 0.3, 32)])
def test_fast_voxel_index_equals_the_division(lo, ext, n):
    rng = np.random.default_rng(abs(hash((lo, ext, n))) % 2**32)
    x = rng.uniform(lo - 0.2 * ext, lo + 1.2 * ext, 2_000_000).astype(F)
    # samples packed around every voxel boundary, a few ulps either side
    b = (F(lo) + (np.arange(n + 1, dtype=F) * F(ext) / F(n))).astype(F)
    near = b
    for _ in range(4):
        near = np.concatenate([near, np.nextafter(near, F(np.inf)).astype(F), np.nextafter(near, F(-np.inf)).astype(F)])
    far_out = np.array([lo - 1e6, lo + 1e6, lo - 1e-30, np.float32(np.inf), np.float32(-np.inf)], F)
    xs = np.concatenate([x, near, far_out]).astype(F)
    got, fast = fast_axis(xs, lo, ext, n)
    want = ref_axis(xs, lo, ext, n)
    assert np.array_equal(got, want)
    assert fast[: len(x)].mean() > 0.99          # the division is rarely needed
