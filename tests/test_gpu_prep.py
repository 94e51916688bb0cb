"""The `prep` mode (rc_prep_mesh, poc_gpu_l3 prep) on the GPU: a generated street mesh becomes a
format-3 scene with references that the frame loop, the reference's own kernels and an
independent brute-force trace all accept."""
import json
import os
import subprocess

import numpy as np
import pytest

from oracle import pyref
from render_engine_gb300 import build
from render_engine_gb300 import methods as M
from render_engine_gb300 import native as N
from render_engine_gb300 import scene as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def prepared(tmp_path_factory):
    d = tmp_path_factory.mktemp("prep")
    V, alb, ds = S.street_mesh(buildings=6, seed=2, facade_cell=2.0, size=60.0)
    mesh = d / "street.msh"
    mesh.write_bytes(S.write_msh1(V, alb, ds))
    scene = d / "street.bin"
    exe = os.path.join(os.path.dirname(build.build()), "poc_gpu_l3")
    env = dict(os.environ, PREP_ITER_MAX="256")
    r = subprocess.run([exe, "prep", str(mesh), str(scene), "20000"], capture_output=True, text=True, timeout=900, env=env)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    return line, scene.read_bytes(), len(V)


def test_prep_line_and_scene(prepared):
    line, data, nt = prepared
    assert line["type"] == "prep" and line["triangles"] == nt
    assert len(line["bruit_ref"]) == 5 and len(line["iterations_ref"]) == 5 and len(line["lampes"]) == 3
    assert all(n <= 0.03 or it >= 256 for n, it in zip(line["bruit_ref"], line["iterations_ref"]))
    sc = S.read(data)
    assert sc.fmt == 3 and len(sc.L) == 3 and len(sc.states) == 5 and line["np"] == len(sc.A)
    assert abs(sc.mesh["npst"] - 20000) / 20000 < 0.1
    assert 0.2 < line["points_valides"] <= 1.0
    assert all(st.ref is not None for st in sc.states)
    # intensities normalised: mean direct light 1 in state 0 over all lights and points
    ctx = N.Context()
    ctx.load_bytes(data)
    ed = ctx.state_array(0, N.SA_EDIR)
    assert ed.sum() / len(sc.A) == pytest.approx(1.0, rel=1e-3)
    ctx.close()


def _hash32(x):
    x &= 0xFFFFFFFF
    x ^= x >> 16; x = (x * 0x7FEB352D) & 0xFFFFFFFF
    x ^= x >> 15; x = (x * 0x846CA68B) & 0xFFFFFFFF
    return x ^ (x >> 16)


def _rnd(s):
    s = (s * 747796405 + 2891336453) & 0xFFFFFFFF
    w = (((s >> ((s >> 28) + 4)) ^ s) * 277803737) & 0xFFFFFFFF
    w = (w >> 22) ^ w
    return s, np.float32(w >> 8) * np.float32(1.0 / 16777216.0)


def _first_ray(seed, frame, i, N):
    """Direction of the first ray of point i in a fixed-budget frame of one ray (poc_gpu.cu:442-462)."""
    s = _hash32((seed * 0x9E3779B9) ^ _hash32((frame * 0x85EBCA6B) ^ _hash32(i + 1)))
    s, _ = _rnd(s)            # the budget's Bernoulli draw
    s, u1 = _rnd(s)
    s, u2 = _rnd(s)
    n = N.astype(np.float64)
    r, ph = np.sqrt(u1), 6.28318530718 * u2
    a = np.array([0.0, 1.0, 0.0]) if abs(n[0]) > 0.9 else np.array([1.0, 0.0, 0.0])
    t = np.cross(n, a)
    t /= np.linalg.norm(t)
    b = np.cross(n, t)
    return t * r * np.cos(ph) + b * r * np.sin(ph) + n * np.sqrt(max(0.0, 1 - u1))


def _closest(O, D, tri):
    v0, e1, e2 = tri[:, 0:3], tri[:, 3:6], tri[:, 6:9]
    p = np.cross(D, e2)
    det = np.einsum("ij,ij->i", e1, p)
    ok = np.abs(det) > 1e-12
    inv = np.where(ok, 1.0 / np.where(ok, det, 1.0), 0.0)
    tv = O - v0
    u = np.einsum("ij,ij->i", tv, p) * inv
    q = np.cross(tv, e1)
    v = np.einsum("j,ij->i", D, q) * inv
    t = np.einsum("ij,ij->i", e2, q) * inv
    hit = ok & (u >= 0) & (u <= 1) & (v >= 0) & (u + v <= 1) & (t > 1e-4)
    if not hit.any():
        return -1, np.inf
    j = int(np.argmin(np.where(hit, t, np.inf)))
    return j, float(t[j])


def test_prepared_bvh_finds_the_closest_triangle(prepared):
    """The GPU's hits through the prepared BVH against an FP64 brute force over every static and
    dynamic triangle, for the first ray of 400 points (directions recomputed in FP64: rays that
    graze an edge may differ)."""
    _, data, _ = prepared
    sc = S.read(data)
    st0 = sc.states[0]
    ST = sc.mesh["ST"].astype(np.float64)
    T = st0.T.astype(np.float64)
    nst = len(ST)
    ctx = N.Context()
    ctx.load_bytes(data)
    ctx.begin(M.Method(name="one ray", mode=0, nmax=64.0, budget=1.0), 0, 5)
    pts = np.arange(0, len(sc.A), max(1, len(sc.A) // 400), dtype=np.int32)
    recs = [r for r in ctx.probe(0, pts) if r[1] == 0]
    ctx.close()
    same = 0
    for point, _, q, _, _, t in recs:
        O = st0.P[point].astype(np.float32) + st0.N[point].astype(np.float32) * np.float32(1e-3)
        D = _first_ray(5, 0, int(point), st0.N[point])
        j, tb = _closest(O.astype(np.float64), D, np.concatenate([ST, T]))
        want = -1 if j < 0 else (-2 - j if j < nst else int(st0.TQ[j - nst]))
        if want == q and (q == -1 or abs(tb - t) <= 1e-4 * max(1.0, tb)):
            same += 1
    assert len(recs) >= 300 and same / len(recs) > 0.99, (same, len(recs))


def test_prepared_scene_runs_the_reference_kernels_bitexact(prepared):
    if not pyref.available(3):
        pytest.skip("reference kernels not built")
    from test_gpu_parity import _frames_vs_reference
    _, data, _ = prepared
    m = M.by_name(M.timing_methods(), "v4-A2C suivi 1/4")
    seq = [0] * 12 + [1] * 8 + [2] * 8 + [3] * 6
    _frames_vs_reference(data, 3, m, seq, 17)
