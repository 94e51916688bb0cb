"""rc_adjoint on the GPU against the FP64 oracle.

* The frozen rays are the oracle's rays (the same FP32 trace as every frame) except at the
  rare near-ties where the CPU's cosf / sinf / 1/sqrtf and the GPU's differ by an ulp (fewer
  than 1 in 10^4 rays); the FP64 solve then uses the GPU's own rays.
* The gradient dJ/dE_l, the objective J, the forward solution L and the adjoint importance u
  match the FP64 solution of the same frozen transport (oracle/transport.py), whose adjoint is
  itself checked against central finite differences.
* Size-independent properties at 1.08 M points and 16 lights: J = sum_l E_l dJ/dE_l (linearity
  in the emissions), converged sweeps, bit-identical repeats.
* The GPU references (rc_reference_build) agree with the FP64 path tracer.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from oracle import transport as tr
from render_engine_gb300 import native as N
from render_engine_gb300 import scene as S

pytestmark = pytest.mark.gpu


def _weights(n, k, seed):
    rng = np.random.default_rng(seed)
    w = np.zeros(n, np.float32)
    w[rng.choice(n, k, replace=False)] = 1.0 / k
    return w


def _case(data, state, K, seed, nw=512, iters=96):
    sc = S.read(data)
    o = po.Scene(data=data)
    o.build()
    ctx = N.Context()
    ctx.load_bytes(data)
    w = _weights(o.Np, min(nw, o.Np), 3 + state)
    g, res = ctx.adjoint(state, w, K=K, seed=seed, iterations=iters)
    L, u, hits = ctx.adjoint_arrays()
    ctx.close()
    return sc, o, w, g, res, L, u, hits


@pytest.mark.parametrize("name,state", [("scene_main", 0), ("scene_main", 1), ("scene_stress", 4)])
def test_adjoint_matches_fp64(request, name, state):
    data = request.getfixturevalue(name + "_bytes")
    sc, o, w, g, res, L, u, hits = _case(data, state, K=16, seed=7)
    want_hits = o.frozen_hits(state, 7, 16)
    assert (hits != want_hits).mean() < 1e-4, (hits != want_hits).sum()
    T = tr.Transport(hits, sc.A, o.direct_unit(state))
    E = np.asarray(sc.states[state].inten, np.float64)
    ga = T.adjoint_gradient(w)
    assert np.allclose(ga, T.fd_gradient(E, w), rtol=1e-9, atol=0)
    assert np.allclose(g, ga, rtol=2e-5, atol=1e-7 * np.abs(ga).max())
    Lw = T.radiance(E)
    assert res["J"] == pytest.approx(float(w @ Lw), rel=2e-5)
    assert res["J_grad"] == pytest.approx(res["J"], rel=2e-5)
    assert np.allclose(L, Lw, rtol=1e-4, atol=1e-5 * Lw.max())
    uw = T.importance(w)
    assert np.allclose(u, uw, rtol=1e-4, atol=1e-5 * uw.max())
    assert res["rays"] == o.Np * 16 and res["back"] == int((hits < 0).sum())
    assert res["max_incoming"] == int(np.bincount(hits[hits >= 0], minlength=o.Np).max())
    assert res["fwd_change"] < 1e-6 and res["adj_change"] < 1e-6


def test_adjoint_street_format3():
    data = S.write(S.street_scene(points=12000, buildings=6, seed=2, lights=16))
    sc, o, w, g, res, L, u, hits = _case(data, 3, K=8, seed=11)
    want_hits = o.frozen_hits(3, 11, 8)
    assert (hits != want_hits).mean() < 1e-4
    T = tr.Transport(hits, sc.A, o.direct_unit(3))
    ga = T.adjoint_gradient(w)
    assert len(g) == 16
    assert np.allclose(g, ga, rtol=1e-4, atol=1e-6 * np.abs(ga).max())
    assert res["J_grad"] == pytest.approx(res["J"], rel=2e-5)


def test_adjoint_full_size_properties():
    """1,082,802 points, 16 lights (emission U[1, 50] beyond the first three): linearity,
    convergence and bit-identical repeats."""
    data = S.write(S.box_room(points=1_082_802, seed=0, lights=16))
    ctx = N.Context()
    info = ctx.load_bytes(data)
    assert info["nl"] == 16
    w = _weights(info["np"], 4096, 1)
    g1, r1 = ctx.adjoint(0, w, K=16, seed=5, iterations=64)
    g2, r2 = ctx.adjoint(0, w, K=16, seed=5, iterations=64)
    ctx.close()
    assert (g1 == g2).all() and r1["J"] == r2["J"]
    assert r1["J_grad"] == pytest.approx(r1["J"], rel=1e-5)
    assert r1["fwd_change"] < 1e-6 and r1["adj_change"] < 1e-6
    assert (g1 > 0).all()


def test_gpu_references_agree_with_the_path_tracer(scene_main_bytes):
    ctx = N.Context()
    ctx.load_bytes(scene_main_bytes)
    noise, _ = ctx.build_reference()
    o = po.Scene(data=scene_main_bytes)
    rng = np.random.default_rng(21)
    for si in range(len(noise)):
        ref = ctx.state_array(si, N.SA_REF).astype(np.float64)
        valid = ctx.state_array(si, N.SA_VALID).astype(bool) & (ref > 0)
        pts = np.flatnonzero(valid)[rng.choice(int(valid.sum()), 48, replace=False)]
        m, se = o.path_trace(si, pts, paths=8192, min_bounces=3, seed=40 + si)
        r = ref[pts]
        nz = noise[si] * float(ref[valid].mean())
        z = (m - r) / np.sqrt(se ** 2 + (noise[si] * r) ** 2 + nz ** 2)
        assert abs((m - r).mean()) / r.mean() < 0.02, si
        assert (z * z).mean() < 1.5 and np.abs(z).max() < 4.5, si
    ctx.close()


def test_adjoint_unit_build_kept_per_state(scene_main_bytes):
    """The context keeps the unit-emission direct light of the last state it built: calls that
    alternate states give, bit for bit, what fresh contexts give."""
    n = S.read(scene_main_bytes).states[0].P.shape[0]
    w = _weights(n, 256, 11)

    def fresh(state):
        c = N.Context()
        c.load_bytes(scene_main_bytes)
        g, _ = c.adjoint(state, w, K=8, seed=3, iterations=32)
        c.close()
        return g

    want = {s: fresh(s) for s in (0, 2)}
    ctx = N.Context()
    ctx.load_bytes(scene_main_bytes)
    for s in (0, 2, 2, 0):
        g, _ = ctx.adjoint(s, w, K=8, seed=3, iterations=32)
        assert np.array_equal(g, want[s]), s
    ctx.close()
