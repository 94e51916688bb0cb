"""The FP64 oracle of the adjoint and the FP64 path tracer, on the CPU.

* The adjoint gradient of the frozen-ray transport equals central finite differences and
  satisfies J = sum_l E_l dJ/dE_l (J is linear in the emissions).
* The FP64 path tracer (an estimator independent of any frame or reference kernel) agrees with
  the converged references the reference's own scene preparation stored in the golden scenes
  (prep_mesh.cuh:459-518), which pins it before it is used to check the GPU references.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from oracle import transport as tr
from render_engine_gb300 import scene as S


@pytest.fixture(scope="module")
def main(scene_main_bytes):
    o = po.Scene(data=scene_main_bytes)
    o.build()
    return o, S.read(scene_main_bytes)


def _weights(n, k, seed):
    rng = np.random.default_rng(seed)
    w = np.zeros(n)
    w[rng.choice(n, k, replace=False)] = 1.0 / k
    return w


def test_unit_direct_light_scales_to_the_state_light(main):
    o, sc = main
    for si in (0, 1):
        G = o.direct_unit(si)
        E = np.asarray(sc.states[si].inten, np.float32)
        Ed = o.state_array(si, 0).reshape(-1, o.NL)
        assert np.allclose(G * E, Ed, rtol=1e-6, atol=1e-6 * Ed.max())


@pytest.mark.parametrize("state", [0, 1])   # state 1 has light 0 off: its derivative still exists
def test_adjoint_equals_finite_differences(main, state):
    o, sc = main
    hits = o.frozen_hits(state, 7, 16)
    assert hits.shape == (o.Np, 16) and (hits >= -1).all() and (hits < o.Np).all()
    T = tr.Transport(hits, sc.A, o.direct_unit(state))
    E = np.asarray(sc.states[state].inten, np.float64)
    w = _weights(o.Np, 512, state)
    ga = T.adjoint_gradient(w)
    gf = T.fd_gradient(E, w)
    assert np.allclose(ga, gf, rtol=1e-9, atol=0)
    assert (ga > 0).all()
    assert T.objective(E, w) == pytest.approx(float(E @ ga), rel=1e-12)


def test_frozen_hits_follow_the_seed(main):
    o, _ = main
    a = o.frozen_hits(0, 7, 8)
    b = o.frozen_hits(0, 7, 16)
    c = o.frozen_hits(0, 8, 8)
    assert (a == b[:, :8]).all()            # the first rays of a longer set are the same rays
    assert (a != c).mean() > 0.5


@pytest.mark.parametrize("name", ["scene_main.bin", "scene_stress.bin"])
def test_path_tracer_pins_the_embedded_references(name):
    from conftest import golden_bytes
    data = golden_bytes(name)
    sc = S.read(data)
    o = po.Scene(data=data)
    rng = np.random.default_rng(11)
    for si, st in enumerate(sc.states):
        ok = st.valid.astype(bool) & (st.ref > 0)
        pts = np.flatnonzero(ok)[rng.choice(int(ok.sum()), 48, replace=False)]
        m, se = o.path_trace(si, pts, paths=8192, min_bounces=3, seed=5 + si)
        r = st.ref[pts].astype(np.float64)
        # per point: the path tracer's standard error and the references' own noise (their
        # preparation stops when the chains disagree by 3 % RMS of the mean over all points)
        noise = 0.03 * float(st.ref[ok].mean())
        z = (m - r) / np.sqrt(se ** 2 + (0.03 * r) ** 2 + noise ** 2)
        assert abs((m - r).mean()) / r.mean() < 0.02, si
        assert (z * z).mean() < 1.5 and np.abs(z).max() < 4.5, si
