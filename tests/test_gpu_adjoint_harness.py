"""The adjoint as a torch.autograd.Function (render_engine_gb300/adjoint.py) and the ranking of an
invalidation set by sensitivity, on the reference's scene_main (10,728 points, 3 lights).

* gradcheck: the backward pass (the GPU's adjoint solve) against central differences of the
  forward pass (the GPU's forward solve at perturbed emissions), in float64 on the host side;
* linearity: J(E) from the forward solve equals sum_l E_l dJ/dE_l;
* ranking: the points the reference's k_touched marks when light 0 comes back on (every point
  whose dependency mask holds a voxel of the light's event list), ordered by dL_i/dE_0: the
  ordered list is the same set, bit for bit, with sensitivities that do not increase."""
import numpy as np
import pytest

from oracle import pyoracle as po
from render_engine_gb300 import adjoint as ADJ
from render_engine_gb300 import methods as M
from render_engine_gb300 import native as N

pytestmark = pytest.mark.gpu


def _weights(n, k, seed):
    rng = np.random.default_rng(seed)
    w = np.zeros(n, np.float32)
    w[rng.choice(n, k, replace=False)] = 1.0 / k
    return w


def test_gradcheck_against_central_differences(scene_main_bytes):
    torch = pytest.importorskip("torch")
    ctx = N.Context()
    info = ctx.load_bytes(scene_main_bytes)
    w = _weights(info["np"], 256, 4)
    E0 = torch.tensor(ctx.state_lights(0).astype(np.float64), requires_grad=True)
    CT = ADJ.cache_transport()
    f = lambda E: CT.apply(E, ctx, 0, w, 16, 3, 96)
    # J is linear in E: central differences are exact up to the forward solve's float rounding
    assert torch.autograd.gradcheck(f, (E0,), eps=0.05, atol=1e-5, rtol=2e-4)
    J = f(E0)
    J.backward()
    g = E0.grad.numpy()
    assert float(J.detach()) == pytest.approx(float((E0.detach().numpy() * g).sum()), rel=1e-5)
    # other emissions: the same derivatives, J scaled accordingly
    E1 = torch.tensor([3.0, 0.5, 7.0], dtype=torch.float64, requires_grad=True)
    J1 = f(E1)
    J1.backward()
    np.testing.assert_allclose(E1.grad.numpy(), g, rtol=1e-6)
    assert float(J1.detach()) == pytest.approx(float((E1.detach().numpy() * g).sum()), rel=1e-5)
    ctx.close()


def test_invalidation_set_ranked_by_sensitivity(scene_main_bytes):
    ctx = N.Context()
    info = ctx.load_bytes(scene_main_bytes)
    np_, ns = info["np"], info["ns"]
    m = M.by_name(M.timing_methods(), "v3 complet")
    ctx.begin(m, 1, 9)
    for _ in range(40):
        ctx.frame(1)
    masks = (ctx.array(N.A_CUR) | ctx.array(N.A_PREV)).reshape(-1, np_)
    V = po.Scene(data=scene_main_bytes).event_list(1 * ns + 0, 1 + 0)   # light 0 on: its voxels
    assert len(V) > 0
    touched = np.zeros(np_, bool)
    for v in V:
        touched |= (masks[v // 32] >> np.uint32(v % 32)) & 1 == 1
    pts = np.flatnonzero(touched)
    assert 0 < len(pts) < np_
    ranked, sens = ADJ.rank_invalidation(ctx, 0, 0, pts, K=16, seed=2, iterations=64)
    assert np.array_equal(np.sort(ranked), pts)          # the same set
    assert (np.diff(sens) <= 0).all() and sens[0] > 0     # in order of sensitivity
    top = max(1, len(sens) // 10)
    share = float(sens[:top].sum() / max(sens.sum(), 1e-30))
    assert share > 0.1
    print("invalidation set %d points; top 10%% hold %.1f %% of the sensitivity" % (len(pts), 100 * share))
    ctx.close()
