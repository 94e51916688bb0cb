"""The learned radiance cache in the frame loop (render_engine_gb300/learned.py): the network of
include/rc_mlp.h trained online, every frame, on the one-bounce estimates the tracer makes with
the network's own radiance at its hit points, and served as the cache.  On the reference's
scene_main (10,728 points, 3 lights, converged references stored in the file):

* what the network gains: its error against the references is far below that of the same
  frame loop without it (the uncached one-bounce estimate, where the light beyond the first
  hit is missing), before and after a light is switched off;
* against the per-point cache (the reference's Classique 1.0x, the hash-grid-style cache the
  learned one is compared with): near it before the event, and its 30-frame post-event error far
  below it (the switched-off light reaches the network through its direct-light input);
* loss scaling: a step whose gradient is not finite is skipped (weights untouched) and the scale
  halved."""
import math

import numpy as np
import pytest

from render_engine_gb300 import learned as LC
from render_engine_gb300 import methods as M
from render_engine_gb300 import mlp as MLP
from render_engine_gb300 import native as N

pytestmark = pytest.mark.gpu

SEQ = [0] * 80 + [1] * 30


def _err(ctx, state):
    nl = ctx.info()["nl"]
    est = ctx.array(N.A_LC).reshape(-1, nl).astype(np.float64).sum(axis=1)
    ref = ctx.state_array(state, N.SA_REF).astype(np.float64)
    ok = ctx.state_array(state, N.SA_VALID) != 0
    return math.sqrt(((est[ok] - ref[ok]) ** 2).mean()) / ref[ok].mean()


def _learned_errors(data, stream):
    ctx = N.Context(stream=stream)
    ctx.load_bytes(data)
    lc = LC.LearnedCache(ctx, data, stream, batch=1 << 14, lr=1e-2, seed=3, steps_per_frame=4)
    lc.begin(SEQ[0], 5)
    errs = []
    for s in SEQ:
        lc.predict(s)
        errs.append(_err(ctx, s))
        lc.frame(s, predicted=True)
    scale, steps, skipped = lc.mlp.loss_scale()
    lc.close()
    assert ctx.device_flags() == 0
    ctx.close()
    return np.array(errs), steps, skipped


def _uncached_errors(data):
    """The same loop without the network: the cache is zero before every frame, so a point's value
    is A(hit) Edir(hit), the light of the first bounce alone."""
    ctx = N.Context()
    ctx.load_bytes(data)
    nl = ctx.info()["nl"]
    ctx.begin(LC.LEARNED_METHOD, SEQ[0], 5)
    zero = np.zeros(ctx.info()["np"] * nl, np.float32)
    errs = []
    for s in SEQ:
        ctx.set_array(N.A_LC, zero)
        ctx.frame(s)
        errs.append(_err(ctx, s))
    ctx.close()
    return np.array(errs)


def _cache_errors(data, name):
    ctx = N.Context()
    ctx.load_bytes(data)
    ctx.begin(M.by_name(M.timing_methods() + M.scen_methods(), name), SEQ[0], 5)
    errs = []
    for s in SEQ:
        ctx.frame(s)
        errs.append(_err(ctx, s))
    ctx.close()
    return np.array(errs)


def test_learned_cache_gains_over_the_uncached_loop(scene_main_bytes):
    import torch
    st = torch.cuda.Stream()
    le, steps, skipped = _learned_errors(scene_main_bytes, st.cuda_stream)
    un = _uncached_errors(scene_main_bytes)
    cl = _cache_errors(scene_main_bytes, "Classique 1.0x")
    pre_l, post_l = le[60:80].mean(), le[80:110].mean()
    pre_u, post_u = un[60:80].mean(), un[80:110].mean()
    pre_c, post_c = cl[60:80].mean(), cl[80:110].mean()
    print("learned pre %.4f post %.4f | uncached pre %.4f post %.4f | Classique 1.0x post %.4f" % (pre_l, post_l, pre_u, post_u, post_c))
    assert steps == 4 * len(SEQ) and skipped == 0
    assert np.isfinite(le).all()
    assert pre_l < 0.6 * pre_u and post_l < 0.6 * post_u       # the network carries the light beyond the first bounce
    assert pre_l < 2.0 * pre_c                                  # near the per-point cache in a steady state
    assert post_l < 0.5 * post_c                                # and far below it after a light is switched off


def test_loss_scaling_skips_a_non_finite_step():
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(2)
    n = 1024
    P = (torch.rand(n, 4, device="cuda", generator=g) * torch.tensor([8.0, 4.0, 3.0, 0.0], device="cuda")).contiguous()
    Nn = torch.randn(n, 4, device="cuda", generator=g)
    Nn[:, :3] /= Nn[:, :3].norm(dim=1, keepdim=True)
    aux = torch.rand(n, 4, device="cuda", generator=g).contiguous()
    t = torch.rand(n, 3, device="cuda", generator=g).contiguous()
    net = MLP.Mlp(n_out=3, max_batch=n, loss_scale=4096.0)
    net.train(P, Nn.contiguous(), aux, t)
    assert net.loss_scale() == (4096.0, 1, 0)
    w0 = net.weights()
    t[5, 1] = float("nan")
    net.train(P, Nn.contiguous(), aux, t)
    assert net.loss_scale() == (2048.0, 1, 1)                  # skipped, scale halved
    assert np.array_equal(net.weights(), w0)                   # weights untouched
    t[5, 1] = 0.5
    net.train(P, Nn.contiguous(), aux, t)
    assert net.loss_scale() == (2048.0, 2, 1)
    assert not np.array_equal(net.weights(), w0)
    net.close()
