"""The tensor-core radiance cache (include/rc_mlp.h) on the GPU, against FP32 references of
the same products computed by torch from the same bf16 values."""
import pytest
import torch

from render_engine_gb300 import mlp

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("K,N", [(16, 16), (64, 64), (176, 64), (64, 16), (128, 128), (256, 256)])
def test_tile_product_matches_fp32(K, N):
    g = torch.Generator(device="cuda").manual_seed(K * 1000 + N)
    a = torch.randn(128, K, device="cuda", generator=g).to(torch.bfloat16)
    b = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    d = torch.zeros(128, N, device="cuda", dtype=torch.float32)
    err = torch.zeros(1, device="cuda", dtype=torch.int32)
    mlp.tile_product(a, b, d, err)
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    want = a.float() @ b.float().t()
    # bf16 x bf16 products are exact in FP32; only the order of the K-sum differs
    assert torch.allclose(d, want, rtol=1e-5, atol=1e-4 * K ** 0.5), (d - want).abs().max().item()


# ---------------------------------------------------------------- the network vs a torch emulation
import math  # noqa: E402

import numpy as np  # noqa: E402

LO = torch.tensor([0.0, 0.0, 0.0])
HI = torch.tensor([8.0, 4.0, 3.0])


def _q(x):
    return x.to(torch.bfloat16).float()


def _encode(P, N, aux):
    """The 176 input features, as the kernels compute them (FP32)."""
    lo, hi = LO.to(P.device), HI.to(P.device)
    p = ((P[:, :3] - lo) * (1.0 / (hi - lo))).clamp(0, 1)
    n = N[:, :3]
    f = torch.zeros(P.shape[0], 176, device=P.device)
    for ax in range(3):
        w = math.pi * p[:, ax]
        for o in range(12):
            f[:, ax * 24 + 2 * o] = torch.sin(w)
            f[:, ax * 24 + 2 * o + 1] = torch.cos(w)
            w = w * 2
        u = math.pi * n[:, ax]
        for o in range(4):
            f[:, 72 + ax * 8 + 2 * o] = torch.sin(u)
            f[:, 72 + ax * 8 + 2 * o + 1] = torch.cos(u)
            u = u * 2
        bp, bn = p[:, ax] * 16, (n[:, ax] * 0.5 + 0.5) * 4
        for b in range(16):
            f[:, 96 + ax * 16 + b] = (1 - (bp - (b + 0.5)).abs()).clamp(min=0)
        for b in range(4):
            f[:, 144 + ax * 4 + b] = (1 - (bn - (b + 0.5)).abs()).clamp(min=0)
        f[:, 156 + ax] = p[:, ax]
        f[:, 159 + ax] = n[:, ax]
    f[:, 162:165] = aux[:, 1:4]
    f[:, 165] = aux[:, 0]
    f[:, 166] = 1.0
    return f


def _forward(Ws, P, N, aux):
    a = [_q(_encode(P, N, aux))]
    for l, W in enumerate(Ws):
        z = a[-1] @ _q(W).t()
        if l < 4:
            a.append(_q(torch.relu(z)))
    return a, z


def _inputs(n, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    P = torch.rand(n, 4, device="cuda", generator=g) * torch.tensor([8.0, 4.0, 3.0, 0.0], device="cuda")
    N = torch.randn(n, 4, device="cuda", generator=g)
    N[:, :3] = N[:, :3] / N[:, :3].norm(dim=1, keepdim=True)
    N[:, 3] = 0
    aux = torch.rand(n, 4, device="cuda", generator=g)
    return P.contiguous(), N.contiguous(), aux.contiguous()


def test_infer_matches_emulation():
    net = mlp.Mlp(n_out=3, seed=5)
    Ws = [torch.from_numpy(w.copy()).cuda() for w in mlp.split_weights(net.weights())]
    P, N, aux = _inputs(1000, 1)
    out = torch.zeros(1000, 3, device="cuda")
    net.infer(P, N, aux, out)
    torch.cuda.synchronize()
    assert net.error_flags() == 0
    _, z = _forward(Ws, P, N, aux)
    want = z[:, :3]
    rel = (out - want).norm() / want.norm()
    assert rel < 2e-2, rel.item()
    assert torch.allclose(out, want, rtol=5e-2, atol=5e-2 * want.abs().max().item())


def test_gradients_match_emulation():
    n = 512
    net = mlp.Mlp(n_out=3, seed=7, lr=0.0)
    Ws = [torch.from_numpy(w.copy()).cuda() for w in mlp.split_weights(net.weights())]
    P, N, aux = _inputs(n, 2)
    target = torch.rand(n, 4, device="cuda") * 2
    net.train(P, N, aux, target)
    torch.cuda.synchronize()
    assert net.error_flags() == 0
    g = torch.from_numpy(net.gradients()).cuda()
    a, z = _forward(Ws, P, N, aux)
    y = z
    dy = torch.zeros_like(y)
    t = target[:, :3]
    dy[:, :3] = 2 * (y[:, :3] - t) / (y[:, :3] ** 2 + 0.01) / (n * 3)
    dz = _q(dy)
    grads = [None] * 5
    for l in range(4, -1, -1):
        grads[l] = dz.t() @ a[l]
        if l >= 1:
            da = dz @ _q(Ws[l])
            dz = _q(da * (a[l] > 0))
    want = torch.cat([x.reshape(-1) for x in grads])
    rel = (g - want).norm() / want.norm()
    assert rel < 2e-2, rel.item()
    for l, (k, m) in enumerate(mlp.LAYERS):
        gl = mlp.split_weights(g.cpu().numpy())[l]
        wl = grads[l].cpu().numpy()
        assert np.linalg.norm(gl - wl) <= 3e-2 * np.linalg.norm(wl) + 1e-9, l


def test_training_fits_a_smooth_field():
    n = 8192
    net = mlp.Mlp(n_out=3, seed=3, lr=1e-2, max_batch=n)
    P, N, aux = _inputs(n, 3)
    p = P[:, :3] / torch.tensor([8.0, 4.0, 3.0], device="cuda")
    target = torch.stack([1 + torch.sin(3 * p[:, 0]) * p[:, 1], 0.5 + p[:, 2] ** 2, 0.2 + aux[:, 1] * p[:, 0]], dim=1).contiguous()
    loss = torch.zeros(1, device="cuda")
    losses = []
    for step in range(200):
        loss.zero_()
        net.train(P, N, aux, target, loss=loss)
        losses.append(loss.item() / (n * 3))
    assert net.error_flags() == 0
    assert losses[-1] < 0.05 * losses[0], (losses[0], losses[-1])
    out = torch.zeros(n, 3, device="cuda")
    net.infer(P, N, aux, out)
    rel = ((out - target).norm() / target.norm()).item()
    assert rel < 0.2, rel   # 0.117 after 200 steps on the GB300


def test_bounded_wait_gives_up_and_reports():
    """Failure detection without a fault: a completion wait on an mbarrier that nothing arrives on
    gives up after its poll limit and raises the error bit (the kernel ends, the context stays
    usable); with one arrival the same wait succeeds."""
    import torch
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    mlp.wait_check(1 << 12, True, err)
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    mlp.wait_check(1 << 12, False, err)
    torch.cuda.synchronize()
    assert int(err.item()) == 1
    # the context still runs work
    err.zero_()
    mlp.wait_check(1 << 12, True, err)
    torch.cuda.synchronize()
    assert int(err.item()) == 0


def test_captured_training_steps_equal_direct_launches():
    """A caller that trains on the same buffers step after step gets the step replayed from a
    captured CUDA graph (from the second call on); one whose buffers change every call gets direct
    launches.  Same data, same seed: the weights after 6 steps are identical bit for bit, and so
    are the loss-scale state and the step counts."""
    n = 2048
    P, N, aux = _inputs(n, 5)
    target = torch.rand(n, 4, device="cuda")
    same = mlp.Mlp(n_out=3, seed=11, lr=1e-2, max_batch=n)
    alt = mlp.Mlp(n_out=3, seed=11, lr=1e-2, max_batch=n)
    copies = [(P.clone(), N.clone(), aux.clone(), target.clone()) for _ in range(2)]
    for step in range(6):
        same.train(P, N, aux, target)
        c = copies[step % 2]
        alt.train(*c)
    torch.cuda.synchronize()
    assert same.error_flags() == 0 and alt.error_flags() == 0
    assert np.array_equal(same.weights(), alt.weights())
    assert same.loss_scale() == alt.loss_scale()
    same.close()
    alt.close()
