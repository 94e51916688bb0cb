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
