"""The adjoint of the cache transport as a torch.autograd.Function, and the ranking of an
event's invalidation set by sensitivity (host side of rc_adjoint, include/rc_api.h).

``CacheTransport.apply(emission, ctx, state, weights, K, seed, iterations)`` returns
J(E) = sum_i w_i sum_l L_l[i](E), the weighted cache radiance of the frozen-ray transport of
`state` with light emissions E, from the GPU's forward solve; its backward pass returns
dJ/dE from the GPU's adjoint solve (one solve for all lights, path vertices recomputed from
the frozen rays' hit lists, no stored paths).  The two solves are independent, so
torch.autograd.gradcheck against central differences of the forward tests the adjoint.

``rank_invalidation(ctx, state, light, points)`` orders the points of an invalidation set (as
the reference's k_touched marks them, bit for bit) by dL_i/dE_l, the sensitivity of point i's
cache radiance to the emission of the light that changed: the forward solution at unit
emission of that light alone.  The set is not changed, only ordered.
"""
from __future__ import annotations

import numpy as np

from . import native as N


def _make():
    import torch

    class CacheTransport(torch.autograd.Function):
        @staticmethod
        def forward(fctx, emission, rc: N.Context, state: int, weights, K: int, seed: int, iterations: int):
            em = emission.detach().to("cpu", torch.float64).numpy().astype(np.float32)
            g, res = rc.adjoint(state, weights, K=K, seed=seed, iterations=iterations, emission=em)
            fctx.save_for_backward(torch.from_numpy(g.astype(np.float64)).to(emission.dtype))
            return torch.tensor(res["J"], dtype=emission.dtype)

        @staticmethod
        def backward(fctx, grad):
            (g,) = fctx.saved_tensors
            return grad * g, None, None, None, None, None, None

    return CacheTransport


_CT = None


def cache_transport():
    """The torch.autograd.Function (built on first use, torch imported lazily)."""
    global _CT
    if _CT is None:
        _CT = _make()
    return _CT


def sensitivity(ctx: N.Context, state: int, light: int, K: int = 16, seed: int = 0, iterations: int = 64) -> np.ndarray:
    """dL_i/dE_l for every point i: the forward solution with light `light` at unit emission and
    the others off (L is linear in the emissions)."""
    nl, np_ = ctx.info()["nl"], ctx.info()["np"]
    em = np.zeros(nl, np.float32)
    em[light] = 1.0
    ctx.adjoint(state, np.zeros(np_, np.float32), K=K, seed=seed, iterations=iterations, emission=em)
    L, _, _ = ctx.adjoint_arrays()
    return L


def rank_invalidation(ctx: N.Context, state: int, light: int, points, K: int = 16, seed: int = 0,
                      iterations: int = 64) -> tuple[np.ndarray, np.ndarray]:
    """The points of an invalidation set ordered by decreasing dL_i/dE_light (ties by index), and
    their sensitivities in that order."""
    pts = np.asarray(points, np.int64)
    s = sensitivity(ctx, state, light, K, seed, iterations)[pts]
    order = np.lexsort((pts, -s.astype(np.float64)))
    return pts[order], s[order]
